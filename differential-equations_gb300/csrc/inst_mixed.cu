// Mixed-precision variants: FP32 stages, Kahan-compensated y, FP64 t / norm / controller.
#include "registry.cuh"

namespace degpu {
void register_mixed() {
    register_variant<TabDopri5, RhsLorenz, PrecMixed>();
    register_variant<TabDopri5, RhsVanDerPol, PrecMixed>();
    register_variant<TabDopri5, RhsPendulum, PrecMixed>();
    register_variant<TabDop853, RhsLorenz, PrecMixed>();
    register_variant<TabDop853, RhsVanDerPol, PrecMixed>();
    register_variant<TabDop853, RhsPendulum, PrecMixed>();
    register_variant<TabRK4, RhsLorenz, PrecMixed>();
    register_variant<TabRK4, RhsVanDerPol, PrecMixed>();
    register_variant<TabRK4, RhsPendulum, PrecMixed>();
    register_round_all_methods<RhsLorenz, PrecMixed>();
    register_round_all_methods<RhsVanDerPol, PrecMixed>();
    register_round_all_methods<RhsPendulum, PrecMixed>();
    register_rhs<RhsLorenz, PrecMixed>();
    register_rhs<RhsVanDerPol, PrecMixed>();
    register_rhs<RhsPendulum, PrecMixed>();
}
}  // namespace degpu
