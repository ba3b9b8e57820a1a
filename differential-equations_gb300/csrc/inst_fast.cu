// FP64 variants with FMA contraction and the CUDA math library.
#include "registry.cuh"

namespace degpu {
void register_fast() {
    register_variant<TabDopri5, RhsLorenz, PrecFast>();
    register_variant<TabDopri5, RhsVanDerPol, PrecFast>();
    register_variant<TabDopri5, RhsPendulum, PrecFast>();
    register_variant<TabDop853, RhsLorenz, PrecFast>();
    register_variant<TabDop853, RhsVanDerPol, PrecFast>();
    register_variant<TabDop853, RhsPendulum, PrecFast>();
    register_variant<TabRK4, RhsLorenz, PrecFast>();
    register_variant<TabRK4, RhsVanDerPol, PrecFast>();
    register_variant<TabRK4, RhsPendulum, PrecFast>();
    register_round_all_methods<RhsLorenz, PrecFast>();
    register_round_all_methods<RhsVanDerPol, PrecFast>();
    register_round_all_methods<RhsPendulum, PrecFast>();
    register_rhs<RhsLorenz, PrecFast>();
    register_rhs<RhsVanDerPol, PrecFast>();
    register_rhs<RhsPendulum, PrecFast>();
}
}  // namespace degpu
