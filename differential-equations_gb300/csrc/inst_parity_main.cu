// Parity (FP64, no FMA contraction) variants of the three production families.
// Compiled with -fmad=false.
#include "registry.cuh"

#if defined(__CUDACC__) && !defined(DEGPU_NO_FMAD)
#error "parity translation units must be compiled with -fmad=false -DDEGPU_NO_FMAD"
#endif

namespace degpu {
void register_parity_main() {
    register_variant<TabDopri5, RhsLorenz, PrecParity>();
    register_variant<TabDopri5, RhsVanDerPol, PrecParity>();
    register_variant<TabDopri5, RhsPendulum, PrecParity>();
    register_variant<TabDop853, RhsLorenz, PrecParity>();
    register_variant<TabDop853, RhsVanDerPol, PrecParity>();
    register_variant<TabDop853, RhsPendulum, PrecParity>();
    register_variant<TabRK4, RhsLorenz, PrecParity>();
    register_variant<TabRK4, RhsVanDerPol, PrecParity>();
    register_variant<TabRK4, RhsPendulum, PrecParity>();
    register_round_all_methods<RhsLorenz, PrecParity>();
    register_round_all_methods<RhsVanDerPol, PrecParity>();
    register_round_all_methods<RhsPendulum, PrecParity>();
    register_rhs<RhsLorenz, PrecParity>();
    register_rhs<RhsVanDerPol, PrecParity>();
    register_rhs<RhsPendulum, PrecParity>();
}
}  // namespace degpu
