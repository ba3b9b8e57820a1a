// FP32-pair stage kernels (PrecMixedPair) of DOP853 on the Van der Pol, pendulum and Lorenz
// families, and DOPRI5's dense multi-family kernel: the tight-tolerance part of a DEGPU_MIXED solve.
#include "registry.cuh"

namespace degpu {
void register_mixed_pair853() {
    register_thread_variant<TabDop853, RhsLorenz, PrecMixedPair>();
    register_thread_variant<TabDop853, RhsVanDerPol, PrecMixedPair>();
    register_thread_variant<TabDop853, RhsPendulum, PrecMixedPair>();
    register_multi<TabDop853, PrecMixedPair>();
    multi_registry()[{method_id<TabDopri5>(), PrecMixedPair::ID, 1}] = &launch_multi<TabDopri5, PrecMixedPair, true>;
    register_round<TabDop853, RhsLorenz, PrecMixedPair>();
    register_round<TabDop853, RhsVanDerPol, PrecMixedPair>();
    register_round<TabDop853, RhsPendulum, PrecMixedPair>();
    register_round<TabDop853, RhsLorenz, PrecMixedPair, true>();
    register_round<TabDop853, RhsVanDerPol, PrecMixedPair, true>();
    register_round<TabDop853, RhsPendulum, PrecMixedPair, true>();
}
}  // namespace degpu
