// FP32-pair stage kernels (PrecMixedPair) of DOPRI5 on the Van der Pol, pendulum and Lorenz
// families: the tight-tolerance part of a DEGPU_MIXED solve.
#include "registry.cuh"

namespace degpu {
void register_mixed_pair() {
    register_thread_variant<TabDopri5, RhsLorenz, PrecMixedPair>();
    register_thread_variant<TabDopri5, RhsVanDerPol, PrecMixedPair>();
    register_thread_variant<TabDopri5, RhsPendulum, PrecMixedPair>();
    multi_registry()[{method_id<TabDopri5>(), PrecMixedPair::ID, 0}] = &launch_multi<TabDopri5, PrecMixedPair, false>;
    register_round<TabDopri5, RhsLorenz, PrecMixedPair>();
    register_round<TabDopri5, RhsVanDerPol, PrecMixedPair>();
    register_round<TabDopri5, RhsPendulum, PrecMixedPair>();
    register_round<TabDopri5, RhsLorenz, PrecMixedPair, true>();
    register_round<TabDopri5, RhsVanDerPol, PrecMixedPair, true>();
    register_round<TabDopri5, RhsPendulum, PrecMixedPair, true>();
}
}  // namespace degpu
