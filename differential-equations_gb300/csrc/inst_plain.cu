// FP64_PLAIN variants (FMA contraction, correctly rounded controller power) of DOPRI5 and DOP853
// on the Van der Pol, pendulum and Lorenz families: one-launch-per-family and persistent kernels.
#include "registry.cuh"

#if defined(DEGPU_NO_FMAD)
#error "the plain FP64 translation unit is compiled with FMA contraction"
#endif

namespace degpu {
void register_plain() {
    register_thread_variant<TabDopri5, RhsLorenz, PrecPlain>();
    register_thread_variant<TabDopri5, RhsVanDerPol, PrecPlain>();
    register_thread_variant<TabDopri5, RhsPendulum, PrecPlain>();
    register_thread_variant<TabDop853, RhsLorenz, PrecPlain>();
    register_thread_variant<TabDop853, RhsVanDerPol, PrecPlain>();
    register_thread_variant<TabDop853, RhsPendulum, PrecPlain>();
    register_multi<TabDopri5, PrecPlain>();
    register_multi<TabDop853, PrecPlain>();
}
}  // namespace degpu
