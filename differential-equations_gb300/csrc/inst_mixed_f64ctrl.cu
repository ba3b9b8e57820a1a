// MIXED_FP64_CTRL variants (FP32 stages, Kahan-compensated y, FP64 error norm, controller and t)
// of DOPRI5 and DOP853 on the Van der Pol, pendulum and Lorenz families.
#include "registry.cuh"

namespace degpu {
void register_mixed_f64ctrl() {
    register_thread_variant<TabDopri5, RhsLorenz, PrecMixedF64Ctrl>();
    register_thread_variant<TabDopri5, RhsVanDerPol, PrecMixedF64Ctrl>();
    register_thread_variant<TabDopri5, RhsPendulum, PrecMixedF64Ctrl>();
    register_thread_variant<TabDop853, RhsLorenz, PrecMixedF64Ctrl>();
    register_thread_variant<TabDop853, RhsVanDerPol, PrecMixedF64Ctrl>();
    register_thread_variant<TabDop853, RhsPendulum, PrecMixedF64Ctrl>();
    register_multi<TabDopri5, PrecMixedF64Ctrl>();
    register_multi<TabDop853, PrecMixedF64Ctrl>();
}
}  // namespace degpu
