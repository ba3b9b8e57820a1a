// FP64_FAST and MIXED multi-family persistent kernels.
#include "registry.cuh"

namespace degpu {
void register_multi_fast_mixed() {
    register_multi<TabDopri5, PrecFast>();
    register_multi<TabDop853, PrecFast>();
    register_multi<TabRK4, PrecFast>();
    register_multi<TabDopri5, PrecMixed>();
    register_multi<TabDop853, PrecMixed>();
    register_multi<TabRK4, PrecMixed>();
}
}  // namespace degpu
