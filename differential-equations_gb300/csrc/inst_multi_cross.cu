// inst_multi_cross.cu — multi-family persistent kernels with crossing / event detection, FP64 fast
// and mixed; a mixed solve's instances below the mixed-precision bound run the FP32-pair kernel
// (DOPRI5) or the fast one (DOP853).
#include "registry.cuh"

namespace degpu {
void register_multi_cross() {
    register_multi_cross<TabDopri5, PrecFast>();
    register_multi_cross<TabDopri5, PrecMixed>();
    register_multi_cross<TabDopri5, PrecMixedPair>();  // DOPRI5's tight class
    register_multi_cross<TabDop853, PrecFast>();
    register_multi_cross<TabDop853, PrecMixed>();
}
}  // namespace degpu
