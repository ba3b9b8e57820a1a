// Parity (FP64, no FMA contraction) multi-family persistent kernels.  Compiled with -fmad=false.
#include "registry.cuh"

#if defined(__CUDACC__) && !defined(DEGPU_NO_FMAD)
#error "parity translation units must be compiled with -fmad=false -DDEGPU_NO_FMAD"
#endif

namespace degpu {
void register_parity_multi() {
    register_multi<TabDopri5, PrecParity>();
    register_multi<TabDop853, PrecParity>();
    register_multi<TabRK4, PrecParity>();
}
}  // namespace degpu
