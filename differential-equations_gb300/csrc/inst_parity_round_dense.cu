// Resumable round kernels with output times (the server's dense-output requests), FP64 parity.
// Compiled with -fmad=false.
#include "registry.cuh"

#if defined(__CUDACC__) && !defined(DEGPU_NO_FMAD)
#error "parity translation units must be compiled with -fmad=false -DDEGPU_NO_FMAD"
#endif

namespace degpu {
void register_round_dense_parity() {
    register_round_all_methods<RhsLorenz, PrecParity, true>();
    register_round_all_methods<RhsVanDerPol, PrecParity, true>();
    register_round_all_methods<RhsPendulum, PrecParity, true>();
}
}  // namespace degpu
