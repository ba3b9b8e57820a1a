// Parity (FP64, no FMA contraction) instantiation of the Gray–Scott passes.
// Compiled with -fmad=false.
#include "stencil.cuh"

#if defined(__CUDACC__) && !defined(DEGPU_NO_FMAD)
#error "parity translation units must be compiled with -fmad=false -DDEGPU_NO_FMAD"
#endif

namespace degpu {
GsPassFn64 gs_parity_pass(bool pow2) { return pow2 ? &gs_launch_pass<double, true> : &gs_launch_pass<double, false>; }
}  // namespace degpu
