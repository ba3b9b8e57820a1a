// Method-of-lines drivers in the crate's operation order (FP64, no contraction).  Compiled with
// -fmad=false.
#include "mol.cuh"

#if defined(__CUDACC__) && !defined(DEGPU_NO_FMAD)
#error "parity translation units must be compiled with -fmad=false -DDEGPU_NO_FMAD"
#endif

namespace degpu {
void register_mol_parity() { register_mol_all<double>(0); }
}  // namespace degpu
