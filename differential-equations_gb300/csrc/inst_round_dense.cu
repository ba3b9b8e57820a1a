// Resumable round kernels with output times (the server's dense-output requests), FP64 fast and
// mixed.
#include "registry.cuh"

namespace degpu {
void register_round_dense_fast_mixed() {
    register_round_all_methods<RhsLorenz, PrecFast, true>();
    register_round_all_methods<RhsVanDerPol, PrecFast, true>();
    register_round_all_methods<RhsPendulum, PrecFast, true>();
    register_round_all_methods<RhsLorenz, PrecMixed, true>();
    register_round_all_methods<RhsVanDerPol, PrecMixed, true>();
    register_round_all_methods<RhsPendulum, PrecMixed, true>();
}
}  // namespace degpu
