// inst_parity_embedded.cu — the Adaptive ERK family (RKF45, Cash-Karp), FP64 parity arithmetic
// (compiled with -fmad=false like every inst_parity_* translation unit), one system per thread.
#include "registry.cuh"

namespace degpu {

template <class Rhs>
static void reg_pair() {
    register_thread_variant<TabRKF45, Rhs, PrecParity>();
    register_thread_variant<TabCashKarp, Rhs, PrecParity>();
}

void register_embedded_parity() {
    reg_pair<RhsExpGrowth>();
    reg_pair<RhsLinear>();
    reg_pair<RhsHarmonic>();
    reg_pair<RhsLogistic>();
    reg_pair<RhsVanDerPol>();
    reg_pair<RhsPendulum>();
    reg_pair<RhsLorenz>();
}

}  // namespace degpu
