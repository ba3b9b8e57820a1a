// inst_embedded.cu — the Adaptive ERK family (RKF45, Cash-Karp), FP64 fast and mixed arithmetic,
// one system per thread.
#include "registry.cuh"

namespace degpu {

template <class Rhs, class P>
static void reg_pair() {
    register_thread_variant<TabRKF45, Rhs, P>();
    register_thread_variant<TabCashKarp, Rhs, P>();
}

void register_embedded_fast_mixed() {
    reg_pair<RhsVanDerPol, PrecFast>();
    reg_pair<RhsPendulum, PrecFast>();
    reg_pair<RhsLorenz, PrecFast>();
    reg_pair<RhsHarmonic, PrecFast>();
    reg_pair<RhsVanDerPol, PrecMixed>();
    reg_pair<RhsPendulum, PrecMixed>();
    reg_pair<RhsLorenz, PrecMixed>();
    reg_pair<RhsHarmonic, PrecMixed>();
}

}  // namespace degpu
