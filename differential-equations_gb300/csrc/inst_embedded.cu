// inst_embedded.cu — the Adaptive ERK family (RKF45, Cash-Karp), and DOPRI5 / DOP853 on the
// harmonic and pipe-heat systems, FP64 fast and mixed arithmetic, one system per thread.
#include "registry.cuh"

namespace degpu {

template <class Rhs, class P>
static void reg_pair() {
    register_thread_variant<TabRKF45, Rhs, P>();
    register_thread_variant<TabCashKarp, Rhs, P>();
}

// DOPRI5 / DOP853 on the linear test systems the shooting methods are tested with.
template <class Rhs, class P>
static void reg_dp() {
    register_thread_variant<TabDopri5, Rhs, P>();
    register_thread_variant<TabDop853, Rhs, P>();
}

void register_embedded_fast_mixed() {
    reg_dp<RhsHarmonic, PrecFast>();
    reg_dp<RhsPipeHeat, PrecFast>();
    reg_dp<RhsHarmonic, PrecMixed>();
    reg_dp<RhsPipeHeat, PrecMixed>();
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
