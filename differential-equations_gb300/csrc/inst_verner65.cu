// inst_verner65.cu — Verner's pairs RKV655e and RKV656e of the Adaptive family, FP64 fast arithmetic
// (also what a mixed solve of these pairs runs), one system per thread, with and without dense
// output.
#include "registry.cuh"

namespace degpu {

template <class Rhs, class P>
static void reg() {
    register_thread_variant<TabRKV655E, Rhs, P>();
    register_thread_variant<TabRKV656E, Rhs, P>();
}

void register_verner65_fast() {
    reg<RhsVanDerPol, PrecFast>();
    reg<RhsPendulum, PrecFast>();
    reg<RhsLorenz, PrecFast>();
}

}  // namespace degpu
