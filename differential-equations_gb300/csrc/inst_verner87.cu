// inst_verner87.cu — Verner's pairs RKV877e and RKV878e of the Adaptive family, FP64 fast arithmetic
// (also what a mixed solve of these pairs runs), one system per thread, with and without dense
// output.
#include "registry.cuh"

namespace degpu {

template <class Rhs, class P>
static void reg() {
    register_thread_variant<TabRKV877E, Rhs, P>();
    register_thread_variant<TabRKV878E, Rhs, P>();
}

void register_verner87_fast() {
    reg<RhsVanDerPol, PrecFast>();
    reg<RhsPendulum, PrecFast>();
    reg<RhsLorenz, PrecFast>();
}

}  // namespace degpu
