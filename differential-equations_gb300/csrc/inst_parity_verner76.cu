// inst_parity_verner76.cu — Verner's pairs RKV766e and RKV767e of the Adaptive family, FP64 parity
// arithmetic (compiled with -fmad=false like every inst_parity_* translation unit), one system per
// thread, with and without dense output.
#include "registry.cuh"

namespace degpu {

template <class Rhs>
static void reg() {
    register_thread_variant<TabRKV766E, Rhs, PrecParity>();
    register_thread_variant<TabRKV767E, Rhs, PrecParity>();
}

void register_verner76_parity() {
    reg<RhsExpGrowth>();
    reg<RhsHarmonic>();
    reg<RhsVanDerPol>();
    reg<RhsPendulum>();
    reg<RhsLorenz>();
}

}  // namespace degpu
