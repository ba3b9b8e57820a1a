// Parity (FP64, no FMA contraction) variants of the crate's test systems
// (tests/ode/systems.rs).  Compiled with -fmad=false.
#include "registry.cuh"

#if defined(__CUDACC__) && !defined(DEGPU_NO_FMAD)
#error "parity translation units must be compiled with -fmad=false -DDEGPU_NO_FMAD"
#endif

namespace degpu {
template <class Rhs>
static void reg_all() {
    register_variant<TabDopri5, Rhs, PrecParity>();
    register_variant<TabDop853, Rhs, PrecParity>();
    register_variant<TabRK4, Rhs, PrecParity>();
    register_rhs<Rhs, PrecParity>();
}
void register_parity_tests() {
    reg_all<RhsExpGrowth>();
    reg_all<RhsLinear>();
    reg_all<RhsHarmonic>();
    reg_all<RhsLogistic>();
    reg_all<RhsRobertson>();
    reg_all<RhsHires>();
    reg_all<RhsBrusselator>();
    reg_all<RhsCr3bp>();
    reg_all<RhsPipeHeat>();
    reg_all<RhsDampedQuadrature>();
}
}  // namespace degpu
