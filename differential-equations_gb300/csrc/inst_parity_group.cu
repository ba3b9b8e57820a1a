// Parity (FP64, no FMA contraction) variants of the group-per-system kernel.
// Compiled with -fmad=false.
#include "group_erk.cuh"

#if defined(__CUDACC__) && !defined(DEGPU_NO_FMAD)
#error "parity translation units must be compiled with -fmad=false -DDEGPU_NO_FMAD"
#endif

namespace degpu {
void register_group_parity() {
    reg_group<TabDop853, PrecParity, 8, 1>();
    reg_group<TabDop853, PrecParity, 16, 1>();
    reg_group<TabDop853, PrecParity, 32, 1>();
    reg_group<TabDop853, PrecParity, 16, 2>();
    reg_group<TabDop853, PrecParity, 16, 4>();
    reg_group<TabDop853, PrecParity, 32, 2>();
    reg_group<TabDop853, PrecParity, 32, 4>();
    reg_group<TabDop853, PrecParity, 32, 8>();
    reg_group<TabDopri5, PrecParity, 8, 1>();
    reg_group<TabDopri5, PrecParity, 16, 1>();
    reg_group<TabDopri5, PrecParity, 32, 1>();
    reg_group<TabDopri5, PrecParity, 32, 2>();
    reg_group<TabDopri5, PrecParity, 32, 4>();
    reg_group<TabDopri5, PrecParity, 32, 8>();
}
}  // namespace degpu
