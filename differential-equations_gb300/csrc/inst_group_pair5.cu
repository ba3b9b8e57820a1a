// FP32-pair stage group-per-system kernels (DOPRI5, the tight class of a mixed solve of FPU-beta chains),
// run to completion and resumable (the server), every layout of the default dimension buckets.
#include "group_erk.cuh"

namespace degpu {
void register_group_pair5() {
    reg_group<TabDopri5, PrecMixedPair, 8, 1>();
    reg_group<TabDopri5, PrecMixedPair, 16, 1>();
    reg_group<TabDopri5, PrecMixedPair, 32, 1>();
    reg_group<TabDopri5, PrecMixedPair, 32, 2>();
    reg_group<TabDopri5, PrecMixedPair, 32, 4>();
    reg_group<TabDopri5, PrecMixedPair, 32, 8>();
    reg_group_round<TabDopri5, PrecMixedPair, 8, 1>();
    reg_group_round<TabDopri5, PrecMixedPair, 16, 1>();
    reg_group_round<TabDopri5, PrecMixedPair, 32, 1>();
    reg_group_round<TabDopri5, PrecMixedPair, 32, 2>();
    reg_group_round<TabDopri5, PrecMixedPair, 32, 4>();
    reg_group_round<TabDopri5, PrecMixedPair, 32, 8>();
}
}  // namespace degpu
