// FP32-pair stage group-per-system kernels (DOP853, the tight class of a mixed solve of FPU-beta chains),
// run to completion, every layout of the default dimension buckets (the resumable ones for the
// server are in inst_group_pair853_round.cu).
#include "group_erk.cuh"

namespace degpu {
void register_group_pair853() {
    reg_group<TabDop853, PrecMixedPair, 8, 1>();
    reg_group<TabDop853, PrecMixedPair, 16, 1>();
    reg_group<TabDop853, PrecMixedPair, 32, 1>();
    reg_group<TabDop853, PrecMixedPair, 32, 2>();
    reg_group<TabDop853, PrecMixedPair, 32, 4>();
    reg_group<TabDop853, PrecMixedPair, 32, 8>();
}
}  // namespace degpu
