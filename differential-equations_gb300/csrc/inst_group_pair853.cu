// FP32-pair stage group-per-system kernels (DOP853, the tight class of a mixed solve of FPU-beta
// chains), run to completion, the layouts of up to 64 components (with output times) or 128
// (without; beyond, FP64 fast is as fast or faster) (the resumable ones for the server are in
// inst_group_pair853_round.cu).
#include "group_erk.cuh"

namespace degpu {
void register_group_pair853() {
    reg_group<TabDop853, PrecMixedPair, 8, 1>();
    reg_group<TabDop853, PrecMixedPair, 16, 1>();
    reg_group<TabDop853, PrecMixedPair, 32, 1>();
    reg_group<TabDop853, PrecMixedPair, 32, 2>();
    reg_group_final<TabDop853, PrecMixedPair, 32, 4>();
}
}  // namespace degpu
