// FP32-pair stage group-per-system kernels (DOP853), resumable: the server's rounds of the tight
// class of a mixed request of FPU-beta chains, the layouts of up to 64 components (with output
// times) or 128 (without; beyond, FP64 fast is as fast or faster).
#include "group_erk.cuh"

namespace degpu {
void register_group_pair853_rounds() {
    reg_group_round<TabDop853, PrecMixedPair, 8, 1>();
    reg_group_round<TabDop853, PrecMixedPair, 16, 1>();
    reg_group_round<TabDop853, PrecMixedPair, 32, 1>();
    reg_group_round<TabDop853, PrecMixedPair, 32, 2>();
    reg_group_round_final<TabDop853, PrecMixedPair, 32, 4>();
}
}  // namespace degpu
