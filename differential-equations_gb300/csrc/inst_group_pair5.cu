// FP32-pair stage group-per-system kernels (DOPRI5, the tight class of a mixed solve of FPU-beta
// chains), run to completion and resumable (the server), the layouts of up to 64 components (with
// output times) or 128 (without; beyond, FP64 fast is as fast or faster).
#include "group_erk.cuh"

namespace degpu {
void register_group_pair5() {
    reg_group<TabDopri5, PrecMixedPair, 8, 1>();
    reg_group<TabDopri5, PrecMixedPair, 16, 1>();
    reg_group<TabDopri5, PrecMixedPair, 32, 1>();
    reg_group<TabDopri5, PrecMixedPair, 32, 2>();
    reg_group_final<TabDopri5, PrecMixedPair, 32, 4>();
    reg_group_round<TabDopri5, PrecMixedPair, 8, 1>();
    reg_group_round<TabDopri5, PrecMixedPair, 16, 1>();
    reg_group_round<TabDopri5, PrecMixedPair, 32, 1>();
    reg_group_round<TabDopri5, PrecMixedPair, 32, 2>();
    reg_group_round_final<TabDopri5, PrecMixedPair, 32, 4>();
}
}  // namespace degpu
