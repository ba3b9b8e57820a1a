// Resumable group-per-system kernels of the server (ragged FPU-beta requests): DOPRI5 and DOP853,
// FP64_FAST and the FP32-stage mixed form, every (G, CPL) layout of the default buckets.
#include "group_erk.cuh"

namespace degpu {
void register_group_rounds() {
    reg_group_round<TabDop853, PrecFast, 8, 1>();
    reg_group_round<TabDop853, PrecFast, 16, 1>();
    reg_group_round<TabDop853, PrecFast, 32, 1>();
    reg_group_round<TabDop853, PrecFast, 32, 2>();
    reg_group_round<TabDop853, PrecFast, 32, 4>();
    reg_group_round<TabDop853, PrecFast, 32, 8>();
    reg_group_round<TabDop853, PrecMixed, 8, 1>();
    reg_group_round<TabDop853, PrecMixed, 16, 1>();
    reg_group_round<TabDop853, PrecMixed, 32, 1>();
    reg_group_round<TabDop853, PrecMixed, 32, 2>();
    reg_group_round<TabDop853, PrecMixed, 32, 4>();
    reg_group_round<TabDop853, PrecMixed, 32, 8>();
    reg_group_round<TabDopri5, PrecFast, 8, 1>();
    reg_group_round<TabDopri5, PrecFast, 16, 1>();
    reg_group_round<TabDopri5, PrecFast, 32, 1>();
    reg_group_round<TabDopri5, PrecFast, 32, 2>();
    reg_group_round<TabDopri5, PrecFast, 32, 4>();
    reg_group_round<TabDopri5, PrecFast, 32, 8>();
    reg_group_round<TabDopri5, PrecMixed, 8, 1>();
    reg_group_round<TabDopri5, PrecMixed, 16, 1>();
    reg_group_round<TabDopri5, PrecMixed, 32, 1>();
    reg_group_round<TabDopri5, PrecMixed, 32, 2>();
    reg_group_round<TabDopri5, PrecMixed, 32, 4>();
    reg_group_round<TabDopri5, PrecMixed, 32, 8>();
}
}  // namespace degpu
