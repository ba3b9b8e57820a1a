// side_paths.cuh — solve paths implemented outside the one-system-per-thread kernels: the
// group-per-system kernels for ragged systems (group_erk.cu) and run-time compiled right-hand
// sides (nvrtc_rhs.cu).
#pragma once

#include <cuda_runtime.h>

#include "erk_core.cuh"

namespace degpu {
// Group-per-system solve of ragged (per-instance dimension) problems: the FPU-beta chain family.
degpu_status group_solve(const degpu_problem* pb, const degpu_method_cfg* cfg, const EnsArgs& a, const int32_t* dims,
                        cudaStream_t s);
// Right-hand sides compiled at run time with NVRTC.
degpu_status nvrtc_rhs_info(int32_t id, int32_t* dim, int32_t* n_params);
degpu_status nvrtc_solve(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                         degpu_batch_out* out, cudaStream_t s);
}  // namespace degpu
