#include "wps.cuh"
namespace degpu {
degpu_status nvrtc_rhs_info(int32_t, int32_t*, int32_t*) { return DEGPU_UNSUPPORTED; }
degpu_status nvrtc_solve(const degpu_problem*, const degpu_method_cfg*, const degpu_batch_in*, degpu_batch_out*, cudaStream_t) { return DEGPU_UNSUPPORTED; }
}
extern "C" {
degpu_status degpu_register_rhs_nvrtc(const char*, const char*, int32_t, int32_t, int32_t*, char*, size_t) { return DEGPU_UNSUPPORTED; }
degpu_status degpu_gray_scott_rk4(const degpu_gray_scott*, int32_t, double, double, int64_t, void*, void*, void*) { return DEGPU_UNSUPPORTED; }
degpu_status degpu_gray_scott_rhs(const degpu_gray_scott*, const double*, const double*, double*, double*, void*) { return DEGPU_UNSUPPORTED; }
}
