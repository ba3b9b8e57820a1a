// Host build of dd_math.cuh (and f32_math.cuh) so that their results can be tested without a GPU.
// Compiled with -ffp-contract=off, like the parity device code (-fmad=false).
#include <stdint.h>
#include "dd_math.cuh"
#include "f32_math.cuh"

extern "C" {
void degpu_host_pow_ctrl(const double* x, double y, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = degpu::ddm::pow_ctrl(x[i], y);
}
void degpu_host_pow_ctrl_neg(const double* x, double y, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = degpu::ddm::pow_ctrl_neg(x[i], y);
}
// e[i] = 1 - x[i] s[i]^q through the controller power's fixed-point residual; NaN where x s^q lies
// outside [1/2, 2)
void degpu_host_pow_residual(const double* x, const double* s, int q, double* e, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        bool ok;
        const double r = degpu::ddm::pow_ctrl_residual(x[i], s[i], q, ok);
        e[i] = ok ? r : NAN;
    }
}
void degpu_host_sincos_f32(const float* x, float* s, float* c, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        s[i] = degpu::f32m::sin_f32(x[i]);
        c[i] = degpu::f32m::cos_f32(x[i]);
    }
}
void degpu_host_sincos_cr(const double* x, double* s, double* c, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        s[i] = degpu::ddm::sin_cr(x[i]);
        c[i] = degpu::ddm::cos_cr(x[i]);
    }
}
}
