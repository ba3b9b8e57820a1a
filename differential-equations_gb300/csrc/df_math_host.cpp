// Host build of df_math.cuh and f64_tab_math.cuh so that the pair arithmetic and the pair and
// FP64 table-driven sin/cos can be tested without a GPU.  Compiled with -ffp-contract=off: every fused multiply-add is an explicit fmaf, as on the
// device.
#include <stdint.h>

#include "df_math.cuh"
#include "f64_tab_math.cuh"

extern "C" {
// sin and cos of the pairs (hi[i], lo[i])
void degpu_host_df_sincos(const float* hi, const float* lo, double* s, double* c, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        const degpu::df x(hi[i], lo[i]);
        s[i] = degpu::to_f64(degpu::df_sin(x));
        c[i] = degpu::to_f64(degpu::df_cos(x));
    }
}
// a * b + c on pairs, and a - b
void degpu_host_df_ops(const float* ah, const float* al, const float* bh, const float* bl, const float* ch,
                       const float* cl, double* fma_out, double* sub_out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        const degpu::df a(ah[i], al[i]), b(bh[i], bl[i]), c(ch[i], cl[i]);
        fma_out[i] = degpu::to_f64(a * b + c);
        sub_out[i] = degpu::to_f64(a - b);
    }
}
// the plain FP64 form's table-driven sin and cos
void degpu_host_f64t_sincos(const double* x, double* s, double* c, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        s[i] = degpu::f64t::sin(x[i]);
        c[i] = degpu::f64t::cos(x[i]);
    }
}
// y + sum_j a_j k_j over m terms through the lazily normalised accumulator (the stage sums);
// a, k: [m][n], the last term's factor is FP32 (the step size) when last_f32 is set
void degpu_host_df_stage_sum(const float* yh, const float* yl, const float* ah, const float* al, const float* kh,
                             const float* kl, int32_t m, int32_t last_f32, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        degpu::dfacc s = degpu::acc_begin(degpu::df(yh[i], yl[i]));
        for (int32_t j = 0; j < m; ++j) {
            const degpu::df k(kh[j * n + i], kl[j * n + i]);
            if (last_f32 && j == m - 1)
                degpu::acc_fma(s, k, ah[j * n + i]);
            else
                degpu::acc_fma(s, degpu::df(ah[j * n + i], al[j * n + i]), k);
        }
        out[i] = degpu::to_f64(degpu::acc_end(s));
    }
}
}
