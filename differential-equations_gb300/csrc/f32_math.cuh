// f32_math.cuh — FP32 sine and cosine for the mixed form's right-hand sides.
//
// Method:
//   * Cody–Waite argument reduction (W. J. Cody and W. Waite, "Software Manual for the
//     Elementary Functions", 1980): sin reduces x by the nearest multiple k*pi, cos by the
//     nearest odd multiple (k + 1/2)*pi. pi is split into three FP32 parts, each removed with one
//     fused multiply-add, leaving r in [-pi/2, pi/2];
//   * on r, the Taylor polynomial of sin to r^13 (truncation below 7e-10 on [-pi/2, pi/2]),
//     evaluated by Horner's rule with fused multiply-adds;
//   * the parity of k gives the sign: sin x = (-1)^k sin r, cos x = (-1)^(k+1) sin r.
// One polynomial serves both functions, so a call evaluates one polynomial and takes no branch on
// the quadrant. Every operation is an explicit FP32 multiply or fused multiply-add, so a host
// build (g++) returns the same bits as the device.
// Accurate to about one unit in the last place for |x| < 1e5 (sin(-0) returns +0). Beyond that
// the functions fall back to the library's sinf/cosf.
#pragma once

#if !defined(__CUDACC_RTC__)
#include <math.h>
#include <string.h>
#endif

#if defined(__CUDACC__)
#define F32M_HD __host__ __device__ __forceinline__
#else
#define F32M_HD static inline
#endif

namespace degpu {
namespace f32m {

// sin r for |r| <= pi/2
F32M_HD float sin_poly(float r) {
    const float r2 = r * r;
    float p = fmaf(r2, 0x1.612462p-33f, -0x1.ae6456p-26f);  //  1/13!, -1/11!
    p = fmaf(p, r2, 0x1.71de3ap-19f);                         //  1/9!
    p = fmaf(p, r2, -0x1.a01a02p-13f);                        // -1/7!
    p = fmaf(p, r2, 0x1.111112p-7f);                          //  1/5!
    p = fmaf(p, r2, -0x1.555556p-3f);                         // -1/3!
    return fmaf(r * r2, p, r);
}

// x - m*pi for an integral or half-integral m, pi = P1 + P2 + P3 (+ 2.1e-23)
F32M_HD float reduce_pi(float x, float m) {
    float r = fmaf(m, -0x1.921fb6p+1f, x);
    r = fmaf(m, 0x1.777a5cp-24f, r);
    return fmaf(m, 0x1.ee59dap-49f, r);
}

F32M_HD float flip_sign(float v, int odd) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(__float_as_uint(v) ^ ((unsigned int)odd << 31));
#else
    unsigned int u;
    memcpy(&u, &v, 4);
    u ^= (unsigned int)odd << 31;
    memcpy(&v, &u, 4);
    return v;
#endif
}

F32M_HD float sin_f32(float x) {
    if (!(fabsf(x) < 1.0e5f)) return sinf(x);
    const float k = rintf(x * 0x1.45f306p-2f);  // x / pi
    return flip_sign(sin_poly(reduce_pi(x, k)), (int)k & 1);
}

F32M_HD float cos_f32(float x) {
    if (!(fabsf(x) < 1.0e5f)) return cosf(x);
    const float k = rintf(fmaf(x, 0x1.45f306p-2f, -0.5f));  // x / pi - 1/2
    return flip_sign(sin_poly(reduce_pi(x, k + 0.5f)), ((int)k & 1) ^ 1);
}

}  // namespace f32m
}  // namespace degpu
