// f64_tab_math.cuh — FP64 sine and cosine for the plain FP64 form's right-hand sides.
//
// Method: table-driven reduction (Tang's table-driven elementary functions, ACM TOMS
// 1989-1992).  x = j pi/64 + d with |d| <= about pi/128:
//   * j and d: x 64/pi is rounded to an integer by adding 1.5 2^52 (the integer sits in the low
//     bits of the sum, so j mod 128 is read from the bit pattern without a conversion); pi/64 is
//     split into two doubles, each removed with one fused multiply-add (Cody and Waite);
//   * S, C = sin, cos(j pi/64) from a 128-row table of double-double values (two 16-byte loads);
//     the low parts enter the small terms, so the table adds no rounding of its own;
//   * the Taylor series of the small d, z = d^2:
//       sin d = d + sm,  sm = d z (-1/6 + z (1/120 - z/5040))     (next term below 1e-20)
//       cos d = 1 + cm,  cm = z (-1/2 + z (1/24 - z/720))           (next term below 4e-18)
//   * sin x = S + (C d + (S cm + (C sm + S_lo))),  cos x = C - (S d - (C cm - (S sm - C_lo))).
// About 16 FP64 instructions, against several times that for a general-purpose routine.  Within
// one unit in the last place for |x| < 2^40 and correctly rounded on about 98 % of arguments
// (tested against correctly rounded values on the host).  Larger or non-finite arguments fall
// back to the library's sin and cos.
#pragma once

#if !defined(__CUDACC_RTC__)
#include <math.h>
#include <stdint.h>
#include <string.h>
#endif

#include "df_tables.inc"

#if defined(__CUDACC__)
#define F64T_DEV __device__ __forceinline__
#else
#define F64T_DEV static inline
#endif

namespace degpu {
namespace f64t {

#if defined(__CUDACC__)
static __device__ __align__(32) const double kTrig64[128][4] = {F64_TRIG_TAB_ROWS};
#else
alignas(32) static const double kTrig64[128][4] = {F64_TRIG_TAB_ROWS};
#endif

// S, C (and their low parts Sl, Cl), d, sm and cm of the method above
F64T_DEV void parts(double x, double& S, double& C, double& Sl, double& Cl, double& d, double& sm, double& cm) {
    const double MAGIC = 0x1.8p52;
    const double t = fma(x, F64_64_OVER_PI, MAGIC);
    const double kf = t - MAGIC;
#if defined(__CUDACC__)
    const int j = __double2loint(t) & 127;
    const double2 hi = __ldg(reinterpret_cast<const double2*>(&kTrig64[j][0]));
    const double2 lo = __ldg(reinterpret_cast<const double2*>(&kTrig64[j][2]));
    S = hi.x;
    C = hi.y;
    Sl = lo.x;
    Cl = lo.y;
#else
    uint64_t bits;
    memcpy(&bits, &t, sizeof bits);
    const int j = (int)(bits & 127u);
    S = kTrig64[j][0];
    C = kTrig64[j][1];
    Sl = kTrig64[j][2];
    Cl = kTrig64[j][3];
#endif
    d = fma(-kf, F64_PIO64_1, x);
    d = fma(-kf, F64_PIO64_2, d);
    const double z = d * d;
    sm = (d * z) * fma(z, fma(z, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0);
    cm = z * fma(z, fma(z, -1.0 / 720.0, 1.0 / 24.0), -0.5);
}

F64T_DEV double sin(double x) {
    if (!(fabs(x) < 0x1p40)) return ::sin(x);
    double S, C, Sl, Cl, d, sm, cm;
    parts(x, S, C, Sl, Cl, d, sm, cm);
    return S + fma(C, d, fma(S, cm, fma(C, sm, Sl)));
}

F64T_DEV double cos(double x) {
    if (!(fabs(x) < 0x1p40)) return ::cos(x);
    double S, C, Sl, Cl, d, sm, cm;
    parts(x, S, C, Sl, Cl, d, sm, cm);
    return C - fma(S, d, fma(-C, cm, fma(S, sm, -Cl)));
}

}  // namespace f64t
}  // namespace degpu
