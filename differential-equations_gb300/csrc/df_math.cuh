// df_math.cuh — double-float arithmetic ("FP32 pairs"): a value is the unevaluated sum hi + lo
// of two FP32 numbers with |lo| <= ulp(hi) / 2, about 48 significant bits.
//
// Why: on this GPU an FP64 instruction costs the issue time of 64 FP32 ones, while a pair
// operation takes 6 to 11 FP32 instructions.  The mixed form uses pairs for the stages of
// instances whose tolerance is below what FP32 stages can meet (their rounding puts a floor of
// about 1e-7 under the error), so those instances keep FP64-like accuracy at a fraction of the
// FP64 cost.
//
// Methods (published, standard): TwoSum (Knuth), FastTwoSum (Dekker), TwoProduct through a
// fused multiply-add, and Dekker's pair addition and multiplication as analysed by Joldes,
// Muller and Popescu ("Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 2017).  Additions are the "sloppy" form: its error is below
// 2^-46 of the larger operand, which is what an ODE stage needs (the state's magnitude sets the
// scale).  sin and cos reduce by multiples of pi/2 (split in three FP32 parts, the products
// formed exactly), then evaluate the Taylor series with the leading terms in pairs and the tail
// in FP32 (relative error about 1e-11 on the reduced range).
#pragma once

#if !defined(__CUDACC_RTC__)
#include <math.h>
#include <stdint.h>
#endif

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#define DF_CTOR __host__ __device__ constexpr
#else
#define DF_HD static inline
#define DF_CTOR constexpr
#endif

namespace degpu {

struct df {
    float hi, lo;
    df() = default;
    DF_CTOR df(float h, float l) : hi(h), lo(l) {}
    DF_CTOR df(float x) : hi(x), lo(0.0f) {}
    DF_CTOR df(int x) : hi((float)x), lo(0.0f) {}
    // nearest pair to a double (a compile-time constant in the stage loops)
    DF_CTOR df(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    // FP32 bookkeeping (the norm, the controller, stiffness detection) reads the leading part
    DF_CTOR operator float() const { return hi; }
};

DF_HD df df_fast_two_sum(float a, float b) {
    const float s = a + b;
    return df(s, b - (s - a));
}
DF_HD df df_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return df(s, (a - (s - bb)) + (b - bb));
}

DF_HD df operator+(df a, df b) {
    df s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
DF_HD df operator+(df a, float b) {
    df s = df_two_sum(a.hi, b);
    return df_fast_two_sum(s.hi, s.lo + a.lo);
}
DF_HD df operator+(float a, df b) { return b + a; }
DF_HD df operator-(df a) { return df(-a.hi, -a.lo); }
DF_HD df operator-(df a, df b) { return a + (-b); }
DF_HD df operator-(df a, float b) { return a + (-b); }
DF_HD df operator-(float a, df b) { return (-b) + a; }
DF_HD df operator*(df a, df b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}
DF_HD df operator*(df a, float b) {
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return df_fast_two_sum(p, e);
}
DF_HD df operator*(float a, df b) { return b * a; }
DF_HD df& operator+=(df& a, df b) { return a = a + b; }

// The value of a pair as a double (exact: the sum of two FP32 numbers fits in 53 bits)
DF_HD double to_f64(df x) { return (double)x.hi + (double)x.lo; }
DF_HD double to_f64(float x) { return (double)x; }
DF_HD double to_f64(double x) { return x; }

// sin and cos of a pair.  x = k pi/2 + r with |r| <= pi/4; pi/2 = C1 + C2 + C3 (FP32 parts).
DF_HD df df_reduce_pio2(df x, float& kq) {
    const float C1 = 0x1.921fb6p+0f, C2 = -0x1.777a5cp-25f, C3 = -0x1.ee59dap-50f;
    const float k = rintf(x.hi * 0x1.45f306p-1f);  // x / (pi/2)
    kq = k;
    // x - k C1 - k C2 - k C3, each product exact as a pair (TwoProduct)
    const float p1 = k * C1, e1 = fmaf(k, C1, -p1);
    df r = df_two_sum(x.hi, -p1);          // cancels most of x.hi
    r = r + (x.lo - e1);
    const float p2 = k * C2, e2 = fmaf(k, C2, -p2);
    r = r - df(p2, e2);
    r = r - k * C3;
    return r;
}

// sin r and cos r for |r| <= pi/4 (z = r^2): the terms through r^7 (r^6) in pairs, the tail in FP32
DF_HD df df_sin_poly(df r, df z) {
    const float zf = z.hi;
    float t = fmaf(zf, 0x1.952c78p-49f, -0x1.ae7f3ep-41f);  //  1/17!, -1/15!
    t = fmaf(t, zf, 0x1.612462p-33f);                       //  1/13!
    t = fmaf(t, zf, -0x1.ae6456p-26f);                      // -1/11!
    t = fmaf(t, zf, 0x1.71de3ap-19f);                       //  1/9!
    // -1/7! + z t, 1/5! + z (..), -1/3! + z (..) in pairs
    df s = z * t + df(-0x1.a01a02p-13f, 0x1.7f97fap-39f);   // -1/5040
    s = z * s + df(0x1.111112p-7f, -0x1.dddddep-32f);       //  1/120
    s = z * s + df(-0x1.555556p-3f, 0x1.555556p-28f);       // -1/6
    return r + (r * z) * s;
}
DF_HD df df_cos_poly(df z) {
    const float zf = z.hi;
    float t = fmaf(zf, -0x1.682786p-53f, 0x1.ae7f3ep-45f);  // -1/18!, 1/16!
    t = fmaf(t, zf, -0x1.93974ap-37f);                      // -1/14!
    t = fmaf(t, zf, 0x1.1eed8ep-29f);                       //  1/12!
    t = fmaf(t, zf, -0x1.27e4fcp-22f);                      // -1/10!
    df s = z * t + df(0x1.a01a02p-16f, -0x1.7f97fap-42f);   //  1/40320
    s = z * s + df(-0x1.6c16c2p-10f, 0x1.27d27ep-35f);      // -1/720
    s = z * s + df(0x1.555556p-5f, -0x1.555556p-30f);       //  1/24
    s = z * s + df(-0.5f);
    return z * s + df(1.0f);
}
DF_HD df df_sin(df x) {
    float k;
    const df r = df_reduce_pio2(x, k);
    const df z = r * r;
    const int q = (int)k & 3;
    df v = (q & 1) ? df_cos_poly(z) : df_sin_poly(r, z);
    return (q & 2) ? -v : v;
}
DF_HD df df_cos(df x) {
    float k;
    const df r = df_reduce_pio2(x, k);
    const df z = r * r;
    const int q = (int)k & 3;
    df v = (q & 1) ? df_sin_poly(r, z) : df_cos_poly(z);
    return (q == 1 || q == 2) ? -v : v;
}

}  // namespace degpu
