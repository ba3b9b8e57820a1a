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
// scale).  sin and cos are table-driven (see df_sin below).
#pragma once

#if !defined(__CUDACC_RTC__)
#include <math.h>
#include <stdint.h>
#endif

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#define DF_DEV __device__ __forceinline__
#define DF_CTOR __host__ __device__ constexpr
#else
#define DF_HD static inline
#define DF_DEV static inline
#define DF_CTOR constexpr
#endif

#include "df_tables.inc"

// A product that the compiler must not fuse into a following addition: the error-free
// transformations below rely on the rounded product, and every build (ahead of time or at run
// time) then evaluates a pair expression identically.
#if defined(__CUDA_ARCH__)
#define DF_MUL(a, b) __fmul_rn((a), (b))
#else
#define DF_MUL(a, b) ((a) * (b))
#endif

namespace degpu {

// sin and cos of j pi/64, j = 0..127, as pairs: one 16-byte row per j (sin hi, sin lo, cos hi,
// cos lo), read through the read-only data cache
#if defined(__CUDACC__)
static __device__ __align__(16) const float kDfTrigTab[128][4] = {DF_TRIG_TAB_ROWS};
#else
alignas(16) static const float kDfTrigTab[128][4] = {DF_TRIG_TAB_ROWS};
#endif

struct df {
    float hi, lo;
    df() = default;
    DF_CTOR df(float h, float l) : hi(h), lo(l) {}
    DF_CTOR df(float x) : hi(x), lo(0.0f) {}
    DF_CTOR df(int x) : hi((float)x), lo(0.0f) {}
    // nearest pair to a double (a compile-time constant in the stage loops)
    DF_CTOR df(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    // FP32 bookkeeping (the norm, the controller, stiffness detection) reads the leading part.
    // Explicit, so that a function without a pair overload never takes a pair silently.
    DF_CTOR explicit operator float() const { return hi; }
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
// Products are left as (p, e) without the final FastTwoSum: e is the product's rounding error plus
// the cross terms, within about 1.5 units of p's last place, a pair every operation here accepts
// (sums re-split the leading parts with TwoSum; products only need |lo| small against |hi|).
DF_HD df operator*(df a, df b) {
    const float p = DF_MUL(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df(p, e);
}
DF_HD df operator*(df a, float b) {
    const float p = DF_MUL(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return df(p, e);
}
DF_HD df operator*(float a, df b) { return b * a; }
DF_HD df& operator+=(df& a, df b) { return a = a + b; }

// Stage sums y + sum_j a_j k_j.  For pairs the sum is kept unnormalised: each product is formed
// as a pair (TwoProduct plus the cross terms), its leading part is added to the running leading
// part with TwoSum, and every low-order part goes into the running low part; one FastTwoSum
// normalises at the end.  12 FP32 instructions per term instead of 18 for a pair product followed
// by a pair addition, with the same error bound (a few units of 2^-48 of the largest term).  For
// FP32 and FP64 the accumulator is the number itself and a term is `s + a * b`, the expression
// the stage sums have always used.
struct dfacc {
    float hi, lo;
};
template <class S>
struct AccOf {
    using type = S;
};
template <>
struct AccOf<df> {
    using type = dfacc;
};
DF_HD float acc_begin(float y) { return y; }
DF_HD double acc_begin(double y) { return y; }
DF_HD dfacc acc_begin(df y) { return dfacc{y.hi, y.lo}; }
DF_HD void acc_fma(float& s, float a, float b) { s = s + a * b; }
DF_HD void acc_fma(double& s, double a, double b) { s = s + a * b; }
DF_HD void acc_add_pair(dfacc& s, float p, float e) {
    const float t = s.hi + p;
    const float bb = t - s.hi;
    const float err = (s.hi - (t - bb)) + (p - bb);
    s.hi = t;
    s.lo = s.lo + (e + err);
}
DF_HD void acc_fma(dfacc& s, df a, df b) {
    const float p = DF_MUL(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    acc_add_pair(s, p, e);
}
DF_HD void acc_fma(dfacc& s, df a, float b) {
    const float p = DF_MUL(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    acc_add_pair(s, p, e);
}
DF_HD float acc_end(float s) { return s; }
DF_HD double acc_end(double s) { return s; }
DF_HD df acc_end(dfacc s) { return df_fast_two_sum(s.hi, s.lo); }

// The leading FP32 part (the FP32 bookkeeping's view of a stage value)
DF_HD float lead(df x) { return x.hi; }
DF_HD float lead(float x) { return x; }

// The value of a pair as a double (exact: the sum of two FP32 numbers fits in 53 bits)
DF_HD double to_f64(df x) { return (double)x.hi + (double)x.lo; }
DF_HD double to_f64(float x) { return (double)x; }
DF_HD double to_f64(double x) { return x; }

// sin and cos of a pair, table-driven (the method of Tang's table-driven elementary functions,
// ACM TOMS 1989-1992): x = j pi/64 + d with |d| <= about pi/128, then
//     sin x = S cos d + C sin d,   cos x = C cos d - S sin d,
// S, C = sin, cos(j pi/64) from a 128-row table of pairs, and the Taylor series of the small d:
//     cos d = 1 - h + h q,  h = d^2/2 (a pair), q = d^2/12 - d^4/360 (FP32, |q| < 5.1e-5)
//     sin d = d + s,        s = -d^3/6 + d^5/120 (FP32, |s| < 2.5e-6)
// The neglected terms are below 4e-16.  The sums run through the stage-sum accumulator, so a
// call costs about 60 FP32 instructions and one 16-byte table load.  Absolute error about 1e-12
// (the FP32 parts s and h q), plus 2^-47 |x| from the reduction's FP32 tail.
DF_DEV df df_reduce_pio64(df x, int& j) {
    const float kf = rintf(x.hi * DF_64_OVER_PI);
    j = (int)kf & 127;  // the table row of kf mod 128 (two's complement for kf < 0)
    const float p1 = DF_MUL(kf, DF_PIO64_1), e1 = fmaf(kf, DF_PIO64_1, -p1);
    const float p2 = DF_MUL(kf, DF_PIO64_2), e2 = fmaf(kf, DF_PIO64_2, -p2);
    const df r = df_two_sum(x.hi, -p1);  // exact
    // the parts below ulp(x.hi): x.lo, the low part of kf C1, kf C2 and kf C3
    const float b = (((r.lo + x.lo) - e1) - p2) - fmaf(kf, DF_PIO64_3, e2);
    return df_fast_two_sum(r.hi, b);
}

DF_DEV void df_trig_row(int j, df& S, df& C) {
#if defined(__CUDACC__)
    const float4 row = __ldg(reinterpret_cast<const float4*>(&kDfTrigTab[j][0]));
    S = df(row.x, row.y);
    C = df(row.z, row.w);
#else
    S = df(kDfTrigTab[j][0], kDfTrigTab[j][1]);
    C = df(kDfTrigTab[j][2], kDfTrigTab[j][3]);
#endif
}

// d^2/2 as a pair (hh, hl), h q and s of the series above.  s is formed from d^3 to about
// 2^-40 (its leading product exact, the low parts of d and d^2 folded in) and 1/6 as a pair, so
// that its one final rounding is its only sizeable error.
DF_DEV void df_small_series(df d, float& hh, float& hl, float& hq, float& s) {
    const float p = DF_MUL(d.hi, d.hi);
    float e = fmaf(d.hi, d.hi, -p);
    e = fmaf(2.0f * d.hi, d.lo, e);  // d^2 = p + e
    hh = 0.5f * p;
    hl = 0.5f * e;
    hq = hh * (p * fmaf(p, -1.0f / 360.0f, 1.0f / 12.0f));
    const float t = DF_MUL(d.hi, p);
    float tl = fmaf(d.hi, p, -t);
    tl = fmaf(d.hi, e, tl);
    tl = fmaf(p, d.lo, tl);  // d^3 = t + tl (d.hi e already carries 2 d.hi^2 d.lo of the 3)
    const float C6H = 0x1.555556p-3f, C6L = -0x1.555556p-28f;  // 1/6 = C6H + C6L
    const float inner = fmaf(t, C6L, tl * C6H);
    s = fmaf(t, -C6H, -inner);                    // -d^3/6
    s = fmaf(t * p, 1.0f / 120.0f, s);            // + d^5/120
}

DF_DEV df df_sin(df x) {
    int j;
    const df d = df_reduce_pio64(x, j);
    df S, C;
    df_trig_row(j, S, C);
    float hh, hl, hq, s;
    df_small_series(d, hh, hl, hq, s);
    dfacc a = acc_begin(S);
    acc_fma(a, C, d);
    acc_fma(a, -S, df(hh, hl));
    a.lo = fmaf(S.hi, hq, a.lo);
    a.lo = fmaf(C.hi, s, a.lo);
    return acc_end(a);
}
DF_DEV df df_cos(df x) {
    int j;
    const df d = df_reduce_pio64(x, j);
    df S, C;
    df_trig_row(j, S, C);
    float hh, hl, hq, s;
    df_small_series(d, hh, hl, hq, s);
    dfacc a = acc_begin(C);
    acc_fma(a, -S, d);
    acc_fma(a, -C, df(hh, hl));
    a.lo = fmaf(C.hi, hq, a.lo);
    a.lo = fmaf(-S.hi, s, a.lo);
    return acc_end(a);
}

// sin and cos under their usual names for pairs only (a run-time right-hand side written as
// `sin(y[0])` finds them by argument-dependent lookup when R is a pair).  They are templates that
// accept nothing but a pair, so no other argument is ever converted to one.
template <class T>
struct df_only {};
template <>
struct df_only<df> {
    using type = df;
};
template <class T>
DF_DEV typename df_only<T>::type sin(T x) {
    return df_sin(x);
}
template <class T>
DF_DEV typename df_only<T>::type cos(T x) {
    return df_cos(x);
}

}  // namespace degpu
