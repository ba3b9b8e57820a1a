// dd_math.cuh — correctly rounded (in practice) FP64 pow, sin and cos for the parity path.
//
// The crate computes `err.powf(-1/order)` in its step-size controller
// (src/methods/erk/dormandprince/ordinary.rs:152-157), `(0.01/der12).powf(1/order)` in its
// initial step heuristic (src/methods/h_init.rs:116-125), and user right-hand sides call
// `sin`/`cos`.  All of these go to the platform libm.  A GPU integrator can only reproduce the
// crate's accept/reject sequence bit for bit if these values are the same on both sides, so the
// parity path rounds them correctly: each function evaluates its result in double-double
// arithmetic to a relative accuracy near 2^-100 and rounds once.  The rounded result then equals
// the correctly rounded value except when the exact value lies within ~2^-100 of a rounding
// boundary, which for the inputs an integrator produces does not happen in practice.
//
// Methods (all standard published techniques):
//  - error-free transformations TwoSum / FastTwoSum (Knuth; Dekker) and TwoProduct via FMA
//    (Ogita, Rump, Oishi 2005), double-double arithmetic (Dekker 1971; Hida, Li, Bailey 2001);
//  - x^(±1/5): one double-double Newton step on r^5 = x from a few-ulp starting value
//    (quadratic convergence), then the factor x^(2^-54/5) = exp(2^-54 ln(x)/5) that turns 1/5
//    into the binary64 value 0.2 = (1/5)(1 + 2^-54) (truncated exponential series);
//  - the controller's x^(-0.2) and x^(-0.125) with few FP64 instructions (pow_ctrl_neg): an FP32
//    start on the range-reduced exponent, the residual 1 - x s^q in 128-bit fixed point on the
//    integer pipe, the binomial series of (1 - e)^(-1/q) and Ziv's rounding test (Ziv 1991), with
//    the double-double power behind it;
//  - x^(±1/8): three double-double square roots (Karp–Markstein correction);
//  - x^(±1/q), q = 6, 7, 9: Newton on s^-q = x finished in double-double, reciprocal for the
//    positive exponent, and the same exp correction for binary64 1/q;
//  - sin/cos: Cody–Waite reduction by pi/2 split into 33+33+53+53 bits (valid for |x| < 2^20),
//    reduction to |u| <= 1/128 around the table point j/64, double-double Taylor series and
//    the angle-addition formulas with the table sin(j/64), cos(j/64).
//
// Everything is written with explicit fma() where an exact product is needed and compiled
// without FMA contraction on the parity path, so host and device builds agree.
#pragma once

#if !defined(__CUDACC_RTC__)
#include <math.h>
#include <stdint.h>
#include <string.h>
#endif

#if defined(__CUDACC__)
#define DD_HD __host__ __device__ __forceinline__
#else
#define DD_HD static inline
#endif

namespace degpu {
namespace ddm {

#include "dd_tables.inc"

// sin(j/64), cos(j/64) as double-doubles: one copy for device code, one for host builds.
#if defined(__CUDACC__)
static __device__ const double dd_sincos_tab_dev[DD_TAB_N][4] = {DD_SINCOS_ROWS};
#endif
static const double dd_sincos_tab_host[DD_TAB_N][4] = {DD_SINCOS_ROWS};
DD_HD const double* dd_tab_row(int j) {
#if defined(__CUDA_ARCH__)
    return dd_sincos_tab_dev[j];
#else
    return dd_sincos_tab_host[j];
#endif
}

struct dd {
    double hi, lo;
};

DD_HD dd two_sum(double a, double b) {
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
// requires |a| >= |b| (or a == 0)
DD_HD dd fast_two_sum(double a, double b) {
    double s = a + b;
    double e = b - (s - a);
    return {s, e};
}
DD_HD dd two_prod(double a, double b) {
    double p = a * b;
    double e = fma(a, b, -p);
    return {p, e};
}
DD_HD dd dd_mul(dd a, dd b) {
    dd p = two_prod(a.hi, b.hi);
    double t = a.hi * b.lo;
    t = t + a.lo * b.hi;
    p.lo = p.lo + t;
    return fast_two_sum(p.hi, p.lo);
}
DD_HD dd dd_mul_d(dd a, double b) {
    dd p = two_prod(a.hi, b);
    p.lo = p.lo + a.lo * b;
    return fast_two_sum(p.hi, p.lo);
}
DD_HD dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    dd t = two_sum(a.lo, b.lo);
    s.lo = s.lo + t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo = s.lo + t.lo;
    return fast_two_sum(s.hi, s.lo);
}
DD_HD dd dd_neg(dd a) { return {-a.hi, -a.lo}; }

// Square root of a double-double (a.hi > 0).
DD_HD dd dd_sqrt(dd a) {
    double s = sqrt(a.hi);
    double e = fma(-s, s, a.hi);
    e = e + a.lo;
    double c = e / (s + s);
    return fast_two_sum(s, c);
}

// Reciprocal of a double-double (a.hi != 0, finite).
DD_HD dd dd_recip(dd a) {
    double q = 1.0 / a.hi;
    double r = fma(-q, a.hi, 1.0);  // exact residual of the rounded quotient
    r = r - q * a.lo;
    return fast_two_sum(q, q * r);
}

// x^(1/5) as a double-double for finite x in [2^-800, 2^800].
DD_HD dd fifth_root_dd(double x, double r0) {
    dd r2 = two_prod(r0, r0);
    dd r4 = dd_mul(r2, r2);
    dd r5 = dd_mul_d(r4, r0);
    double e = (r5.hi - x) + r5.lo;
    double c = e / (5.0 * r4.hi);
    return fast_two_sum(r0, -c);
}

// x^(-1/q) as a double-double for q in {5, 8} and finite x in [2^-800, 2^800], without division:
// an FP32 estimate (about 2^-21), two FP64 Newton steps on s^-q = x,
//     s <- s ((q+1) - x s^q) / q          (error ~ (q+1)/2 e^2, so 2^-21 -> 2^-40 -> FP64 rounding),
// then one Newton step whose residual 1 - x s^q is formed in double-double (error ~ 2^-100).
DD_HD dd inv_root_dd(double xs, int q) {
    int ex = 0;
    double m = frexp(xs, &ex);  // xs = m 2^ex, m in [0.5, 1)
    float t = -((float)ex + log2f((float)m)) / (float)q;
    float kf = floorf(t);
    double s = ldexp((double)exp2f(t - kf), (int)kf);
    const double qd = (double)q, q1 = (double)(q + 1), iq = q == 5 ? 0.2 : 0.125;
    for (int it = 0; it < 2; ++it) {
        double s2 = s * s;
        double s4 = s2 * s2;
        double sq = q == 5 ? s4 * s : s4 * s4;
        s = s * (q1 - xs * sq) * iq;
    }
    (void)qd;
    dd s2 = two_prod(s, s);
    dd s4 = dd_mul(s2, s2);
    dd sq = q == 5 ? dd_mul_d(s4, s) : dd_mul(s4, s4);
    dd xsq = dd_mul_d(sq, xs);
    double e = (1.0 - xsq.hi) - xsq.lo;  // 1 - xsq.hi is exact: xsq.hi is within 2^-50 of 1
    return fast_two_sum(s, s * e * iq);
}

// s^q as a double-double, q >= 2 (q - 1 products; relative error a few units of 2^-104).
DD_HD dd dd_pow_int(double s, int q) {
    dd p = two_prod(s, s);
    for (int i = 2; i < q; ++i) p = dd_mul_d(p, s);
    return p;
}

// x^(-1/q) as a double-double for q in {6, 7, 9} and finite x in [2^-800, 2^800]: the scheme of
// inv_root_dd with s^q formed by dd_pow_int.
DD_HD dd inv_root_dd_q(double xs, int q) {
    int ex = 0;
    double m = frexp(xs, &ex);
    float t = -((float)ex + log2f((float)m)) / (float)q;
    float kf = floorf(t);
    double s = ldexp((double)exp2f(t - kf), (int)kf);
    const double q1 = (double)(q + 1), iq = 1.0 / (double)q;
    for (int it = 0; it < 2; ++it) {
        double sq = s;
        for (int i = 1; i < q; ++i) sq = sq * s;
        s = s * (q1 - xs * sq) * iq;
    }
    dd xsq = dd_mul_d(dd_pow_int(s, q), xs);
    double e = (1.0 - xsq.hi) - xsq.lo;  // 1 - xsq.hi is exact: xsq.hi is within 2^-50 of 1
    return fast_two_sum(s, s * e * iq);
}

// pow(x, y) for y = ±1/q, q in {6, 7, 9} (the controller and initial-step exponents of Verner's
// pairs): x^(±1/q) in double-double, then the factor x^(±d/q) with d = q |y| - 1 (the relative
// difference between binary64 y and ±1/q, exact from TwoProduct), as exp(g) = 1 + g + g^2/2.
DD_HD double pow_root_q(double x, double y, int q) {
    if (x != x) return x;
    if (x < 0.0) return (x - x) / (x - x);  // NaN
    if (x == 0.0) return y < 0.0 ? 1.0 / 0.0 : 0.0;
    if (x == 1.0 / 0.0) return y < 0.0 ? 0.0 : x;
    // bring x into [2^-800, 2^800] by a multiple of q binades
    const int E = q * (800 / q);
    double xs = x, post = 1.0;
    if (x < 0x1p-800) {
        xs = ldexp(x, E);
        post = ldexp(1.0, -E / q);
    } else if (x > 0x1p+800) {
        xs = ldexp(x, -E);
        post = ldexp(1.0, E / q);
    }
    dd r = inv_root_dd_q(xs, q);
    if (y < 0.0)
        post = 1.0 / post;  // exact: power of two
    else
        r = dd_recip(r);
    const dd qy = two_prod((double)q, fabs(y));
    const double d = (qy.hi - 1.0) + qy.lo;
    double g = d / (double)q * log(x);
    if (y < 0.0) g = -g;
    g = g + 0.5 * g * g;
    const double tt = r.lo + r.hi * g;
    return (r.hi + tt) * post;
}

// pow(x, y) for the exponents of the crate's controller and initial-step heuristic:
// y = ±1/q for q in {5, 6, 7, 8, 9} (binary64 values; 0.2 and 0.125 for DOPRI5 / the order-5
// pairs and DOP853).  Other y fall back to the platform pow and are not guaranteed to be correctly
// rounded.
DD_HD double pow_ctrl(double x, double y) {
    const bool fifth = (y == 0.2 || y == -0.2);
    const bool eighth = (y == 0.125 || y == -0.125);
    if (!(fifth || eighth)) {
        const double ay = fabs(y);
        if (ay == 1.0 / 6.0) return pow_root_q(x, y, 6);
        if (ay == 1.0 / 7.0) return pow_root_q(x, y, 7);
        if (ay == 1.0 / 9.0) return pow_root_q(x, y, 9);
        return pow(x, y);
    }
    // IEEE special cases of pow for these y
    if (x != x) return x;
    if (x < 0.0) return (x - x) / (x - x);  // NaN
    if (x == 0.0) return y < 0.0 ? 1.0 / 0.0 : 0.0;
    if (x == 1.0 / 0.0) return y < 0.0 ? 0.0 : x;
    // bring x into [2^-800, 2^800]; the scale is a multiple of 5 and 8 binades
    double xs = x, post = 1.0;
    if (x < 0x1p-800) {
        xs = ldexp(x, 800);
        post = ldexp(1.0, fifth ? -160 : -100);
    } else if (x > 0x1p+800) {
        xs = ldexp(x, -800);
        post = ldexp(1.0, fifth ? 160 : 100);
    }
    dd r;
    if (y < 0.0) {
        // the controller's exponents: x^(-1/q) directly
        r = inv_root_dd(xs, fifth ? 5 : 8);
        post = 1.0 / post;  // exact: power of two
    } else if (fifth) {
        double r0 = pow(xs, 0.2);  // starting value, a few ulp from x^(1/5)
        r = fifth_root_dd(xs, r0);
    } else {
        r = dd_sqrt(dd_sqrt(dd_sqrt(dd{xs, 0.0})));
    }
    if (fifth) {
        // binary64 0.2 = (1/5)(1 + 2^-54): multiply by exp(+-2^-54 ln(x) / 5)
        double g = 1.1102230246251566e-17 /* 2^-54 / 5 */ * log(x);
        if (y < 0.0) g = -g;
        g = g + 0.5 * g * g;
        double t = r.lo + r.hi * g;
        return (r.hi + t) * post;
    }
    return (r.hi + r.lo) * post;
}

// Bit-pattern access for host and device builds.
DD_HD long long dd_bits(double x) {
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x);
#else
    long long b;
    memcpy(&b, &x, 8);
    return b;
#endif
}
DD_HD double dd_from_bits(long long b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}
DD_HD unsigned int dd_fbits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    unsigned int b;
    memcpy(&b, &x, 4);
    return b;
#endif
}
DD_HD float dd_ffrom(unsigned int b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x;
    memcpy(&x, &b, 4);
    return x;
#endif
}

// a * b rounded on its own: never contracted with a later addition into an FMA, in device code
// compiled with contraction as on the host.
DD_HD double dd_mul_nc(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}

// 128-bit fixed-point helpers for the controller power's residual (integer pipe only).
typedef unsigned long long dd_u64;
DD_HD dd_u64 dd_umulhi(dd_u64 a, dd_u64 b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (dd_u64)(((unsigned __int128)a * b) >> 64);
#endif
}
DD_HD int dd_clz64(dd_u64 a) {  // a != 0
#if defined(__CUDA_ARCH__)
    return __clzll((long long)a);
#else
    return __builtin_clzll(a);
#endif
}
// A positive number M 2^(E - 127) with the 128-bit mantissa M = (h, l) in [2^127, 2^128).
struct dd_fx {
    dd_u64 h, l;
    int e;
};
DD_HD dd_fx dd_fx_norm(dd_u64 h, dd_u64 l, int e) {
    if (!(h >> 63)) {
        h = (h << 1) | (l >> 63);
        l <<= 1;
        e -= 1;
    }
    return {h, l, e};
}
// a times the 64-bit mantissa m in [2^63, 2^64) (the number m 2^-63): the top 128 bits of the
// product, truncated (below 2^-126 relative)
DD_HD dd_fx dd_fx_mul64(dd_fx a, dd_u64 m) {
    dd_u64 h = dd_umulhi(a.h, m), l = a.h * m;
    const dd_u64 c = dd_umulhi(a.l, m);
    l += c;
    h += (l < c);
    return dd_fx_norm(h, l, a.e + 1);
}
// a squared: the top 128 bits, truncated (below 2^-125 relative)
DD_HD dd_fx dd_fx_sqr(dd_fx a) {
    dd_u64 h = dd_umulhi(a.h, a.h), l = a.h * a.h;
    const dd_u64 m = dd_umulhi(a.h, a.l);  // 2 a.h a.l / 2^64, less its low bit
    const dd_u64 t = m << 1;
    l += t;
    h += (m >> 63) + (l < t);
    return dd_fx_norm(h, l, 2 * a.e + 1);
}

// e = 1 - x s^q for q = 5 or 8, x and s normal and x s^q in [1/2, 2), on the integer pipe: the
// mantissas multiplied out in 128-bit fixed point (truncated products, relative error below
// 2^-120), e rounded toward zero to 53 bits.  ok = false when x s^q lies outside [1/2, 2).
DD_HD double pow_ctrl_residual(double x, double s, int q, bool& ok) {
    const long long b = dd_bits(x), sb = dd_bits(s);
    const int ex = (int)((b >> 52) & 0x7ff) - 1023, es = (int)((sb >> 52) & 0x7ff) - 1023;
    // x s^q = W 2^(ex + q es) with W = v u^q, u and v the mantissas of s and x in [1, 2)
    const dd_u64 U = ((dd_u64)sb << 11) | (1ull << 63), V = ((dd_u64)b << 11) | (1ull << 63);
    dd_fx w = dd_fx_norm(dd_umulhi(U, U), U * U, 1);  // u^2
    w = dd_fx_sqr(w);                                 // u^4
    w = q == 5 ? dd_fx_mul64(w, U) : dd_fx_sqr(w);    // u^5 or u^8
    w = dd_fx_mul64(w, V);
    const int T = w.e + ex + q * es;  // x s^q = M 2^(T - 127): 0 (x s^q in [1, 2)) or -1
    ok = T == 0 || T == -1;
    if (!ok) return 0.0;
    // D = |1 - x s^q| 2^(127 - T) as a 128-bit integer
    dd_u64 dh, dl;
    if (T == 0) {
        dh = w.h & 0x7fffffffffffffffull;
        dl = w.l;
    } else {
        dl = 0ull - w.l;
        dh = ~w.h + (w.l == 0);
    }
    if (!(dh | dl)) return 0.0;
    // leading bit p, the 53 bits from it (truncated) and e = +-D 2^(T - 127)
    const int p = dh ? 127 - dd_clz64(dh) : 63 - dd_clz64(dl);
    const int n = p - 52;
    dd_u64 mnt;
    if (n >= 64)
        mnt = dh >> (n - 64);
    else if (n > 0)
        mnt = (dl >> n) | (dh << (64 - n));
    else
        mnt = dl << (-n);
    const long long eb = ((long long)(p + T - 127 + 1023) << 52) | (long long)(mnt & 0xfffffffffffffull);
    return dd_from_bits(T == 0 ? (eb | (long long)0x8000000000000000ull) : eb);
}

// The controller's power x^(-0.2) (DOPRI5 and the order-5 pairs) and x^(-0.125) (DOP853),
// correctly rounded as pow_ctrl, for the contracted FP64 forms, with as few FP64 instructions as
// possible (FP64 runs at 1/64 of the FP32 rate on this GPU, integer and FP32 work issues in its
// shadow):
//  - Start: x = 2^e m with e = q k + r, 0 <= r < q, so x^(-1/q) = 2^-k (2^r m)^(-1/q).  The
//    second factor lies in (1/2, 1] and comes from FP32 log2/exp2 of 2^r m (relative error near
//    2^-22); the exponent -k is put into the bit pattern with integer operations.
//  - The residual e = 1 - x s^q (|e| < 2^-18) in 128-bit fixed point on the integer pipe: the
//    mantissas of s and x multiplied out with truncated 128-bit products (relative error below
//    2^-120), e converted to binary64 by truncation (absolute error below 2^-70).
//  - One correction instead of Newton steps: x^(-1/q) = s (1 - e)^(-1/q)
//    = s (1 + e/q + c2 e^2 + c3 e^3 + c4 e^4 + ...), the binomial series truncated after e^4 (the
//    rest is below 2^-88).
//  - For 1/5, the factor exp(-2^-54 ln(x) / 5) that turns 1/5 into binary64 0.2 takes ln(x) from
//    FP32 (off by less than 2^-69.5 relative).
//  - Ziv's test on the exact remainder of the final addition, in integer arithmetic: the total
//    error is below 2^-68.9 of the result, so the rounded sum is the correctly rounded value
//    unless it lies within 2^-68 of a rounding boundary; only then (about one call in 2^13) does
//    pow_ctrl evaluate it again in double-double arithmetic.
// x must be finite and in [2^-800, 2^800] after the caller's scaling; other x go to pow_ctrl.
DD_HD double pow_ctrl_neg(double x, double y) {
    const bool fifth = y == -0.2;
    if (!(fifth || y == -0.125) || !(x >= 0x1p-800 && x <= 0x1p+800)) return pow_ctrl(x, y);
    const int q = fifth ? 5 : 8;
    const long long b = dd_bits(x);
    const int ex = (int)((b >> 52) & 0x7ff) - 1023;
    const int k = (ex + 1000) / q - 1000 / q;  // floor(ex / q): ex + 1000 > 0
    const int r = ex - q * k;                  // in [0, q)
    const float lm = log2f(dd_ffrom(0x3f800000u | (unsigned int)((b >> 29) & 0x7fffff)));  // log2 m, m in [1, 2)
    const unsigned int fb = dd_fbits(exp2f(-((float)r + lm) * (fifth ? 0.2f : 0.125f)));   // in [1/2, 1]
    const int es = (int)((fb >> 23) & 0xff) - 127 - k;
    const long long sb = ((long long)(es + 1023) << 52) | ((long long)(fb & 0x7fffff) << 29);
    const double s = dd_from_bits(sb);
    bool ok;
    const double e = pow_ctrl_residual(x, s, q, ok);
    if (!ok) return pow_ctrl(x, y);
    double P;
    if (fifth)  // (1 - e)^(-1/5) - 1: 1/5, 6/50, 66/750, 1056/15000
        P = e * fma(e, fma(e, fma(e, 0.0704, 0.088), 0.12), 0.2);
    else        // (1 - e)^(-1/8) - 1: 1/8, 9/128, 51/1024, 1275/32768
        P = e * fma(e, fma(e, fma(e, 0.038909912109375, 0.0498046875), 0.0703125), 0.125);
    const double c = dd_mul_nc(s, P);
    const double hi = s + c;
    double lo = c - (hi - s);  // exact: |c| < 2^-17 |s|
    if (fifth) {
        // binary64 0.2 = (1/5)(1 + 2^-54): multiply by exp(-2^-54 ln(x) / 5) = 1 + g
        const float gf = ((float)ex + lm) * -7.6954796e-18f;  // -(2^-54 / 5) ln 2 log2(x)
        const unsigned int gb = dd_fbits(gf);
        const int ge = (int)((gb >> 23) & 0xff);
        const double g = ge == 0 ? 0.0
                                 : dd_from_bits(((long long)(gb >> 31) << 63) | ((long long)(ge + 896) << 52) |
                                                ((long long)(gb & 0x7fffff) << 29));
        lo = fma(hi, g, lo);
    }
    const double res = hi + lo;
    const double tail = (hi - res) + lo;  // exact: hi + lo - res
    // |tail| against half an ulp of res less the error bound 2^-68 res, compared as bit patterns
    // (both non-negative): half_ulp = 2^(re - 53) (2^(re - 54) just below a power of two, where
    // the spacing halves), bound = 2^(re - 67), biased exponents
    const long long rb = dd_bits(res), tb = dd_bits(tail);
    const int re = (int)((rb >> 52) & 0x7ff);
    const int hu = re - (((rb & 0xfffffffffffffll) == 0 && tb < 0) ? 54 : 53);
    const int kk = hu - (re - 67);  // 14 or 13: half_ulp - bound = 2^(hu - 1) (2 - 2^(1 - kk))
    const long long lim = ((long long)(hu - 1) << 52) | ((1ll << 52) - (1ll << (53 - kk)));
    if ((tb & 0x7fffffffffffffffll) < lim) return res;
    return pow_ctrl(x, y);
}

// sin(u), cos(u) as double-doubles for |u.hi| <= 1/128.
DD_HD void sincos_small(dd u, dd& s, dd& c) {
    dd z = dd_mul(u, u);
    double zh = z.hi;
    // sin u = u + u z (-1/6 + z (1/120 + z Q)),  Q = -1/5040 + z/9! - z^2/11! + z^3/13!
    double Q = -1.0 / 5040.0 + zh * (1.0 / 362880.0 + zh * (-1.0 / 39916800.0 + zh * (1.0 / 6227020800.0)));
    dd R = dd_add(dd{DD_INV120_HI, DD_INV120_LO}, dd_mul_d(z, Q));
    dd T = dd_add(dd{-DD_INV6_HI, -DD_INV6_LO}, dd_mul(z, R));
    dd V = dd_mul(z, T);
    s = dd_add(u, dd_mul(u, V));
    // cos u = 1 + z (-1/2 + z (1/24 + z P)),  P = -1/720 + z/8! - z^2/10! + z^3/12!
    double P = -1.0 / 720.0 + zh * (1.0 / 40320.0 + zh * (-1.0 / 3628800.0 + zh * (1.0 / 479001600.0)));
    dd R2 = dd_add(dd{DD_INV24_HI, DD_INV24_LO}, dd_mul_d(z, P));
    dd T2 = dd_add(dd{-0.5, 0.0}, dd_mul(z, R2));
    c = dd_add(dd{1.0, 0.0}, dd_mul(z, T2));
}

// Reduce x (|x| < 2^20) to r = x - k pi/2 as a double-double; returns k mod 4.
DD_HD int reduce_pio2(double x, dd& r) {
    double k = rint(x * DD_TWO_OVER_PI);
    double t1 = fma(-k, DD_PIO2_1, x);  // exact: k*PIO2_1 has <= 53 bits and t1 is small
    double kp2 = k * DD_PIO2_2;         // exact
    dd s = two_sum(t1, -kp2);
    dd p3 = two_prod(k, DD_PIO2_3);
    dd u = two_sum(s.hi, -p3.hi);
    double lo = s.lo + u.lo;
    lo = lo - p3.lo;
    lo = lo - k * DD_PIO2_4;
    r = fast_two_sum(u.hi, lo);
    long long ki = (long long)k;
    return (int)(ki & 3);
}

// sin or cos (want_cos) of x, correctly rounded in practice for |x| < 2^20.
DD_HD double sincos_cr(double x, bool want_cos) {
    if (x != x) return x;
    double ax = fabs(x);
    if (!(ax < 1048576.0)) return want_cos ? cos(x) : sin(x);  // outside the reduction's range
    dd r;
    int q = reduce_pio2(x, r);
    bool neg = r.hi < 0.0;
    dd a = neg ? dd_neg(r) : r;
    int j = (int)rint(a.hi * 64.0);
    if (j > DD_TAB_N - 1) j = DD_TAB_N - 1;
    dd u = {a.hi - (double)j * 0.015625, a.lo};  // exact difference
    u = fast_two_sum(u.hi, u.lo);
    dd su, cu;
    sincos_small(u, su, cu);
    const double* row = dd_tab_row(j);
    dd sj = {row[0], row[1]};
    dd cj = {row[2], row[3]};
    // sin(a) = sj cu + cj su ; cos(a) = cj cu - sj su
    dd sa = dd_add(dd_mul(sj, cu), dd_mul(cj, su));
    dd ca = dd_add(dd_mul(cj, cu), dd_neg(dd_mul(sj, su)));
    dd sr = neg ? dd_neg(sa) : sa;  // sin(r)
    dd cr = ca;                      // cos(r)
    dd res;
    if (!want_cos) {
        res = q == 0 ? sr : q == 1 ? cr : q == 2 ? dd_neg(sr) : dd_neg(cr);
    } else {
        res = q == 0 ? cr : q == 1 ? dd_neg(sr) : q == 2 ? dd_neg(cr) : sr;
    }
    return res.hi + res.lo;
}

DD_HD double sin_cr(double x) { return sincos_cr(x, false); }
DD_HD double cos_cr(double x) { return sincos_cr(x, true); }

}  // namespace ddm
}  // namespace degpu
