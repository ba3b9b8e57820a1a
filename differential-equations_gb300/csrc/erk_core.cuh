// erk_core.cuh — one instance of the crate's explicit Runge–Kutta solve, as a per-lane state
// machine in registers.
//
// Mirrors, operation for operation on the parity path:
//   driver loop ............ src/ode/solve_ivp.rs:138-277
//   DormandPrince init ..... src/methods/erk/dormandprince/ordinary.rs:16-61
//   DormandPrince step ..... src/methods/erk/dormandprince/ordinary.rs:63-268
//   DormandPrince interp ... src/methods/erk/dormandprince/ordinary.rs:301-336
//   Fixed (RK4) init/step .. src/methods/erk/fixed/ordinary.rs:16-138
//   Hermite interpolation .. src/interpolate.rs:40-60 (fixed/ordinary.rs:206-218)
//   h_init ................. src/methods/h_init.rs:45-136
//   validate / constrain ... src/utils.rs:22-157
//   error_norm ............. src/traits.rs:394-410
//   TEvalSolout ............ src/solout/t_eval.rs:82-137
//
// The state (y, the derivative k0, counters, controller state and, with dense output, the
// dense coefficients) stays in registers for the whole solve; the stage vectors k[1..I) live in
// registers for the duration of one step.  Nothing is allocated.
//
// Work the crate does whose results nothing reads is not repeated: without requested output
// times the three DOP853 dense-output stages (ordinary.rs:210-225) and the dense coefficients are
// skipped, and their three function evaluations are still counted in `fevals` so that the
// counters equal the crate's.
#pragma once

#if !defined(__CUDACC_RTC__)
#include <stdint.h>
#endif

#include "rhs.cuh"
#include "tableau.cuh"
#include "../../include/degpu.h"

namespace degpu {

struct EnsArgs {
    int64_t n;               // SoA stride (instances in the batch)
    int64_t count;           // work items (entries of `index`, or n)
    const int64_t* index;    // optional work-item -> instance map
    const double* t0;
    const double* tf;
    const double* y0;
    const double* params;
    const double* rtol;
    const double* atol;
    const double* rtol_vec;  // [dmax][n] per-component tolerances (Tolerance::Vector) or NULL
    const double* atol_vec;
    const double* t_eval;      // ascending, [n_eval]
    const int32_t* eval_perm;  // ascending position -> caller's index
    int32_t n_eval;
    int32_t dmax;
    double* y_final;
    double* t_final;
    double* dense;
    int64_t* accepted;
    int64_t* rejected;
    int64_t* fevals;
    int32_t* status;
    double h0, h_min, h_max;
    int64_t max_steps;
    double safety, min_scale, max_scale;
    float safety_f, min_scale_f, max_scale_f;  // FP32 copies (mixed form's controller)
    int32_t dense_mode;
    int32_t n_params;
    const int32_t* family;           // per-instance family id (multi-family persistent kernel)
    unsigned long long* ticket;      // persistent queue head
    const int32_t* dims;             // per-instance dimension (ragged systems, serving rounds)
    // crossing and event detection (erk_cross_kernel), by cross_mode:
    //  0 component crossing: y[cross_comp] - cross_value changes sign;
    //  1 hyperplane crossing: sum_j (y[term_comp[j]] - term_a[j]) term_w[j], j < n_terms, with
    //    term_w of unit length; cross_value = sum_j |term_a[j] term_w[j]| (the scale of the mixed
    //    form's FP32 search tolerance);
    //  2 event: g(t, y) = ((sum_j term_w[j] y[term_comp[j]]) + event_tw t) + cross_value (LINEAR)
    //    or max_j |y[term_comp[j]]| + cross_value (MAX_ABS); event_terminate events end the solve.
    int32_t cross_mode, cross_comp, cross_dir, cross_max;  // dir: 0 both, 1 from below, -1 from above
    double cross_value;
    double* cross_t;       // [cross_max][n]
    double* cross_y;       // [cross_max][dmax][n]
    int32_t* cross_count;  // [n]
    int32_t n_terms, event_kind, event_terminate;
    int32_t term_comp[DEGPU_HYPERPLANE_MAX_DIM];
    double term_a[DEGPU_HYPERPLANE_MAX_DIM];
    double term_w[DEGPU_HYPERPLANE_MAX_DIM];
    double event_tw;
    // FP32 copies for the mixed form (its per-step offsets are FP32 data)
    float cross_value_f, event_tw_f;
    float term_a_f[DEGPU_HYPERPLANE_MAX_DIM], term_w_f[DEGPU_HYPERPLANE_MAX_DIM];
};

// PickT<B, T, F>::type: T when B, else F (no standard library under run-time compilation).
template <bool B, class T, class F>
struct PickT {
    using type = T;
};
template <class T, class F>
struct PickT<false, T, F> {
    using type = F;
};

// f64::signum (Rust std): +-1 for signed zeros and infinities, NaN for NaN.
__device__ __forceinline__ double rs_signum(double x) { return x != x ? x : copysign(1.0, x); }
__device__ __forceinline__ float rs_signum(float x) { return x != x ? x : copysignf(1.0f, x); }

static_assert(DEGPU_EVENT_MAX_TERMS == DEGPU_HYPERPLANE_MAX_DIM, "event terms and plane components share arrays");

// Brent–Dekker root search as the crate runs it for events (src/solout/event.rs:395-490): at most
// 50 iterations of inverse quadratic interpolation or secant steps, taken when they stay well
// inside the bracket, else bisection; converged when half the bracket is within
// max(abs_tol, rel_tol |b|) or g vanishes. f(x, ok) evaluates g on the step's interpolant and
// clears ok when x lies outside the step (the crate's interpolator then fails and no root is
// returned). R is double, or float for the mixed form's search in the step's normalised
// coordinate.
template <class R, class F>
__device__ bool brent_dekker(R a, R b, R fa, R fb, R abs_tol, R rel_tol, F f, R& root) {
    if (fabs(fa) < fabs(fb)) {
        R x = a;
        a = b;
        b = x;
        x = fa;
        fa = fb;
        fb = x;
    }
    R c = a, fc = fa, d = b - a, e = d;
    const R one = 1, two = 2, half = one / two, three = 3;
    for (int it = 0; it < 50; ++it) {
        if (fb == (R)0) {
            root = b;
            return true;
        }
        if (rs_signum(fa) == rs_signum(fb)) {
            a = c;
            fa = fc;
            c = b;
            fc = fb;
            d = b - a;
            e = d;
        }
        if (fabs(fa) < fabs(fb)) {
            c = b;
            b = a;
            a = c;
            fc = fb;
            fb = fa;
            fa = fc;
        }
        const R tol = fmax(abs_tol, rel_tol * fabs(b));
        const R m = half * (a - b);
        if (fabs(m) <= tol || fb == (R)0) {
            root = b;
            return true;
        }
        bool use_bis = true;
        if (fabs(e) > tol && fabs(fa) > fabs(fb)) {
            const R s = fb / fa;
            R p, q;
            if (a == c) {
                p = two * m * s;
                q = one - s;
            } else {
                const R q1 = fa / fc;
                const R r = fb / fc;
                p = s * (two * m * q1 * (q1 - r) - (b - a) * (r - one));
                q = (q1 - one) * (r - one) * (s - one);
            }
            if (q > (R)0)
                p = -p;
            else
                q = -q;
            if (fabs(two * p) < (three * m * q - fabs(tol * q)) && p < fabs(e * half * q)) {
                e = d;
                d = p / q;
                use_bis = false;
            }
        }
        if (use_bis) {
            d = m;
            e = m;
        }
        a = b;
        fa = fb;
        if (fabs(d) > tol)
            b = b + d;
        else
            b = b + (m > (R)0 ? tol : -tol);
        bool ok = true;
        fb = f(b, ok);
        if (!ok) return false;
        c = a;
        fc = fa;
    }
    return false;
}

// Conversions between FP32 and FP64 done with integer operations on the bit patterns, for the
// mixed form's per-step bookkeeping: a hardware conversion involving FP64 occupies the FP64 pipe,
// which runs at 1/64 of the FP32 rate on this GPU.
// widen_f32: exact FP32 -> FP64 (subnormal inputs become signed zero; inf and NaN are kept).
__device__ __forceinline__ double widen_f32(float f) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int e = (b >> 23) & 0xffu;
    const unsigned int sign = b & 0x80000000u;
    if (e == 0u) return __hiloint2double((int)sign, 0);
    const unsigned int ee = e == 0xffu ? 0x7ffu : e + 896u;  // rebias 127 -> 1023
    const unsigned int hi = sign | (ee << 20) | ((b & 0x7fffffu) >> 3);
    const unsigned int lo = (b & 0x7u) << 29;
    return __hiloint2double((int)hi, (int)lo);
}
// narrow_rz: FP64 -> FP32 rounded toward zero (|result| <= |x|); magnitudes below the FP32
// normal range become signed zero, above it infinity; NaN stays NaN.
__device__ __forceinline__ float narrow_rz(double x) {
    const unsigned int hi = (unsigned int)__double2hiint(x);
    const unsigned int lo = (unsigned int)__double2loint(x);
    const unsigned int e = (hi >> 20) & 0x7ffu;
    const unsigned int sign = hi & 0x80000000u;
    if (e <= 896u) return __uint_as_float(sign);
    if (e == 0x7ffu && ((hi & 0xfffffu) | lo)) return __uint_as_float(0x7fc00000u);
    if (e >= 1151u) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// Comparisons, minima and maxima of non-negative doubles on their bit patterns, for the FP64
// paths' bookkeeping: an FP64 compare or min/max instruction occupies the FP64 pipe (1/64 of the
// FP32 rate on this GPU), a 64-bit integer one does not.  The order of doubles >= +0 (with +inf)
// is the order of their bit patterns, so each helper gives exactly the FP64 result, NaN included
// as noted.
__device__ __forceinline__ long long nn_bits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool nn_is_nan(long long b) { return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll; }
// a < b for a >= +0 or NaN and b >= +0 (false for a NaN, as the FP64 compare)
__device__ __forceinline__ bool nn_lt(double a, double b) { return nn_bits(a) < nn_bits(b); }
// a <= b for a >= +0 or NaN and b >= +0 (false for a NaN)
__device__ __forceinline__ bool nn_le(double a, double b) {
    const long long x = nn_bits(a);
    return !nn_is_nan(x) && x <= nn_bits(b);
}
// |a| < b for any a and b >= +0 (false for a NaN)
__device__ __forceinline__ bool abs_lt(double a, double b) { return (nn_bits(a) & 0x7fffffffffffffffll) < nn_bits(b); }
// fmax(|a|, |b|): the larger magnitude, the other operand when one is NaN
__device__ __forceinline__ double fmax_abs(double a, double b) {
    const long long x = nn_bits(a) & 0x7fffffffffffffffll, y = nn_bits(b) & 0x7fffffffffffffffll;
    if (nn_is_nan(x)) return __longlong_as_double(y);
    if (nn_is_nan(y)) return __longlong_as_double(x);
    return __longlong_as_double(x > y ? x : y);
}
// fmin(fmax(v, lo), hi) for v >= +0 or NaN and +0 <= lo <= hi (a NaN v gives lo, as fmax does)
__device__ __forceinline__ double nn_clamp(double v, double lo, double hi) {
    long long x = nn_bits(v);
    const long long l = nn_bits(lo), h = nn_bits(hi);
    if (nn_is_nan(x) || x < l) x = l;
    if (x > h) x = h;
    return __longlong_as_double(x);
}
// fmin(v, m) for v, m >= +0 (neither NaN)
__device__ __forceinline__ double nn_min(double v, double m) {
    const long long x = nn_bits(v), y = nn_bits(m);
    return __longlong_as_double(x < y ? x : y);
}

// The earliest stage (>= 1) of a tableau at the same node c as stage i, and the last stage at
// c = 1 (-1 if none): stages at one time share a time-dependent drive term.
template <class Tab>
__host__ __device__ constexpr int first_stage_at_c(int i) {
    for (int j = 1; j < i; ++j)
        if (Tab::c(j) == Tab::c(i)) return j;
    return i;
}
template <class Tab>
__host__ __device__ constexpr int last_stage_at_one() {
    for (int j = Tab::S - 1; j >= 1; --j)
        if (Tab::c(j) == 1.0) return j;
    return -1;
}

// CROSS: crossing detection instead of output times (needs DENSE for the step's interpolant).
template <class Tab, class Rhs, class P, bool DENSE, bool CROSS = false>
struct Lane {
    static_assert(!CROSS || DENSE, "crossing detection interpolates within the step");
    static constexpr int D = Rhs::D;
    static constexpr int I = Tab::I;
    static constexpr int NS = Tab::S;
    static constexpr int O = Tab::ORDER;
    // dense-output rows: the DP coefficients; Hermite: y_prev, dydt_prev; Verner: y_prev and the
    // step's I stages
    static constexpr int NC = DENSE ? (Tab::DP ? O : (Tab::HAS_BI ? 1 + I : 2)) : 1;
    // stage rows of an embedded step: the dense-output stages only when they are read
    static constexpr int KN = (DENSE && Tab::HAS_BI) ? I : NS;
    static constexpr int NPP = Rhs::NP > 0 ? Rhs::NP : 1;
    using S = typename P::S;
    using AccT = typename AccOf<S>::type;  // stage sums: S itself, or a lazily normalised pair
    static constexpr bool MIX = P::KAHAN && Tab::ADAPTIVE;
    static constexpr bool PHASE = MIX && PhaseOf<Rhs>::value;
    static constexpr bool PF = MIX && FloatParamsOf<Rhs>::value;  // FP32 parameter copies
    // Mixed form without output: t as an FP32 pair th + tl (about 48 bits), advanced and compared
    // with tf in FP32 arithmetic, so that an accepted step issues no FP64 instruction. A drive
    // phase is advanced as an FP32 pair too; a right-hand side that reads t gets th + tl widened
    // (tnow). The FP64-controller form (PrecMixedF64Ctrl) keeps t in FP64.
    static constexpr bool FFT = MIX && !DENSE && P::F32_CTRL;
    // Mixed form of a first-same-as-last tableau (DOPRI5): the last stage is evaluated at y_new
    // itself, and the evaluation the crate repeats at the new point on acceptance is that stage.
    static constexpr bool FSAL_MIX = MIX && Tab::FSAL;
    // FP64 forms of a family with a drive term: one drive evaluation per distinct stage time,
    // shared with the evaluation at the new point (t + h, the time of the c = 1 stage)
    static constexpr bool DRV = !P::KAHAN && DriveOf<Rhs>::value && Tab::DP;

    int64_t inst;
    double t, tf, h, h_prev, t_prev, dir, rtol, atol;
    float th, tl, tfh, tfl;  // FFT: t = th + tl, tf = tfh + tfl
    bool at_tf;              // FFT: the last step ended exactly at tf
    float phl, omh, oml;     // drive phase = ph0 + phl (FFT or pair stages), rate = omh + oml (FFT)
    double rem;    // tf - t (mixed form of RK4)
    float h_lim;   // 1e-14 |h_prev| in FP32 (mixed form's step-size guard)
    double h_lim64;  // 1e-14 |h_prev| (FP64 step-size guard), formed on acceptance
    // Mixed form of the adaptive methods (MIX): the step size, the remaining span used by the
    // overshoot test and the drive phase of time-dependent families are FP32; FP64 is touched
    // only on acceptance (t += h, tf - t, the phase at the new t).
    float hf;        // step size
    float remf;      // tf - t, refreshed on acceptance
    float ph0;       // families with a drive phase: the reduced phase at t
    float rtolf, atolf;  // FP32 copies of the tolerances (mixed form's FP32 error terms)
    bool fwd;        // tf > t0
    bool last_step;  // this attempt was clamped to end at tf
    bool bounded;  // h_min / h_max differ from the defaults 0 / +inf
    double p[NPP];
    typename P::PS pf[NPP];  // mixed form: FP32 (or FP32-pair) copies of p, made once per instance
    S y[D];
    S yc[D];  // Kahan compensation of y (mixed precision only)
    S k0[D];  // derivative at (t, y): k[0] of the next step
    S cont[NC][D];
    int64_t steps, acc, rej, fev;
    int stiff, nonstiff;
    int mod100;  // steps % 100, kept incrementally (the stiffness test runs every 100th attempt)
    int next_eval;
    int status;
    // crossing detection: previous offset (events: previous g); FP32 in the mixed form
    // FP32-stage lanes search in FP32; pair lanes, like FP64 ones, run the crate's FP64 search on
    // their (pair) interpolant
    static constexpr bool F32_SEARCH = P::KAHAN && !P::PAIR;
    using OffT = typename PickT<F32_SEARCH, float, double>::type;
    OffT last_off;
    bool have_last_off;
    int ncross;          // crossings / events recorded
    int nevents;         // events counted (recorded or within 1e-14 of the last point)
    double last_push;    // events: time of the last point of the crate's solution
    bool have_push;
    bool last_rejected;
    bool done;

    __device__ __forceinline__ void rhs(double tt, const S* yy, S* dd) const {
        if constexpr (PF)
            Rhs::template diff<P>(tt, yy, dd, pf);
        else
            Rhs::template diff<P>(tt, yy, dd, p);
    }
    // The current time: under FFT the FP32 pair (dead code for autonomous families), else t.
    __device__ __forceinline__ double tnow() const {
        if constexpr (FFT)
            return (double)th + (double)tl;
        else
            return t;
    }
    // Right-hand side at t + dt in the mixed form: a family with a drive phase adds Omega dt to
    // the phase at t in FP32; the others get the stage time t + dt (unused by autonomous ones).
    // DT: FP32, or for pair stages the stage's offset c_i h as a pair (so that a time-dependent
    // right-hand side sees the stage time to the pairs' accuracy, not to FP32 rounding).
    template <class DT>
    __device__ __forceinline__ void rhs_at(DT dt, const S* yy, S* dd) const {
        if constexpr (PHASE) {
            if constexpr (P::PAIR)
                Rhs::template diff_phase<P>(df(ph0, phl), dt, yy, dd, pf);  // the phase pair
            else
                Rhs::template diff_phase<P>(ph0, dt, yy, dd, pf);
        } else {
            rhs(tnow() + to_f64(dt), yy, dd);
        }
    }
    // c_i h of a stage: FP32 for the FP32 stages, a pair for the pair stages
    __device__ __forceinline__ auto stage_offset(double ci) const {
        if constexpr (P::PAIR)
            return df(ci) * hf;
        else
            return (float)ci * hf;
    }

    // The drive phase at tt outside FFT: reduced to [-pi, pi] in FP64; pair stages keep it as an
    // FP32 pair (ph0 + phl), the FP32 stages its leading part.
    __device__ __forceinline__ void set_phase(double tt) {
        if constexpr (P::PAIR) {
            const double ph = p[Rhs::PHASE_RATE] * tt;
            const double r = fma(-rint(ph * 0.15915494309189535), 6.283185307179586, ph);
            ph0 = (float)r;
            phl = (float)(r - (double)ph0);
        } else {
            ph0 = Rhs::phase(tt, p);
        }
    }
    // FFT: t += hf as an FP32 pair (TwoSum, then FastTwoSum), or t = tf after a clamped last step
    __device__ __forceinline__ void ff_advance() {
        if (last_step) {
            th = tfh;
            tl = tfl;
            at_tf = true;
            return;
        }
        const float s = th + hf;
        const float bp = s - th;
        const float e = (th - (s - bp)) + (hf - bp);
        const float lo = tl + e;
        const float hi = s + lo;
        tl = lo - (hi - s);
        th = hi;
    }
    // FFT with a drive phase: phase += Omega hf as an FP32 pair (the product's error from fmaf and
    // the rate's low part), reduced by 2 pi (an FP32 pair) to [-pi, pi]
    __device__ __forceinline__ void ff_phase_advance() {
        const float pr = omh * hf;
        const float pe = fmaf(omh, hf, -pr) + oml * hf;
        float s = ph0 + pr;
        float bp = s - ph0;
        float e = (ph0 - (s - bp)) + (pr - bp);
        float lo = (phl + e) + pe;
        float hi = s + lo;
        phl = lo - (hi - s);
        ph0 = hi;
        if (fabsf(ph0) > 3.14159265f) {
            const float k = rintf(ph0 * 0.159154943f);
            const float q = k * 6.28318548f;                   // 2 pi = 6.28318548f - 1.74845553e-7f
            const float qe = fmaf(k, 6.28318548f, -q) + k * -1.74845553e-7f;
            s = ph0 - q;
            bp = s - ph0;
            e = (ph0 - (s - bp)) + (-q - bp);
            lo = (phl + e) - qe;
            hi = s + lo;
            phl = lo - (hi - s);
            ph0 = hi;
        }
    }
    // FFT: tf - t in FP32 (exact in its leading part when t is near tf)
    __device__ __forceinline__ float ff_rem() const { return (tfh - th) + (tfl - tl); }

    // Type of the per-component error terms and their sum: FP64, except in the mixed form built
    // with the FP32 controller (P::F32_CTRL), whose terms are FP32 stage data.
    using NormT = typename Select<P::F32_CTRL, float, double>::type;

    // Tolerances of component c (src/tolerance.rs:33-40): the batch's per-component value when it
    // has one (Tolerance::Vector), else the instance's scalar; FP32 copies for the mixed form.
    // The element offset of component c of this instance, formed where it is used: the empty asm
    // keeps the compiler from hoisting the D offsets out of the solve loop into registers, which
    // every solve would pay for, per-component tolerances or not.
    __device__ __forceinline__ int64_t comp_offset(int c, const EnsArgs& a) const {
        int64_t off = (int64_t)c * a.n + inst;
        asm volatile("" : "+l"(off));
        return off;
    }
    __device__ __forceinline__ double rtol_c(int c, const EnsArgs& a) const {
        return a.rtol_vec ? a.rtol_vec[comp_offset(c, a)] : rtol;
    }
    __device__ __forceinline__ double atol_c(int c, const EnsArgs& a) const {
        return a.atol_vec ? a.atol_vec[comp_offset(c, a)] : atol;
    }
    __device__ __forceinline__ float rtolf_c(int c, const EnsArgs& a) const {
        return a.rtol_vec ? (float)a.rtol_vec[comp_offset(c, a)] : rtolf;
    }
    __device__ __forceinline__ float atolf_c(int c, const EnsArgs& a) const {
        return a.atol_vec ? (float)a.atol_vec[comp_offset(c, a)] : atolf;
    }

    // TV: the batch has per-component tolerances (a uniform branch: the scalar path keeps its
    // registers)
    template <bool TV>
    __device__ __forceinline__ NormT norm_term(int c, S e, S yv, S ynv, const EnsArgs& a) const {
        // sk = atol + rtol * max(|y|, |y_new|); e/sk squared (traits.rs:402-407)
        if constexpr (P::F32_CTRL) {
            const float at = TV ? atolf_c(c, a) : atolf, rt = TV ? rtolf_c(c, a) : rtolf;
            float sk = at + rt * fmaxf(fabsf(lead(yv)), fabsf(lead(ynv)));
            float q = __fdividef(lead(e), sk);
            return q * q;
        } else {
            const double at = TV ? atol_c(c, a) : atol, rt = TV ? rtol_c(c, a) : rtol;
            double sk = at + rt * fmax_abs((double)yv, (double)ynv);
            double q = P::quot((double)e, sk);
            return q * q;
        }
    }

    // ----- h_init: src/methods/h_init.rs:45-136 --------------------------------------------
    __device__ double initial_step(double t0, const EnsArgs& a) {
        if constexpr (MIX) {
            return initial_step_f32(t0, a);
        } else {
        double posneg = rs_signum(tf - t0);
        S f0[D], f1[D], y1[D];
        rhs(t0, y, f0);
        fev += 1;
        double dnf = 0.0, dny = 0.0;
        double sk[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            sk[c] = atol_c(c, a) + rtol_c(c, a) * fabs((double)y[c]);
            double q = (double)f0[c] / sk[c];
            dnf = dnf + q * q;
            double r = (double)y[c] / sk[c];
            dny = dny + r * r;
        }
        double hh;
        if (dnf <= 1.0e-10 || dny <= 1.0e-10)
            hh = 1.0e-6;
        else
            hh = sqrt(dny / dnf) * 0.01;
        hh = fmin(hh, a.h_max);
        hh = hh * posneg;
        S hs = P::from(hh);
#pragma unroll
        for (int c = 0; c < D; ++c) y1[c] = y[c] + hs * f0[c];
        rhs(t0 + hh, y1, f1);
        fev += 1;
        double der2 = 0.0;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            double q = ((double)f1[c] - (double)f0[c]) / sk[c];
            if constexpr (P::KAHAN) q = (double)(f1[c] - f0[c]) / sk[c];
            der2 = der2 + q * q;
        }
        der2 = sqrt(der2) / fabs(hh);
        double der12 = fmax(sqrt(dnf), der2);
        double h1;
        if (der12 <= 1.0e-15)
            h1 = fabs(hh) * fmax(1.0e-3, 1.0e-6);
        else
            h1 = P::pow(0.01 / der12, 1.0 / (double)O);
        double interval = fabs(tf - t0);
        hh = fmin(fmax(fmin(fmin(fabs(hh) * 100.0, h1), a.h_max), a.h_min), interval);
        return hh * posneg;
        }
    }

    // The same heuristic in FP32 for the mixed form (the stage data are FP32; an FP64 version
    // would put dozens of FP64 divisions and square roots on every refill of a lane).
    __device__ double initial_step_f32(double t0, const EnsArgs& a) {
        const double posneg = rs_signum(tf - t0);
        const float pn = (float)posneg;
        S f0[D], f1[D], y1[D];
        rhs_at(0.0f, y, f0);
        fev += 1;
        float dnf = 0.0f, dny = 0.0f;
        float sk[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            sk[c] = atolf_c(c, a) + rtolf_c(c, a) * fabsf(lead(y[c]));
            float q = lead(f0[c]) / sk[c];
            dnf = dnf + q * q;
            float r = lead(y[c]) / sk[c];
            dny = dny + r * r;
        }
        float hh;
        if (dnf <= 1.0e-10f || dny <= 1.0e-10f)
            hh = 1.0e-6f;
        else
            hh = sqrtf(dny / dnf) * 0.01f;
        const float hmax = (float)a.h_max;
        hh = fminf(hh, hmax);
        hh = hh * pn;
#pragma unroll
        for (int c = 0; c < D; ++c) y1[c] = y[c] + hh * f0[c];
        rhs_at(hh, y1, f1);
        fev += 1;
        float der2 = 0.0f;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            float q = lead(f1[c] - f0[c]) / sk[c];
            der2 = der2 + q * q;
        }
        der2 = sqrtf(der2) / fabsf(hh);
        float der12 = fmaxf(sqrtf(dnf), der2);
        float h1;
        if (der12 <= 1.0e-15f)
            h1 = fabsf(hh) * 1.0e-3f;
        else
            h1 = powf(0.01f / der12, 1.0f / (float)O);
        const float interval = (float)fabs(tf - t0);
        hh = fminf(fmaxf(fminf(fminf(fabsf(hh) * 100.0f, h1), hmax), (float)a.h_min), interval);
        // FP32 rounding must not carry the step outside [h_min, |tf - t0|] of the FP64 checks
        double h = (double)hh;
        h = fmin(fmax(h, a.h_min), fabs(tf - t0));
        return h * posneg;
    }

    // ----- validate_step_size_parameters: src/utils.rs:60-157 ------------------------------
    __device__ __forceinline__ bool valid_h0(double h0, double t0, const EnsArgs& a) const {
        if (tf == t0) return false;
        double sign = rs_signum(tf - t0);
        if (rs_signum(h0) != sign) return false;
        if (a.h_min < 0.0 || a.h_max < 0.0 || a.h_min > a.h_max) return false;
        if (fabs(h0) < a.h_min || fabs(h0) > a.h_max) return false;
        if (fabs(h0) > fabs(tf - t0)) return false;
        if (h0 == 0.0) return false;
        return true;
    }

    // ----- dense output at the requested times: src/solout/t_eval.rs:82-137 ------------------
    __device__ __forceinline__ double eval_time(int idx, const EnsArgs& a) const {
        return dir > 0.0 ? a.t_eval[idx] : a.t_eval[a.n_eval - 1 - idx];
    }
    __device__ __forceinline__ int eval_slot(int idx, const EnsArgs& a) const {
        return dir > 0.0 ? a.eval_perm[idx] : a.eval_perm[a.n_eval - 1 - idx];
    }
    __device__ void write_dense(int idx, const S* v, const EnsArgs& a) const {
        int slot = eval_slot(idx, a);
        double* out = a.dense + ((int64_t)slot * a.dmax) * a.n + inst;
#pragma unroll
        for (int c = 0; c < D; ++c) out[(int64_t)c * a.n] = to_f64(v[c]);
    }
    __device__ void interpolate(double te, S* out, const EnsArgs& a) const {
        if constexpr (DENSE) {
            if constexpr (Tab::DP) {
                // ordinary.rs:312-333
                double s = (te - t_prev) / h_prev;
                double s1 = 1.0 - s;
                S ss = P::from(s), ss1 = P::from(s1);
                const bool hairer = a.dense_mode == DEGPU_DENSE_HAIRER;
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    S accv = cont[O - 1][c];
#pragma unroll
                    for (int i = O - 2; i >= 1; --i) {
                        S f;
                        if (i >= 4) {
                            bool odd = ((O - 1 - i) % 2) == 1;
                            if (hairer) odd = !odd;
                            f = odd ? ss1 : ss;
                        } else {
                            f = (i % 2 == 1) ? ss1 : ss;
                        }
                        accv = accv * f;
                        accv = accv + cont[i][c];
                    }
                    out[c] = cont[0][c] + ss * accv;
                }
            } else if constexpr (Tab::HAS_BI) {
                // adaptive/ordinary.rs:251-275: per stage the polynomial sum_j BI[i][j] s^(j+1) by
                // Horner's rule, then y_prev + sum_i (cont_i h_prev) k_i in stage order
                const double hp = P::KAHAN ? t - t_prev : h_prev;
                const S ss = P::from((te - t_prev) / hp), hs = P::from(hp);
#pragma unroll
                for (int c = 0; c < D; ++c) out[c] = cont[0][c];
                static_for<0, I>([&](auto i) {
                    constexpr int ii = decltype(i)::value;
                    S ci = (S)Tab::bi(ii, O - 1);
                    static_for<0, O - 1>([&](auto jr) {
                        constexpr int j = O - 2 - decltype(jr)::value;
                        ci = ci * ss + (S)Tab::bi(ii, j);
                    });
                    ci = ci * ss;
                    const S w = ci * hs;
#pragma unroll
                    for (int c = 0; c < D; ++c) out[c] = out[c] + w * cont[1 + ii][c];
                });
            } else {
                // cubic Hermite over [t_prev, t] with y_prev=cont[0], dydt_prev=cont[1], y, k0
                double t0 = t_prev, t1 = t;
                double hh = t1 - t0;
                double s = (te - t0) / hh;
                double s2 = s * s;
                double s3 = s2 * s;
                double h00 = 2.0 * s3 - 3.0 * s2 + 1.0;
                double h10 = s3 - 2.0 * s2 + s;
                double h01 = -2.0 * s3 + 3.0 * s2;
                double h11 = s3 - s2;
                S c00 = P::from(h00), c10 = P::from(h10 * hh), c01 = P::from(h01), c11 = P::from(h11 * hh);
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    S o = (S)0;
                    o = o + c00 * cont[0][c];
                    o = o + c10 * cont[1][c];
                    o = o + c01 * y[c];
                    o = o + c11 * k0[c];
                    out[c] = o;
                }
            }
        }
    }
    // The interpolant at the normalised position sg in the step ([0, 1] from t_prev to t), in the
    // stage arithmetic S: the mixed form's crossing search runs in this coordinate in FP32.
    __device__ void interpolate_sigma(S ss, S* out, const EnsArgs& a) const {
        if constexpr (DENSE) {
            if constexpr (Tab::DP) {
                const S ss1 = (S)1 - ss;
                const bool hairer = a.dense_mode == DEGPU_DENSE_HAIRER;
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    S accv = cont[O - 1][c];
#pragma unroll
                    for (int i = O - 2; i >= 1; --i) {
                        S f;
                        if (i >= 4) {
                            bool odd = ((O - 1 - i) % 2) == 1;
                            if (hairer) odd = !odd;
                            f = odd ? ss1 : ss;
                        } else {
                            f = (i % 2 == 1) ? ss1 : ss;
                        }
                        accv = accv * f;
                        accv = accv + cont[i][c];
                    }
                    out[c] = cont[0][c] + ss * accv;
                }
            } else if constexpr (Tab::HAS_BI) {
                const S hs = P::from(t - t_prev);
#pragma unroll
                for (int c = 0; c < D; ++c) out[c] = cont[0][c];
                static_for<0, I>([&](auto i) {
                    constexpr int ii = decltype(i)::value;
                    S ci = (S)Tab::bi(ii, O - 1);
                    static_for<0, O - 1>([&](auto jr) {
                        constexpr int j = O - 2 - decltype(jr)::value;
                        ci = ci * ss + (S)Tab::bi(ii, j);
                    });
                    const S w = (ci * ss) * hs;
#pragma unroll
                    for (int c = 0; c < D; ++c) out[c] = out[c] + w * cont[1 + ii][c];
                });
            } else {
                const S hh = P::from(t - t_prev);
                const S s2 = ss * ss, s3 = s2 * ss;
                const S c00 = (S)2 * s3 - (S)3 * s2 + (S)1, c10 = (s3 - (S)2 * s2 + ss) * hh;
                const S c01 = (S)-2 * s3 + (S)3 * s2, c11 = (s3 - s2) * hh;
#pragma unroll
                for (int c = 0; c < D; ++c)
                    out[c] = c00 * cont[0][c] + c10 * cont[1][c] + c01 * y[c] + c11 * k0[c];
            }
        }
    }

    // ----- crossing detection: CrossingSolout (src/solout/crossing.rs:200-330) and
    // HyperplaneCrossingSolout (src/solout/hyperplane.rs) ------------------------------------
    __device__ __forceinline__ S comp_s(const S* v, int comp) const {
        S r = v[0];
#pragma unroll
        for (int c = 1; c < D; ++c)
            if (c == comp) r = v[c];
        return r;
    }
    __device__ __forceinline__ double comp_value(const S* v, int comp) const { return to_f64(comp_s(v, comp)); }
    // The monitored offset of a state given component by component: y[comp] - threshold
    // (crossing.rs:207), or the hyperplane's signed distance (pos - point) . normal
    // (hyperplane.rs signed_distance), the dot product folded from zero in component order
    // (src/traits.rs:551-555).
    template <class Get>
    __device__ __forceinline__ double offset_by(Get get, const EnsArgs& a) const {
        if (a.cross_mode == 0) return get(a.cross_comp) - a.cross_value;
        double sum = 0.0;
#pragma unroll
        for (int j = 0; j < DEGPU_HYPERPLANE_MAX_DIM; ++j)
            if (j < a.n_terms) {
                const double d = get(a.term_comp[j]) - a.term_a[j];
                sum = sum + d * a.term_w[j];
            }
        return sum;
    }
    __device__ __forceinline__ double interp_offset(double te, const EnsArgs& a) const {
        S v[D];
        interpolate(te, v, a);
        return offset_by([&](int c) { return comp_value(v, c); }, a);
    }
    // find_crossing_newton (crossing.rs:254-328, hyperplane.rs find_crossing_newton): Newton on
    // the interpolant with a finite-difference derivative; false when it does not converge. The
    // hyperplane form stops on a derivative below eps (not 10 eps) and has no step-change test.
    __device__ bool find_crossing_newton(double t_lower, double t_upper, double off_lower, double off_upper,
                                         double& t_out, const EnsArgs& a) const {
        const double eps = 2.220446049250313e-16;
        const bool plane = a.cross_mode == 1;
        double tt = t_lower - off_lower * (t_upper - t_lower) / (off_upper - off_lower);
        const double tolerance = eps * 100.0;
        double offset;
        for (int it = 0; it < 10; ++it) {
            offset = interp_offset(tt, a);
            if (fabs(offset) < tolerance) {
                t_out = tt;
                return true;
            }
            const double delta_t = (t_upper - t_lower) * 1e-6;
            const double t_plus = tt + delta_t;
            const double offset_plus = interp_offset(t_plus, a);
            const double derivative = (offset_plus - offset) / delta_t;
            if (fabs(derivative) < (plane ? eps : eps * 10.0)) break;
            const double t_new = tt - offset / derivative;
            if (t_new < t_lower || t_new > t_upper) {
                tt = (t_lower + t_upper) / 2.0;
            } else {
                const double change = fabs(t_new - tt);
                if (!plane && change < tolerance * 0.1) {
                    tt = t_new;
                    break;
                }
                tt = t_new;
            }
        }
        offset = interp_offset(tt, a);
        if (fabs(offset) < tolerance * 10.0) {
            t_out = tt;
            return true;
        }
        return false;
    }
    // Mixed form: find_crossing_newton's iteration on sg in [0, 1] in FP32, with tolerances scaled
    // to FP32 (100 units of FP32 rounding of the monitored quantity's scale: |threshold|, or
    // sum |point_j normal_j| for a hyperplane); the linear estimate when it does not converge.
    __device__ float find_crossing_sigma(float off_l, float off_u, const EnsArgs& a) const {
        const bool plane = a.cross_mode == 1;
        const float thr = a.cross_value_f;
        const float tol = 100.0f * 1.1920929e-7f * fmaxf(1.0f, fabsf(thr));
        const float lin = -off_l / (off_u - off_l);
        auto off_at = [&](float sg) {
            S v[D];
            interpolate_sigma(sg, v, a);
            if (!plane) return (float)comp_s(v, a.cross_comp) - thr;
            float sum = 0.0f;
#pragma unroll
            for (int j = 0; j < DEGPU_HYPERPLANE_MAX_DIM; ++j)
                if (j < a.n_terms) sum += ((float)comp_s(v, a.term_comp[j]) - a.term_a_f[j]) * a.term_w_f[j];
            return sum;
        };
        float sg = lin, offset;
        for (int it = 0; it < 10; ++it) {
            offset = off_at(sg);
            if (fabsf(offset) < tol) return sg;
            const float ds = 1e-6f;
            const float derivative = (off_at(sg + ds) - offset) / ds;
            if (fabsf(derivative) < (plane ? 1.0f : 10.0f) * 1.1920929e-7f) break;
            const float s_new = sg - offset / derivative;
            if (s_new < 0.0f || s_new > 1.0f) {
                sg = 0.5f;
            } else {
                const float change = fabsf(s_new - sg);
                sg = s_new;
                if (!plane && change < tol * 0.1f) break;
            }
        }
        offset = off_at(sg);
        return fabsf(offset) < tol * 10.0f ? sg : lin;
    }

    // The mixed form's offset at the step's end in FP32: (y - compensation) against the FP32 copies
    // of the threshold or plane.
    __device__ __forceinline__ float state_offset_f32(const EnsArgs& a) const {
        if (a.cross_mode == 0) return lead((comp_s(y, a.cross_comp) - a.cross_value_f) - comp_s(yc, a.cross_comp));
        float sum = 0.0f;
#pragma unroll
        for (int j = 0; j < DEGPU_HYPERPLANE_MAX_DIM; ++j)
            if (j < a.n_terms) {
                const int c = a.term_comp[j];
                sum += lead((comp_s(y, c) - a.term_a_f[j]) - comp_s(yc, c)) * a.term_w_f[j];
            }
        return sum;
    }

    __device__ void crossing_solout(const EnsArgs& a) {
        OffT offset;
        if constexpr (F32_SEARCH)
            offset = state_offset_f32(a);
        else
            offset = offset_by([&](int c) { return comp_value(y, c); }, a);
        const OffT zero = (OffT)0;
        if (have_last_off) {
            bool is_crossing = rs_signum(last_off) != rs_signum(offset);
            // hyperplane.rs: leaving or reaching the plane exactly also counts
            if (a.cross_mode == 1)
                is_crossing = is_crossing || (last_off == zero && offset != zero) || (last_off != zero && offset == zero);
            if (is_crossing) {
                bool record;
                if (a.cross_dir > 0)
                    record = last_off < zero && offset >= zero;
                else if (a.cross_dir < 0)
                    record = last_off > zero && offset <= zero;
                else
                    record = true;
                if (record) {
                    double tc;
                    S v[D];
                    if constexpr (F32_SEARCH) {
                        // mixed: the same search in the step's normalised coordinate, in FP32
                        const float sg = find_crossing_sigma(last_off, offset, a);
                        tc = t_prev + (double)sg * (t - t_prev);
                        if (ncross < a.cross_max) interpolate_sigma(sg, v, a);
                    } else {
                        if (!find_crossing_newton(t_prev, t, last_off, offset, tc, a)) {
                            const double frac = -last_off / (offset - last_off);
                            tc = t_prev + frac * (t - t_prev);
                        }
                        if (ncross < a.cross_max) interpolate(tc, v, a);
                    }
                    if (ncross < a.cross_max) {
                        const int64_t n = a.n;
                        a.cross_t[(int64_t)ncross * n + inst] = tc;
                        double* out = a.cross_y + ((int64_t)ncross * a.dmax) * n + inst;
#pragma unroll
                        for (int c = 0; c < D; ++c) out[(int64_t)c * n] = to_f64(v[c]);
                    }
                    ncross += 1;
                }
            }
        }
        last_off = offset;
        have_last_off = true;
    }

    // ----- event detection: EventWrappedSolout, src/solout/event.rs:299-521 -----------------------
    // g(te, y) for the state given component by component (LINEAR folds from zero in term order;
    // MAX_ABS folds f64::max from the first term)
    template <class Get>
    __device__ __forceinline__ double event_by(double te, Get get, const EnsArgs& a) const {
        if (a.event_kind == DEGPU_EVENT_MAX_ABS) {
            double m = fabs(get(a.term_comp[0]));
#pragma unroll
            for (int j = 1; j < DEGPU_EVENT_MAX_TERMS; ++j)
                if (j < a.n_terms) m = fmax(m, fabs(get(a.term_comp[j])));
            return m + a.cross_value;
        }
        double sum = 0.0;
#pragma unroll
        for (int j = 0; j < DEGPU_EVENT_MAX_TERMS; ++j)
            if (j < a.n_terms) {
                const double term = a.term_w[j] * get(a.term_comp[j]);
                sum = sum + term;
            }
        const double tt = a.event_tw * te;
        sum = sum + tt;
        return sum + a.cross_value;
    }
    // The mixed form's FP32 event function: the time term as base + w_t (t - t_prev), base =
    // w_t t_prev + offset taken once per step in FP64, so that FP32 carries only the in-step part.
    __device__ __forceinline__ float event_f32(const S* v, float base, float dt_term, const EnsArgs& a) const {
        if (a.event_kind == DEGPU_EVENT_MAX_ABS) {
            float m = fabsf((float)comp_s(v, a.term_comp[0]));
#pragma unroll
            for (int j = 1; j < DEGPU_EVENT_MAX_TERMS; ++j)
                if (j < a.n_terms) m = fmaxf(m, fabsf((float)comp_s(v, a.term_comp[j])));
            return m + a.cross_value_f;
        }
        float sum = 0.0f;
#pragma unroll
        for (int j = 0; j < DEGPU_EVENT_MAX_TERMS; ++j)
            if (j < a.n_terms) sum += a.term_w_f[j] * (float)comp_s(v, a.term_comp[j]);
        return sum + dt_term + base;
    }
    __device__ void event_solout(const EnsArgs& a) {
        OffT g_curr;
        if constexpr (F32_SEARCH) {
            // mixed: g at the step's end in FP32 on y - compensation; the time term in FP64 once
            S sv[D];
#pragma unroll
            for (int c = 0; c < D; ++c) sv[c] = y[c] - yc[c];
            const float base = a.event_tw != 0.0 ? (float)(a.event_tw * t + a.cross_value) : a.cross_value_f;
            g_curr = event_f32(sv, base, 0.0f, a);
        } else {
            g_curr = event_by(t, [&](int c) { return comp_value(y, c); }, a);
        }
        if (!have_last_off) {  // the first call (at t0) only records g
            have_last_off = true;
            last_off = g_curr;
            return;
        }
        const OffT g_prev = last_off, zero = (OffT)0;
        const bool sign_change = rs_signum(g_prev) != rs_signum(g_curr);
        bool direction_ok;
        if (a.cross_dir > 0)
            direction_ok = sign_change && g_prev < zero && g_curr >= zero;
        else if (a.cross_dir < 0)
            direction_ok = sign_change && g_prev > zero && g_curr <= zero;
        else
            direction_ok = sign_change;
        if (direction_ok) {
            double lo = t_prev, hi = t;
            OffT flo = g_prev, fhi = g_curr;
            if ((dir > 0.0 && lo > hi) || (dir < 0.0 && lo < hi)) {
                const double x = lo;
                lo = hi;
                hi = x;
                const OffT f = flo;
                flo = fhi;
                fhi = f;
            }
            double te;
            bool found;
            if constexpr (F32_SEARCH) {
                // mixed: the same search on sg in [0, 1] (t_prev to t) in FP32 on the FP32
                // interpolant, stopping at 1e-6 of the step; a backward step locates nothing, as
                // the crate's interpolator refuses every time inside it
                float sg = 0.0f;
                found = false;
                if (dir > 0.0 && flo * fhi <= 0.0f) {
                    const float hspan = (float)(t - t_prev);
                    const float base =
                        a.event_tw != 0.0 ? (float)(a.event_tw * t_prev + a.cross_value) : a.cross_value_f;
                    const float twf = a.event_tw_f;
                    found = brent_dekker(0.0f, 1.0f, flo, fhi, 1e-6f, 0.0f,
                                         [&](float x, bool& ok) {
                                             if (x < 0.0f || x > 1.0f) {
                                                 ok = false;
                                                 return 0.0f;
                                             }
                                             S v[D];
                                             interpolate_sigma(x, v, a);
                                             return event_f32(v, base, twf * (x * hspan), a);
                                         },
                                         sg);
                }
                te = t_prev + (double)sg * (t - t_prev);
            } else {
                // the crate's tolerances (event.rs:329-330)
                found = flo * fhi <= 0.0 &&
                        brent_dekker(lo, hi, flo, fhi, 1e-14, 1e-12,
                                     [&](double x, bool& ok) {
                                         if (x < t_prev || x > t) {  // Error::OutOfBounds
                                             ok = false;
                                             return 0.0;
                                         }
                                         S v[D];
                                         interpolate(x, v, a);
                                         return event_by(x, [&](int c) { return comp_value(v, c); }, a);
                                     },
                                     te);
            }
            if (found) {
                if (!have_push || fabs(te - last_push) > 1e-14) {
                    if (ncross < a.cross_max) {
                        S v[D];
                        interpolate(te, v, a);
                        const int64_t n = a.n;
                        a.cross_t[(int64_t)ncross * n + inst] = te;
                        double* out = a.cross_y + ((int64_t)ncross * a.dmax) * n + inst;
#pragma unroll
                        for (int c = 0; c < D; ++c) out[(int64_t)c * n] = to_f64(v[c]);
                    }
                    ncross += 1;
                    have_push = true;
                    last_push = te;
                }
                nevents += 1;
                if (a.event_terminate > 0 && nevents >= a.event_terminate) status = DEGPU_INTERRUPTED;
            }
        }
        last_off = g_curr;
    }

    // TEvalSolout (src/solout/t_eval.rs:82-137) at the requested times within the step
    __device__ void teval_solout(const EnsArgs& a) {
        if constexpr (DENSE) {
            int idx = next_eval;
            while (idx < a.n_eval) {
                double te = eval_time(idx, a);
                bool in_range = dir > 0.0 ? ((te == t_prev && idx == 0) || (te > t_prev && te <= t))
                                          : ((te == t_prev && idx == 0) || (te < t_prev && te >= t));
                if (in_range) {
                    if (te == t) {
                        write_dense(idx, y, a);
                    } else {
                        S v[D];
                        interpolate(te, v, a);
                        write_dense(idx, v, a);
                    }
                    if constexpr (CROSS) {
                        have_push = true;
                        last_push = te;
                    }
                    idx += 1;
                } else {
                    if ((dir > 0.0 && te > t) || (dir < 0.0 && te < t)) break;
                    idx += 1;
                }
            }
            next_eval = idx;
        }
    }

    __device__ void solout(const EnsArgs& a) {
        if constexpr (CROSS) {
            if (a.cross_mode != 2) {
                crossing_solout(a);
                return;
            }
            // EventWrappedSolout: the base output first (the output times, else DefaultSolout,
            // which pushes every step's end), then the event
            if (a.n_eval > 0) {
                teval_solout(a);
            } else {
                have_push = true;
                last_push = t;
            }
            event_solout(a);
            return;
        }
        teval_solout(a);
    }

    // ----- start one instance ------------------------------------------------------------------
    __device__ void begin(int64_t instance, const EnsArgs& a) {
        inst = instance;
        const int64_t n = a.n;
        double t0 = a.t0[inst];
        tf = a.tf[inst];
        rtol = a.rtol[inst];
        atol = a.atol[inst];
        if constexpr (P::KAHAN) {
            rtolf = (float)rtol;
            atolf = (float)atol;
        }
#pragma unroll
        for (int q = 0; q < Rhs::NP; ++q) p[q] = a.params[(int64_t)q * n + inst];
        if constexpr (PF) {
#pragma unroll
            for (int q = 0; q < Rhs::NP; ++q) pf[q] = (typename P::PS)p[q];
        }
#pragma unroll
        for (int c = 0; c < D; ++c) {
            y[c] = P::from(a.y0[(int64_t)c * n + inst]);
            yc[c] = (S)0;
        }
        t = t0;
        if constexpr (PHASE) set_phase(t0);
        t_prev = t0;
        h_prev = 0.0;
        h_lim64 = 0.0;
        rem = tf - t0;
        h_lim = 0.0f;
        bounded = !(a.h_min == 0.0 && isinf(a.h_max) && a.h_max > 0.0);
        steps = acc = rej = fev = 0;
        mod100 = 0;
        stiff = nonstiff = 0;
        next_eval = 0;
        if constexpr (CROSS) {
            have_last_off = false;
            last_off = (OffT)0;
            ncross = 0;
            nevents = 0;
            last_push = 0.0;
            have_push = false;
        }
        last_rejected = false;
        done = false;
        status = DEGPU_COMPLETE;
        // direction (solve_ivp.rs:139-147): signum(tf - t0) must be +-1
        double sg = rs_signum(tf - t0);
        if (!(sg == 1.0 || sg == -1.0)) {
            status = DEGPU_ERR_BAD_INPUT;
            done = true;
            return;
        }
        dir = sg;
        double h0 = a.h0;
        if constexpr (Tab::ADAPTIVE) {
            if (h0 == 0.0) {
                h0 = initial_step(t0, a);
                if constexpr (!Tab::DP) fev += 2;  // adaptive/ordinary.rs:28 counts them a second time
            }
        } else {
            if (h0 == 0.0) h0 = fabs(tf - t0) / 100.0;
        }
        if (!valid_h0(h0, t0, a)) {
            status = DEGPU_ERR_BAD_INPUT;
            done = true;
            return;
        }
        h = h0;
        fwd = dir > 0.0;
        if constexpr (MIX) {
            hf = (float)h0;
            remf = narrow_rz(rem);  // |remf| <= |tf - t|: the overshoot test never lets t pass tf
            last_step = false;
        }
        if constexpr (FFT) {
            th = (float)t0;
            tl = (float)(t0 - (double)th);
            tfh = (float)tf;
            tfl = (float)(tf - (double)tfh);
            at_tf = false;
            if constexpr (PHASE) {
                // the phase at t0 reduced to [-pi, pi] in FP64, kept as an FP32 pair
                const double om = p[Rhs::PHASE_RATE], ph = om * t0;
                const double r = fma(-rint(ph * 0.15915494309189535), 6.283185307179586, ph);
                ph0 = (float)r;
                phl = (float)(r - (double)ph0);
                omh = (float)om;
                oml = (float)(om - (double)omh);
            }
        }
        if constexpr (PHASE)
            rhs_at(0.0f, y, k0);
        else
            rhs(t, y, k0);
        fev += 1;
        if constexpr (DENSE && !Tab::DP) {
#pragma unroll
            for (int c = 0; c < D; ++c) {
                cont[0][c] = y[c];
                cont[1][c] = k0[c];
            }
        }
        solout(a);  // t == t_prev == t0
    }

    // ----- one Dormand–Prince step attempt: ordinary.rs:63-268 -------------------------------
    // returns 1 accepted, 2 rejected, 3 error
    __device__ int step_dp(const EnsArgs& a) {
        if constexpr (MIX) {
            // mixed: the step-size guard in FP32 (h_lim = 1e-14 |h_prev|, set on acceptance)
            if (fabsf(hf) < h_lim) {
                status = DEGPU_ERR_STEP_SIZE;
                return 3;
            }
        } else if (abs_lt(h, h_lim64)) {  // |h| < |h_prev| 1e-14
            status = DEGPU_ERR_STEP_SIZE;
            return 3;
        }
        if (steps >= a.max_steps) {
            status = DEGPU_ERR_MAX_STEPS;
            return 3;
        }
        steps += 1;
        mod100 = mod100 == 99 ? 0 : mod100 + 1;
        S k[I][D];
#pragma unroll
        for (int c = 0; c < D; ++c) k[0][c] = k0[c];
        S ys[D];
        double drv[NS];  // DRV: the drive term at each stage's time
        // ys = y + sum_j (a_ij h) k_j for stage i
        auto stage_state = [&](auto i) {
            AccT acc[D];
#pragma unroll
            for (int c = 0; c < D; ++c) acc[c] = acc_begin(y[c]);
            static_for<0, decltype(i)::value>([&](auto j) {
                constexpr double aij = Tab::a(decltype(i)::value, decltype(j)::value);
                if constexpr (aij != 0.0) {
                    S ah = stage_coef(aij);
#pragma unroll
                    for (int c = 0; c < D; ++c) acc_fma(acc[c], ah, k[j][c]);
                }
            });
#pragma unroll
            for (int c = 0; c < D; ++c) ys[c] = acc_end(acc[c]);
        };
        static_for<1, (FSAL_MIX ? NS - 1 : NS)>([&](auto i) {
            stage_state(i);
            if constexpr (MIX) {
                rhs_at(stage_offset(Tab::c(i)), ys, k[i]);
            } else if constexpr (DRV) {
                constexpr int i0 = first_stage_at_c<Tab>(decltype(i)::value);
                if constexpr (i0 == decltype(i)::value)
                    drv[i0] = Rhs::template drive<P>(t + Tab::c(i) * h, p);
                Rhs::template diff_drive<P>(drv[i0], ys, k[i], p);
            } else {
                rhs(t + Tab::c(i) * h, ys, k[i]);
            }
        });
        // ys now holds the last stage state (ysti, ordinary.rs:107)
        S yseg[D], ynew[D], ycn[D];
        {
            AccT acc[D];
#pragma unroll
            for (int c = 0; c < D; ++c) acc[c] = acc_begin((S)0);
            static_for<0, NS>([&](auto i) {
                constexpr double bi_ = Tab::b(decltype(i)::value);
                if constexpr (bi_ != 0.0) {
#pragma unroll
                    for (int c = 0; c < D; ++c) acc_fma(acc[c], (S)bi_, k[i][c]);
                }
            });
#pragma unroll
            for (int c = 0; c < D; ++c) yseg[c] = acc_end(acc[c]);
        }
        S hs;
        if constexpr (MIX)
            hs = hf;
        else
            hs = P::from(h);
#pragma unroll
        for (int c = 0; c < D; ++c) {
            if constexpr (P::KAHAN && !P::PAIR) {  // pairs carry 48 bits: no compensation
                S inc = hs * yseg[c];
                S yk = inc - yc[c];
                S ts = y[c] + yk;
                ycn[c] = (ts - y[c]) - yk;
                ynew[c] = ts;
            } else if constexpr (P::PAIR) {
                AccT acc = acc_begin(y[c]);
                acc_fma(acc, yseg[c], hf);  // hs = hf: the product of a pair and an FP32 number
                ynew[c] = acc_end(acc);
                ycn[c] = (S)0;
            } else {
                ynew[c] = y[c] + hs * yseg[c];
                ycn[c] = (S)0;
            }
        }
        if constexpr (FSAL_MIX) {
            // the last stage sits at (t + h, y_new): its state is y_new, so it is evaluated there
            // and doubles as the derivative at the new point on acceptance
#pragma unroll
            for (int c = 0; c < D; ++c) ys[c] = ynew[c];
            rhs_at(hf, ynew, k[NS - 1]);
        }
        fev += NS - 1;

        NormT err = (NormT)0, err2 = (NormT)0;
        {
            // the embedded error estimate.  Pair stages sum it in pairs too: its terms are of the
            // size of h k while the estimate is of the size of the tolerance, and an FP32 sum's
            // rounding (about 6e-8 h |k|) would exceed a 1e-10 tolerance and reject good steps.
            // The FP32 norm then reads its leading part.
            using ES = typename PickT<P::PAIR, float, S>::type;
            ES es[D];
            {
                AccT ea[D];
#pragma unroll
                for (int c = 0; c < D; ++c) ea[c] = acc_begin((S)0);
                static_for<0, NS>([&](auto j) {
                    constexpr double e_ = Tab::er(decltype(j)::value);
                    if constexpr (e_ != 0.0) {
#pragma unroll
                        for (int c = 0; c < D; ++c) acc_fma(ea[c], (S)e_, k[j][c]);
                    }
                });
#pragma unroll
                for (int c = 0; c < D; ++c) es[c] = (ES)acc_end(ea[c]);
            }
            if (a.rtol_vec || a.atol_vec) {
#pragma unroll
                for (int c = 0; c < D; ++c) err = err + norm_term<true>(c, es[c], y[c], ynew[c], a);
            } else {
#pragma unroll
                for (int c = 0; c < D; ++c) err = err + norm_term<false>(c, es[c], y[c], ynew[c], a);
            }
        }
        if constexpr (Tab::HAS_BH) {
            S es[D];
            {
                AccT ea[D];
#pragma unroll
                for (int c = 0; c < D; ++c) ea[c] = acc_begin(yseg[c]);
                static_for<0, NS>([&](auto j) {
                    constexpr double bh_ = Tab::bh(decltype(j)::value);
                    if constexpr (bh_ != 0.0) {
#pragma unroll
                        for (int c = 0; c < D; ++c) acc_fma(ea[c], (S)(-bh_), k[j][c]);
                    }
                });
#pragma unroll
                for (int c = 0; c < D; ++c) es[c] = acc_end(ea[c]);
            }
            if (a.rtol_vec || a.atol_vec) {
#pragma unroll
                for (int c = 0; c < D; ++c) err2 = err2 + norm_term<true>(c, es[c], y[c], ynew[c], a);
            } else {
#pragma unroll
                for (int c = 0; c < D; ++c) err2 = err2 + norm_term<false>(c, es[c], y[c], ynew[c], a);
            }
        }
        NormT deno = Tab::HAS_BH ? err + (NormT)0.01 * err2 : err;
        if constexpr (P::F32_CTRL) {
            if (deno <= (NormT)0) deno = (NormT)1;
        } else if (nn_le(deno, 0.0)) {
            deno = 1.0;  // deno >= +0: only a zero (or NaN, kept) reaches here
        }
        double scale = 1.0, errd = 0.0;
        float errf = 0.0f, scalef = 1.0f;
        if constexpr (P::F32_CTRL) {
            // mixed with the FP32 controller: the normalisation and the controller's power in
            // FP32 (the error terms are FP32 data)
            // the norm squared, err^2 h^2 / (deno d), decides and feeds the power directly, so
            // no square root and no IEEE division are needed (DOPRI5: deno = err)
            const float eh = err * fabsf(hf);
            float x;
            if constexpr (Tab::HAS_BH)
                x = __fdividef(eh * eh, deno * (float)D);
            else
                x = eh * fabsf(hf) * (float)(1.0 / (double)D);
            errf = x;
            float pw = exp2f(__log2f(x) * (float)(-0.5 / (double)O));
            scalef = fminf(fmaxf(a.safety_f * pw, a.min_scale_f), a.max_scale_f);
        } else {
            if constexpr (MIX)
                errd = (double)fabsf(hf) * err * P::rsqrt(deno * (double)D);
            else
                errd = fabs(h) * err * P::rsqrt(deno * (double)D);
            double error_exponent = 1.0 / (double)O;
            scale = a.safety * P::pow(errd, -error_exponent);
            scale = nn_clamp(scale, a.min_scale, a.max_scale);
            if constexpr (MIX) scalef = (float)scale;
        }

        int result;
        // mixed: the squared FP32 norm against 1 (the norm itself against 1 in FP64)
        bool accept;
        if constexpr (P::F32_CTRL)
            accept = errf <= 1.0f;
        else
            accept = nn_le(errd, 1.0);
        if (accept) {
            double t_new;
            if constexpr (FFT) {
                ff_advance();
                t_new = t;  // t itself is not kept up to date (finish() forms it from th + tl)
            } else if constexpr (MIX)
                t_new = last_step ? tf : t + widen_f32(hf);  // a clamped last step ends exactly at tf
            else
                t_new = t + h;
            S dydt[D];
            if constexpr (FSAL_MIX) {
#pragma unroll
                for (int c = 0; c < D; ++c) dydt[c] = k[NS - 1][c];
            } else if constexpr (PHASE) {
                rhs_at(hf, ynew, dydt);
            } else if constexpr (FFT) {
                rhs(tnow(), ynew, dydt);
            } else if constexpr (DRV && last_stage_at_one<Tab>() > 0) {
                // t_new = t + h is the time of the c = 1 stage (t + 1.0 h)
                Rhs::template diff_drive<P>(drv[first_stage_at_c<Tab>(last_stage_at_one<Tab>())], ynew, dydt, p);
            } else {
                rhs(t_new, ynew, dydt);
            }
            fev += 1;  // the crate's evaluation at the new point
            // stiffness detection, ordinary.rs:165-194
            if (mod100 == 0) {
                bool den_pos, over;
                if constexpr (MIX) {
                    // mixed: in FP32, like the stage data it measures (a warp runs this block
                    // whenever any of its lanes is at a multiple of 100 attempts)
                    float sn = 0.0f, sd = 0.0f;
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        float d1 = lead(yseg[c] - k[NS - 1][c]);
                        sn = sn + d1 * d1;
                        float d2 = lead(dydt[c] - ys[c]);
                        sd = sd + d2 * d2;
                    }
                    den_pos = sd > 0.0f;
                    over = den_pos && hf * sqrtf(sn / sd) > 6.1f;
                } else {
                    double stdnum = 0.0, stden = 0.0;
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        double d1 = (double)yseg[c] - (double)k[NS - 1][c];
                        stdnum = stdnum + d1 * d1;
                        double d2 = (double)dydt[c] - (double)ys[c];
                        stden = stden + d2 * d2;
                    }
                    den_pos = stden > 0.0;
                    over = den_pos && h * sqrt(stdnum / stden) > 6.1;
                }
                if (den_pos) {
                    if (over) {
                        nonstiff = 0;
                        stiff += 1;
                        if (stiff == 15) {
                            status = DEGPU_ERR_STIFFNESS;
                            return 3;
                        }
                    }
                } else {
                    nonstiff += 1;
                    if (nonstiff == 6) stiff = 0;
                }
            }
            if constexpr (DENSE) {
                dense_coefficients(k, ynew, dydt);
            } else {
                fev += I - NS - (I > NS ? 1 : 0);  // DOP853: three dense stages the crate evaluates
            }
            t_prev = t;
            if constexpr (MIX) {
                if constexpr (DENSE) h_prev = t_new - t;  // the interpolation's step length
                h_lim = fabsf(hf) * 1e-14f;
            } else {
                h_prev = h;
                h_lim64 = fabs(h) * 1e-14;
            }
            t = t_new;
            if constexpr (PHASE) {
                if constexpr (FFT)
                    ff_phase_advance();
                else
                    set_phase(t);
            }
#pragma unroll
            for (int c = 0; c < D; ++c) {
                y[c] = ynew[c];
                yc[c] = ycn[c];
                k0[c] = dydt[c];
            }
            if (last_rejected) {
                last_rejected = false;
                if constexpr (MIX)
                    scalef = fminf(scalef, 1.0f);
                else
                    scale = nn_min(scale, 1.0);
            }
            result = 1;
        } else {
            last_rejected = true;
            result = 2;
        }
        if constexpr (MIX) {
            hf = hf * scalef;
            if (bounded) {
                // constrain_step_size, utils.rs:22-33
                double hd = (double)hf;
                if (fabs(hd) < a.h_min)
                    hd = rs_signum(hd) * a.h_min;
                else if (fabs(hd) > a.h_max)
                    hd = rs_signum(hd) * a.h_max;
                hf = (float)hd;
            }
        } else {
            h = h * scale;
            // constrain_step_size, utils.rs:22-33 (a no-op for the default bounds 0 and +inf)
            if (bounded) {
                if (fabs(h) < a.h_min)
                    h = rs_signum(h) * a.h_min;
                else if (fabs(h) > a.h_max)
                    h = rs_signum(h) * a.h_max;
            }
        }
        return result;
    }

    __device__ __forceinline__ S stage_coef(double aij) const {
        if constexpr (MIX)
            return P::from(aij) * hf;  // FP32, or the pair nearest to a_ij
        else if constexpr (P::KAHAN)
            return (float)aij * (float)h;
        else
            return aij * h;
    }

    // dense-output preparation, ordinary.rs:196-235 (k[S..I) computed here for DOP853)
    __device__ void dense_coefficients(S (&k)[I][D], const S* ynew, const S* dydt) {
        if constexpr (DENSE && Tab::DP) {
            S hs;
            if constexpr (MIX)
                hs = hf;
            else
                hs = P::from(h);
#pragma unroll
            for (int c = 0; c < D; ++c) {
                cont[0][c] = y[c];
                S ydiff = ynew[c] - y[c];
                cont[1][c] = ydiff;
                S bspl = hs * k[0][c];
                bspl = bspl - ydiff;
                cont[2][c] = bspl;
                S c3 = ydiff - hs * dydt[c];
                c3 = c3 - bspl;
                cont[3][c] = c3;
            }
            if constexpr (I > NS) {
#pragma unroll
                for (int c = 0; c < D; ++c) k[NS][c] = dydt[c];
                S ys[D];
                static_for<NS + 1, I>([&](auto i) {
                    AccT acc[D];
#pragma unroll
                    for (int c = 0; c < D; ++c) acc[c] = acc_begin(y[c]);
                    static_for<0, decltype(i)::value>([&](auto j) {
                        constexpr double aij = Tab::a(decltype(i)::value, decltype(j)::value);
                        if constexpr (aij != 0.0) {
                            S ah = stage_coef(aij);
#pragma unroll
                            for (int c = 0; c < D; ++c) acc_fma(acc[c], ah, k[j][c]);
                        }
                    });
#pragma unroll
                    for (int c = 0; c < D; ++c) ys[c] = acc_end(acc[c]);
                    if constexpr (MIX)
                        rhs_at(stage_offset(Tab::c(i)), ys, k[i]);
                    else
                        rhs(t + Tab::c(i) * h, ys, k[i]);
                    fev += 1;
                });
            }
            static_for<4, O>([&](auto i) {
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    S s = (S)0;
                    static_for<0, I>([&](auto j) {
                        constexpr double v = Tab::bi(decltype(i)::value, decltype(j)::value);
                        if constexpr (v != 0.0) s = s + (S)v * k[j][c];
                    });
                    cont[i][c] = s * hs;
                }
            });
        }
    }

    // ----- one step of the Adaptive family (RKF45, Cash-Karp): adaptive/ordinary.rs:63-212 -----
    // returns 1 accepted, 2 rejected, 3 error.  `stiff` counts consecutive rejections here.
    __device__ int step_embedded(const EnsArgs& a) {
        if constexpr (MIX) {
            if (fabsf(hf) < h_lim) {
                status = DEGPU_ERR_STEP_SIZE;
                return 3;
            }
        } else if (abs_lt(h, h_lim64)) {  // |h| < |h_prev| 1e-14
            status = DEGPU_ERR_STEP_SIZE;
            return 3;
        }
        if (steps >= a.max_steps) {
            status = DEGPU_ERR_MAX_STEPS;
            return 3;
        }
        steps += 1;
        S k[KN][D];
#pragma unroll
        for (int c = 0; c < D; ++c) k[0][c] = k0[c];
        S ys[D];
        // stage i from the step's start: y + sum_j (a_ij h) k_j in order (add_scaled)
        auto stage = [&](auto i) {
            AccT acc[D];
#pragma unroll
            for (int c = 0; c < D; ++c) acc[c] = acc_begin(y[c]);
            static_for<0, decltype(i)::value>([&](auto j) {
                constexpr double aij = Tab::a(decltype(i)::value, decltype(j)::value);
                if constexpr (aij != 0.0) {
                    S ah = stage_coef(aij);
#pragma unroll
                    for (int c = 0; c < D; ++c) acc_fma(acc[c], ah, k[j][c]);
                }
            });
#pragma unroll
            for (int c = 0; c < D; ++c) ys[c] = acc_end(acc[c]);
            if constexpr (MIX)
                rhs_at(stage_offset(Tab::c(i)), ys, k[i]);
            else
                rhs(t + Tab::c(i) * h, ys, k[i]);
        };
        static_for<1, NS>(stage);
        fev += NS - 1;
        // y_high = y + sum (b_i h) k_i and y_low = y + sum (bl_i h) k_i, each accumulated in order
        // (add_scaled, traits.rs:316-320); their difference is the error estimate
        S yh[D], ycn[D], err[D];
        if constexpr (P::KAHAN) {
            // mixed: the increments in FP32, y_high added to y with Kahan compensation
            S inc[D], es[D];
#pragma unroll
            for (int c = 0; c < D; ++c) inc[c] = es[c] = (S)0;
            static_for<0, NS>([&](auto i) {
                constexpr double bv = Tab::b(decltype(i)::value), lv = Tab::bl(decltype(i)::value);
                if constexpr (bv != 0.0) {
#pragma unroll
                    for (int c = 0; c < D; ++c) inc[c] = inc[c] + (S)bv * k[i][c];
                }
                if constexpr (bv - lv != 0.0) {
#pragma unroll
                    for (int c = 0; c < D; ++c) es[c] = es[c] + (S)(bv - lv) * k[i][c];
                }
            });
            S hs;
            if constexpr (MIX)
                hs = hf;
            else
                hs = P::from(h);
#pragma unroll
            for (int c = 0; c < D; ++c) {
                S d = hs * inc[c];
                S yk = d - yc[c];
                S ts = y[c] + yk;
                ycn[c] = (ts - y[c]) - yk;
                yh[c] = ts;
                err[c] = hs * es[c];
            }
        } else {
            S yl[D];
#pragma unroll
            for (int c = 0; c < D; ++c) {
                yh[c] = y[c];
                yl[c] = y[c];
                ycn[c] = (S)0;
            }
            static_for<0, NS>([&](auto i) {
                constexpr double bv = Tab::b(decltype(i)::value);
                if constexpr (bv != 0.0) {
                    const S bh_ = bv * h;
#pragma unroll
                    for (int c = 0; c < D; ++c) yh[c] = yh[c] + bh_ * k[i][c];
                }
            });
            static_for<0, NS>([&](auto i) {
                constexpr double lv = Tab::bl(decltype(i)::value);
                if constexpr (lv != 0.0) {
                    const S bl_ = lv * h;
#pragma unroll
                    for (int c = 0; c < D; ++c) yl[c] = yl[c] + bl_ * k[i][c];
                }
            });
#pragma unroll
            for (int c = 0; c < D; ++c) err[c] = yh[c] - yl[c];
        }
        // error_norm_inf (traits.rs:413-433): max |err / sk|, fmax keeping the non-NaN operand
        bool accept;
        double scale = 1.0;
        float scalef = 1.0f;
        if constexpr (MIX) {
            // mixed: the norm, the controller's power and the decision in FP32
            float norm = 0.0f;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const float sk = atolf_c(c, a) + rtolf_c(c, a) * fmaxf(fabsf(y[c]), fabsf(yh[c]));
                norm = fmaxf(norm, fabsf(__fdividef(err[c], sk)));
            }
            const float pw = exp2f(__log2f(norm) * (float)(-1.0 / (double)O));
            scalef = fminf(fmaxf(a.safety_f * pw, a.min_scale_f), a.max_scale_f);
            accept = norm <= 1.0f;
        } else {
            double norm = 0.0;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const double sk = atol_c(c, a) + rtol_c(c, a) * fmax_abs((double)y[c], (double)yh[c]);
                norm = fmax_abs(norm, P::quot((double)err[c], sk));
            }
            scale = a.safety * P::pow(norm, -(1.0 / (double)O));
            scale = nn_clamp(scale, a.min_scale, a.max_scale);
            accept = nn_le(norm, 1.0);
        }
        int result;
        if (accept) {
            if constexpr (DENSE) {
                if constexpr (Tab::HAS_BI) {
                    // the dense-output stages (adaptive/ordinary.rs:146-163), from the step's start
                    static_for<NS, I>(stage);
#pragma unroll
                    for (int c = 0; c < D; ++c) cont[0][c] = y[c];
                    static_for<0, I>([&](auto i) {
#pragma unroll
                        for (int c = 0; c < D; ++c) cont[1 + decltype(i)::value][c] = k[i][c];
                    });
                } else {
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        cont[0][c] = y[c];
                        cont[1][c] = k[0][c];
                    }
                }
            }
            // the crate evaluates the dense-output stages on every accepted step; without
            // requested output nothing reads them, so only their count is kept
            if constexpr (Tab::HAS_BI) fev += I - NS;
            t_prev = t;
            if constexpr (MIX) {
                h_lim = fabsf(hf) * 1e-14f;
            } else {
                h_prev = h;
                h_lim64 = fabs(h) * 1e-14;
            }
            if (last_rejected) {
                last_rejected = false;
                stiff = 0;
                if constexpr (MIX)
                    scalef = fminf(scalef, 1.0f);
                else
                    scale = nn_min(scale, 1.0);
            }
            if constexpr (FFT) {
                ff_advance();
                if constexpr (PHASE) ff_phase_advance();
            } else if constexpr (MIX) {
                t = last_step ? tf : t + widen_f32(hf);  // a clamped last step ends exactly at tf
                if constexpr (PHASE) set_phase(t);
            } else {
                t = t + h;
            }
#pragma unroll
            for (int c = 0; c < D; ++c) {
                y[c] = yh[c];
                yc[c] = ycn[c];
            }
            if constexpr (Tab::FSAL) {
                // first same as last (ordinary.rs:174-177): the last stage is the new derivative
#pragma unroll
                for (int c = 0; c < D; ++c) k0[c] = k[NS - 1][c];
            } else {
                if constexpr (PHASE)
                    rhs_at(0.0f, y, k0);
                else
                    rhs(tnow(), y, k0);
                fev += 1;
            }
            result = 1;
        } else {
            last_rejected = true;
            stiff += 1;
            if (stiff >= 100) {  // max_rejects default, src/methods/erk/mod.rs:140
                status = DEGPU_ERR_STIFFNESS;
                return 3;
            }
            result = 2;
        }
        if constexpr (MIX) {
            hf = hf * scalef;
            if (bounded) {
                double hd = (double)hf;
                if (fabs(hd) < a.h_min)
                    hd = rs_signum(hd) * a.h_min;
                else if (fabs(hd) > a.h_max)
                    hd = rs_signum(hd) * a.h_max;
                hf = (float)hd;
            }
        } else {
            h = h * scale;
            if (bounded) {
                if (fabs(h) < a.h_min)
                    h = rs_signum(h) * a.h_min;
                else if (fabs(h) > a.h_max)
                    h = rs_signum(h) * a.h_max;
            }
        }
        return result;
    }

    // ----- one fixed RK4 step: fixed/ordinary.rs:58-138 -----------------------------------------
    __device__ int step_fixed(const EnsArgs& a) {
        if (steps >= a.max_steps) {
            status = DEGPU_ERR_MAX_STEPS;
            return 3;
        }
        steps += 1;
        S k[I][D];
#pragma unroll
        for (int c = 0; c < D; ++c) k[0][c] = k0[c];
        S ys[D];
        static_for<1, NS>([&](auto i) {
            AccT acc[D];
#pragma unroll
            for (int c = 0; c < D; ++c) acc[c] = acc_begin(y[c]);
            static_for<0, decltype(i)::value>([&](auto j) {
                constexpr double aij = Tab::a(decltype(i)::value, decltype(j)::value);
                if constexpr (aij != 0.0) {
                    S ah = stage_coef(aij);
#pragma unroll
                    for (int c = 0; c < D; ++c) acc_fma(acc[c], ah, k[j][c]);
                }
            });
#pragma unroll
            for (int c = 0; c < D; ++c) ys[c] = acc_end(acc[c]);
            rhs(t + Tab::c(i) * h, ys, k[i]);
        });
        fev += NS - 1;
        t_prev = t;
        h_prev = h;
        if constexpr (DENSE) {
#pragma unroll
            for (int c = 0; c < D; ++c) {
                cont[0][c] = y[c];
                cont[1][c] = k0[c];
            }
        }
        S yn[D];
#pragma unroll
        for (int c = 0; c < D; ++c) yn[c] = y[c];
        if constexpr (P::KAHAN) {
            S inc[D];
#pragma unroll
            for (int c = 0; c < D; ++c) inc[c] = (S)0;
            static_for<0, NS>([&](auto i) {
                S bh_ = (float)Tab::b(i) * (float)h;
#pragma unroll
                for (int c = 0; c < D; ++c) inc[c] = inc[c] + bh_ * k[i][c];
            });
#pragma unroll
            for (int c = 0; c < D; ++c) {
                S yk = inc[c] - yc[c];
                S ts = yn[c] + yk;
                yc[c] = (ts - yn[c]) - yk;
                yn[c] = ts;
            }
        } else {
            static_for<0, NS>([&](auto i) {
                S bh_ = Tab::b(i) * h;
#pragma unroll
                for (int c = 0; c < D; ++c) yn[c] = yn[c] + bh_ * k[i][c];
            });
        }
        t = t + h;
#pragma unroll
        for (int c = 0; c < D; ++c) y[c] = yn[c];
        rhs(t, y, k0);
        fev += 1;
        return 1;
    }

    // ----- one iteration of the driver loop: solve_ivp.rs:191-266 ----------------------------
    __device__ __forceinline__ void iterate(const EnsArgs& a) {
        const double eps10 = 2.220446049250313e-16 * 10.0;
        if constexpr (MIX) {
            // mixed form: the overshoot test on FP32 copies; an attempt that reaches tf is
            // clamped to the remaining span and, if accepted, ends exactly at tf
            last_step = false;
            if (fwd ? hf >= remf : hf <= remf) {
                if (fabsf(remf) < (float)eps10) {
                    done = true;
                    return;
                }
                hf = remf;
                last_step = true;
            }
        } else if constexpr (P::KAHAN) {
            // mixed form of RK4: the remaining interval tf - t is kept (updated on acceptance),
            // so the overshoot test is one comparison
            if (dir > 0.0 ? h > rem : h < rem) {
                if (fabs(rem) < eps10) {
                    done = true;
                    return;
                }
                h = rem;
            }
        } else if (fwd ? t + h > tf : t + h < tf) {  // (t + h - tf) dir > 0, exactly
            double h_new = tf - t;
            if (fabs(h_new) < eps10) {
                done = true;
                return;
            }
            h = h_new;
        }
        int r;
        if constexpr (Tab::DP)
            r = step_dp(a);
        else if constexpr (Tab::ADAPTIVE)
            r = step_embedded(a);
        else
            r = step_fixed(a);
        if (r == 3) {
            done = true;
            return;
        }
        if (r == 2) {
            rej += 1;
            return;
        }
        acc += 1;
        solout(a);
        if constexpr (CROSS) {
            if (status == DEGPU_INTERRUPTED) {  // ControlFlag::Terminate (solve_ivp.rs:254-259)
                done = true;
                return;
            }
        }
        if constexpr (MIX) {
            if (last_step) {
                done = true;  // t == tf
            } else {
                if constexpr (FFT)
                    remf = ff_rem();
                else
                    remf = narrow_rz(tf - t);
                if (fabsf(remf) <= (float)eps10) done = true;
            }
        } else if constexpr (P::KAHAN) {
            rem = tf - t;
            if (fabs(rem) <= eps10) done = true;
        } else {
            if (nn_le(fabs(tf - t), eps10)) done = true;
        }
    }

    __device__ void finish(const EnsArgs& a) const {
        const int64_t n = a.n;
#pragma unroll
        for (int c = 0; c < D; ++c) a.y_final[(int64_t)c * n + inst] = to_f64(y[c]) - to_f64(yc[c]);
        for (int c = D; c < a.dmax; ++c) a.y_final[(int64_t)c * n + inst] = 0.0;
        if (a.t_final) {
            if constexpr (FFT)
                a.t_final[inst] = at_tf ? tf : (double)th + (double)tl;
            else
                a.t_final[inst] = t;
        }
        if (a.accepted) a.accepted[inst] = acc;
        if (a.rejected) a.rejected[inst] = rej;
        if (a.fevals) a.fevals[inst] = fev;
        if (a.status) a.status[inst] = status;
        if constexpr (CROSS) a.cross_count[inst] = ncross;
    }
};

// ---------------------------------------------------------------------------------------------
// Multi-family persistent kernel with longest-first work lists.
//
// The plan kernels (plan.cu) sort every instance into the work list of its family, in descending
// order of estimated cost |tf - t0| * rtol^(-1/order), so that the longest solves start first and
// the end of each list holds the shortest ones.  Each warp works on one family at a time (the
// family switch is warp-uniform, so it costs no divergence); a lane whose instance finishes takes
// the next item of that family's list; when the list is empty and every lane of the warp is idle,
// the warp moves to the next family that still has work.
// ---------------------------------------------------------------------------------------------
struct MultiQueue {
    const int64_t* items;         // work lists of the three families, concatenated
    const int64_t* start;         // [3] first item of each family's list
    const int64_t* count;         // [3] length of each family's list
    unsigned long long* head;     // [3] per-family list heads
};

template <class Tab, class P, bool DENSE, class R0, class R1, class R2, bool CROSS>
struct MultiLane {
    union {
        Lane<Tab, R0, P, DENSE, CROSS> l0;
        Lane<Tab, R1, P, DENSE, CROSS> l1;
        Lane<Tab, R2, P, DENSE, CROSS> l2;
    };
    __device__ MultiLane() {}
};

// CROSS: crossing or event detection (the lanes of erk_cross_kernel) instead of output times only.
template <class Tab, class P, bool DENSE, class R0, class R1, class R2, bool CROSS = false>
__global__ void __launch_bounds__(128, P::MULTI_MIN_BLOCKS) erk_multi_kernel(EnsArgs a, MultiQueue q) {
    MultiLane<Tab, P, DENSE, R0, R1, R2, CROSS> M;
    const int64_t cnt[3] = {q.count[0], q.count[1], q.count[2]};
    const int64_t st[3] = {q.start[0], q.start[1], q.start[2]};
    // every warp starts on the longest list and moves on to the next family when it runs dry, so
    // that most of the time an SM runs one family's code (the three families' step code together
    // overflow the instruction cache)
    int fam = cnt[2] >= cnt[1] && cnt[2] >= cnt[0] ? 2 : (cnt[1] >= cnt[0] ? 1 : 0);
    bool active = false, exhausted = false;
    for (;;) {
        // Lanes refill together: a lane's set-up (the initial-step heuristic, two right-hand
        // sides and the norms) costs the warp the same issue time for one lane as for all, so
        // finished lanes wait until DEGPU_REFILL_BATCH of them are idle (or the warp is) and then
        // start their next instances in one pass.
        const unsigned idle = __ballot_sync(0xffffffffu, !active && !exhausted);
        const bool refill = __popc(idle) >= DEGPU_REFILL_BATCH || __ballot_sync(0xffffffffu, active) == 0u;
        if (refill && !active && !exhausted) {
            unsigned long long w = atomicAdd(&q.head[fam], 1ULL);
            if (w < (unsigned long long)cnt[fam]) {
                int64_t inst = q.items[st[fam] + (int64_t)w];
                if (fam == 0) {
                    M.l0.begin(inst, a);
                    if (M.l0.done) M.l0.finish(a); else active = true;
                } else if (fam == 1) {
                    M.l1.begin(inst, a);
                    if (M.l1.done) M.l1.finish(a); else active = true;
                } else {
                    M.l2.begin(inst, a);
                    if (M.l2.done) M.l2.finish(a); else active = true;
                }
            } else {
                exhausted = true;
            }
        }
        const unsigned amask = __ballot_sync(0xffffffffu, active);
        if (amask == 0u) {
            if (!__any_sync(0xffffffffu, !exhausted)) {
                // the whole warp is idle and its list is empty: find a family with work left
                int nf = -1;
                if ((threadIdx.x & 31) == 0) {
                    for (int f = 0; f < 3; ++f) {
                        int g = (fam + 2 + 2 * f) % 3;  // descending: Lorenz, pendulum, Van der Pol
                        if (atomicAdd(&q.head[g], 0ULL) < (unsigned long long)cnt[g]) {
                            nf = g;
                            break;
                        }
                    }
                }
                nf = __shfl_sync(0xffffffffu, nf, 0);
                if (nf < 0) break;
                fam = nf;
                exhausted = false;
            }
            continue;
        }
        if (active) {
            // the active lanes step together until one of them finishes (it then refills)
            bool fin;
            if (fam == 0) {
                do {
                    M.l0.iterate(a);
                    fin = M.l0.done;
                } while (!__any_sync(amask, fin));
                if (fin) { M.l0.finish(a); active = false; }
            } else if (fam == 1) {
                do {
                    M.l1.iterate(a);
                    fin = M.l1.done;
                } while (!__any_sync(amask, fin));
                if (fin) { M.l1.finish(a); active = false; }
            } else {
                do {
                    M.l2.iterate(a);
                    fin = M.l2.done;
                } while (!__any_sync(amask, fin));
                if (fin) { M.l2.finish(a); active = false; }
            }
        }
    }
}

// Resident per-instance solver state of the serving path: a Lane parked between rounds.
// `phase`: 0 not started, 1 in progress, 2 finished.
template <class LaneT>
struct Parked {
    int32_t phase;
    int32_t pad;
    LaneT lane;
};

// Resumable persistent form used by the server: every instance is visited once per round; a
// visit resumes the parked state (or starts the instance), advances it by at most `budget`
// driver iterations, then parks it again or finishes it.  `done_count` counts finished
// instances across rounds.  Slot w of `park` holds work item w: instance a.index[w] when an
// index list is given (a request split by precision), else instance w.
template <class Tab, class Rhs, class P, bool DENSE>
__global__ void __launch_bounds__(128) erk_round_kernel(EnsArgs a, Parked<Lane<Tab, Rhs, P, DENSE>>* park,
                                                        int budget, unsigned long long* done_count) {
    for (;;) {
        unsigned long long w = atomicAdd(a.ticket, 1ULL);
        if (w >= (unsigned long long)a.count) break;
        Parked<Lane<Tab, Rhs, P, DENSE>>& slot = park[w];
        int phase = slot.phase;
        if (phase == 2) continue;
        Lane<Tab, Rhs, P, DENSE> L;
        if (phase == 0) {
            L.begin(a.index ? a.index[w] : (int64_t)w, a);
        } else {
            L = slot.lane;
        }
        for (int it = 0; it < budget && !L.done; ++it) L.iterate(a);
        if (L.done) {
            L.finish(a);
            slot.phase = 2;
            atomicAdd(done_count, 1ULL);
        } else {
            slot.lane = L;
            slot.phase = 1;
        }
    }
}

// One instance per thread, run to completion.
template <class Tab, class Rhs, class P, bool DENSE>
__global__ void __launch_bounds__(128) erk_thread_kernel(EnsArgs a) {
    int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= a.count) return;
    Lane<Tab, Rhs, P, DENSE> L;
    L.begin(a.index ? a.index[w] : w, a);
    while (!L.done) L.iterate(a);
    L.finish(a);
}

// One instance per thread with crossing detection (degpu_solve_ensemble_crossing).
template <class Tab, class Rhs, class P>
__global__ void __launch_bounds__(128) erk_cross_kernel(EnsArgs a) {
    int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= a.count) return;
    Lane<Tab, Rhs, P, true, true> L;
    L.begin(a.index ? a.index[w] : w, a);
    while (!L.done) L.iterate(a);
    L.finish(a);
}

// Persistent form: a fixed grid; each lane takes a work item from the device queue, steps it,
// and as soon as its instance finishes takes the next one (lane refill), so lanes whose instance
// needs few steps do not idle while their warp-mates finish long ones.
template <class Tab, class Rhs, class P, bool DENSE>
__global__ void __launch_bounds__(128) erk_persistent_kernel(EnsArgs a) {
    Lane<Tab, Rhs, P, DENSE> L;
    bool active = false;
    for (;;) {
        if (!active) {
            unsigned long long w = atomicAdd(a.ticket, 1ULL);
            if (w >= (unsigned long long)a.count) break;
            L.begin(a.index ? a.index[w] : (int64_t)w, a);
            if (L.done) {
                L.finish(a);
                continue;
            }
            active = true;
        }
        L.iterate(a);
        if (L.done) {
            L.finish(a);
            active = false;
        }
    }
}

}  // namespace degpu
