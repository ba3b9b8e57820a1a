// rhs.cuh — CUDA __device__ twins of `ODE::diff(&self, t, &y, &mut dydt)` (src/ode/ode.rs:20-44)
// for the built-in families, and the precision policies they are evaluated under.
//
// Each family is a struct with the state dimension D, the parameter count NP and
//     template <class P, class PT> static void diff(double t, const typename P::S* y,
//                                                   typename P::S* dydt, const PT* p);
// (PT = double, or float for the mixed form's parameter copies).
// The expressions keep the evaluation order of the crate's test systems (tests/ode/systems.rs),
// which is what the parity path (compiled without FMA contraction) must reproduce.
#pragma once

#include "dd_math.cuh"
#include "df_math.cuh"
#include "f32_math.cuh"
#include "f64_tab_math.cuh"

namespace degpu {

// Precision policies --------------------------------------------------------------------------
// Minimum resident blocks per SM requested for the mixed form's persistent kernel (a register
// cap: 65536 / (128 * blocks) registers per thread); 1 leaves the compiler's choice.
#ifndef DEGPU_MIXED_MIN_BLOCKS
#define DEGPU_MIXED_MIN_BLOCKS 1
#endif
// The same for the FP32-pair stage kernels (PrecMixedPair): three blocks of 128 per SM fit the
// register file without spills (measured: four blocks gained nothing, five spill).
#ifndef DEGPU_PAIR_MIN_BLOCKS
#define DEGPU_PAIR_MIN_BLOCKS 3
#endif
// Lanes of the multi-family persistent kernel refill in batches of at least this many.
#ifndef DEGPU_REFILL_BATCH
#define DEGPU_REFILL_BATCH 4
#endif
// Mixed form's sin/cos: 0 uses f32_math.cuh, 1 the CUDA library's sinf/cosf.
#ifndef DEGPU_MIXED_LIBM_TRIG
#define DEGPU_MIXED_LIBM_TRIG 0
#endif

// PhaseOf<R>::value: the family declares PHASE (a drive phase the mixed form advances in FP32,
// with `phase` and `diff_phase`).
template <class R>
struct PhaseOf {
    template <class U>
    __host__ __device__ static constexpr bool test(decltype(U::PHASE)*) { return U::PHASE; }
    template <class U>
    __host__ __device__ static constexpr bool test(...) { return false; }
    static constexpr bool value = test<R>(nullptr);
};

// DriveOf<R>::value: the family declares DRIVE, a time-dependent term that its FP64 forms
// evaluate once per distinct stage time (`drive` and `diff_drive`).
template <class R>
struct DriveOf {
    template <class U>
    __host__ __device__ static constexpr bool test(decltype(U::DRIVE)*) { return U::DRIVE; }
    template <class U>
    __host__ __device__ static constexpr bool test(...) { return false; }
    static constexpr bool value = test<R>(nullptr);
};

// FloatParamsOf<R>::value: the family's diff accepts FP32 parameters (BuiltinRhs).
template <class R>
struct FloatParamsOf {
    template <class U>
    __host__ __device__ static constexpr bool test(decltype(U::FLOAT_PARAMS)*) { return U::FLOAT_PARAMS; }
    template <class U>
    __host__ __device__ static constexpr bool test(...) { return false; }
    static constexpr bool value = test<R>(nullptr);
};

// Reciprocal and reciprocal square root for the contracted FP64 forms: the hardware estimate
// (rcp.approx / rsqrt.approx, about 2^-20 relative) refined by two Newton steps (quadratic, to
// FP64 rounding: within an ulp or two of the IEEE result), five FP64 instructions where the IEEE
// division and square root take about nine each.  Outside [2^-1000, 2^1000] (where the estimate
// flushes subnormals) they fall back to the IEEE operations.
__device__ __forceinline__ bool fp64_mid_range(double x) {
    const long long e = (__double_as_longlong(x) >> 52) & 0x7ff;
    return e > 23 && e < 2023;  // 2^-1000 < |x| < 2^1000
}
__device__ __forceinline__ double rcp_nr(double x) {
    if (!fp64_mid_range(x)) return 1.0 / x;
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}
__device__ __forceinline__ double rsqrt_nr(double x) {
    if (!fp64_mid_range(x) || x < 0.0) return sqrt(1.0 / x);
    double r;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    // r <- r + r (1 - x r^2) / 2
    double e = fma(-x * r, r, 1.0);
    r = fma(0.5 * r, e, r);
    e = fma(-x * r, r, 1.0);
    return fma(0.5 * r, e, r);
}

// Parity: FP64, crate operation order, correctly rounded pow/sin/cos, no FMA contraction (the
// translation units that instantiate it are compiled with -fmad=false).
struct PrecParity {
    using S = double;
    using PS = double;             // parameter copies of the mixed forms (unused here)
    static constexpr bool PAIR = false;  // stages in FP32 pairs (PrecMixedPair)
    static constexpr int ID = 0;
    static constexpr bool KAHAN = false;
    static constexpr bool F32_CTRL = false;
    static constexpr int MULTI_MIN_BLOCKS = 1;
    // the controller's x^(-0.2) and x^(-0.125) through pow_ctrl_neg (fixed-point residual, Ziv's
    // test, pow_ctrl behind it): the same correctly rounded values with far fewer FP64 instructions
    __device__ static __forceinline__ double pow(double x, double y) { return ddm::pow_ctrl_neg(x, y); }
    __device__ static __forceinline__ double sin(double x) { return ddm::sin_cr(x); }
    __device__ static __forceinline__ double cos(double x) { return ddm::cos_cr(x); }
    __device__ static __forceinline__ S from(double x) { return x; }
    // the error norm's quotients and the controller's sqrt(1/x): IEEE, as the crate computes them
    __device__ static __forceinline__ double quot(double a, double b) { return a / b; }
    __device__ static __forceinline__ double rsqrt(double x) { return sqrt(1.0 / x); }
};
// Fast FP64: FMA contraction and the CUDA math library.
struct PrecFast {
    using S = double;
    using PS = double;
    static constexpr bool PAIR = false;
    static constexpr int ID = 1;
    static constexpr bool KAHAN = false;
    static constexpr bool F32_CTRL = false;
    static constexpr int MULTI_MIN_BLOCKS = 1;
    __device__ static __forceinline__ double pow(double x, double y) { return ::pow(x, y); }
    __device__ static __forceinline__ double sin(double x) { return ::sin(x); }
    __device__ static __forceinline__ double cos(double x) { return ::cos(x); }
    __device__ static __forceinline__ S from(double x) { return x; }
    __device__ static __forceinline__ double quot(double a, double b) { return a * rcp_nr(b); }
    __device__ static __forceinline__ double rsqrt(double x) { return rsqrt_nr(x); }
};
// Plain FP64: FMA contraction, the refined hardware reciprocal and reciprocal square root in the
// error norm and the controller, the table-driven sin/cos of f64_tab_math.cuh (within one unit in
// the last place, about 16 FP64 instructions), and the correctly rounded controller power of the
// parity path; results differ from the crate's by rounding only.
struct PrecPlain : PrecFast {
    static constexpr int ID = 3;
    __device__ static __forceinline__ double pow(double x, double y) { return ddm::pow_ctrl_neg(x, y); }
    __device__ static __forceinline__ double sin(double x) { return f64t::sin(x); }
    __device__ static __forceinline__ double cos(double x) { return f64t::cos(x); }
};
// Mixed: stages in FP32, y accumulated with Kahan compensation; the error terms, the norm, the
// controller's power and the accept decision in FP32, t as an FP32 pair (see Lane).
struct PrecMixed {
    using S = float;
    using PS = float;
    static constexpr bool PAIR = false;
    static constexpr int ID = 2;
    static constexpr bool KAHAN = true;
    static constexpr bool F32_CTRL = true;
    static constexpr int MULTI_MIN_BLOCKS = DEGPU_MIXED_MIN_BLOCKS;
    // x^(-1/order) of the controller: FP64 result from an FP32 log2/exp2 estimate refined by
    // one FP64 Newton step on r^q = x^-1 (q = 5 or 8); general y falls back to FP64 pow.
    __device__ static __forceinline__ double pow(double x, double y) {
        if ((y == -0.2 || y == -0.125) && x > 1e-300 && x < 1e300) {
            double q = (y == -0.2) ? 5.0 : 8.0;
            float lx = __log2f((float)x);
            double r = (double)exp2f(lx * (float)y);
            double rq = r * r;  // r^2
            rq = rq * rq;       // r^4
            if (q == 8.0) rq = rq * rq;
            else rq = rq * r;
            // Newton: r <- r (1 + (1 - x r^q)/q)
            double e = fma(-x, rq, 1.0);
            return fma(r, e / q, r);
        }
        return ::pow(x, y);
    }
#if DEGPU_MIXED_LIBM_TRIG
    __device__ static __forceinline__ float sin(float x) { return ::sinf(x); }
    __device__ static __forceinline__ float cos(float x) { return ::cosf(x); }
#else
    __device__ static __forceinline__ float sin(float x) { return f32m::sin_f32(x); }
    __device__ static __forceinline__ float cos(float x) { return f32m::cos_f32(x); }
#endif
    __device__ static __forceinline__ S from(double x) { return (float)x; }
    __device__ static __forceinline__ double quot(double a, double b) { return a * rcp_nr(b); }
    __device__ static __forceinline__ double rsqrt(double x) { return rsqrt_nr(x); }
};
// Mixed with the FP64 controller: FP32 stages and Kahan-compensated y as in PrecMixed; the error
// norm over the FP32 error terms, the controller's power, the accept decision, t and h in FP64.
struct PrecMixedF64Ctrl : PrecMixed {
    static constexpr int ID = 4;
    static constexpr bool F32_CTRL = false;
};
// Mixed with FP32-pair stages (df_math.cuh, about 48 bits): the state, the stage states, the
// right-hand sides and the stage combinations in pairs, everything else (the step size, the error
// norm, the controller, the accept decision, t as an FP32 pair) as in PrecMixed.  A DEGPU_MIXED
// solve runs the instances whose rtol is below the FP32 stages' bound with it: they keep FP64-like
// accuracy, and every pair operation costs 6 to 11 FP32 instructions where an FP64 instruction
// costs the issue time of 64.
struct PrecMixedPair : PrecMixed {
    using S = df;
    using PS = df;
    static constexpr bool PAIR = true;
    static constexpr int ID = 5;
    static constexpr int MULTI_MIN_BLOCKS = DEGPU_PAIR_MIN_BLOCKS;
    __device__ static __forceinline__ df sin(df x) { return df_sin(x); }
    __device__ static __forceinline__ df cos(df x) { return df_cos(x); }
    __device__ static __forceinline__ S from(double x) { return df(x); }
};

// Families -------------------------------------------------------------------------------------
// `diff` takes the parameters as FP64 or, in the mixed form, as FP32 copies made once per
// instance (PT = float), so that no stage converts a parameter.  Built-in families derive from
// BuiltinRhs to say they accept both; run-time (NVRTC) families take FP64 parameters only.
struct BuiltinRhs {
    static constexpr bool FLOAT_PARAMS = true;
};
// tests/ode/systems.rs:85-101
struct RhsLorenz : BuiltinRhs {
    static constexpr int ID = 1, D = 3, NP = 3;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        S sigma = (S)p[0], rho = (S)p[1], beta = (S)p[2];
        S x = y[0], yv = y[1], z = y[2];
        dydt[0] = sigma * (yv - x);
        dydt[1] = x * (rho - z) - yv;
        dydt[2] = x * yv - beta * z;
    }
};

// tests/ode/systems.rs:62-78
struct RhsVanDerPol : BuiltinRhs {
    static constexpr int ID = 2, D = 2, NP = 1;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        S mu = (S)p[0];
        S y1 = y[0], y2 = y[1];
        dydt[0] = y2;
        dydt[1] = mu * ((S)1 - y1 * y1) * y2 - y1;
    }
};

// Damped driven pendulum, g/l = 1: theta' = omega, omega' = -gamma omega - sin(theta) + A cos(Omega t)
// (the model of examples/ode/05_damped_pendulum/main.rs:34-40 plus a periodic drive).
struct RhsPendulum : BuiltinRhs {
    static constexpr int ID = 3, D = 2, NP = 3;
    // Mixed form: the drive phase Omega t reduced to [-pi, pi] in FP64 once per accepted step;
    // a stage at t + dt adds Omega dt to it in FP32 (diff_phase), so the stages need no FP64.
    static constexpr bool PHASE = true;
    static constexpr int PHASE_RATE = 2;  // the parameter that is d(phase)/dt (Omega)
    __device__ static __forceinline__ float phase(double t, const double* p) {
        double ph = p[2] * t;
        double k = rint(ph * 0.15915494309189535);
        return (float)fma(-k, 6.283185307179586, ph);
    }
    // PH: float, or an FP32 pair (the phase and its low part) for pair stages; DT: the stage offset
    // c_i h, FP32 or a pair
    template <class P, class PH, class DT>
    __device__ static __forceinline__ void diff_phase(PH ph0, DT dt, const typename P::S* y, typename P::S* dydt,
                                                      const typename P::PS* pf) {
        using S = typename P::S;
        S theta = y[0], omega = y[1];
        PH r = ph0 + pf[2] * dt;
        dydt[0] = omega;
        dydt[1] = -pf[0] * omega - P::sin(theta) + pf[1] * P::cos(r);
    }
    // FP64 forms: the drive term A cos(Omega t) on its own, so that stages at the same time (the
    // last two DOPRI5 stages and the new point all sit at t + h) share one evaluation; diff_drive
    // then forms (-gamma omega - sin theta) + drive, the order of diff.
    static constexpr bool DRIVE = true;
    template <class P>
    __device__ static __forceinline__ double drive(double t, const double* p) {
        return p[1] * P::cos(p[2] * t);
    }
    template <class P>
    __device__ static __forceinline__ void diff_drive(double drv, const double* y, double* dydt, const double* p) {
        const double omega = y[1];
        dydt[0] = omega;
        dydt[1] = -p[0] * omega - P::sin(y[0]) + drv;
    }
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double t, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        S theta = y[0], omega = y[1];
        dydt[0] = omega;
        if constexpr (P::KAHAN) {
            // FP32 stage arithmetic; the drive phase Omega t is formed and reduced in FP64 so that
            // the long horizon does not cost phase accuracy.
            double ph = p[2] * t;
            double k = rint(ph * 0.15915494309189535);
            float r = (float)fma(-k, 6.283185307179586, ph);
            dydt[1] = -(float)p[0] * omega - P::sin(theta) + (float)p[1] * P::cos(r);
        } else {
            double gamma = p[0], A = p[1], Omega = p[2];
            dydt[1] = -gamma * omega - P::sin(theta) + A * P::cos(Omega * t);
        }
    }
};

// tests/ode/systems.rs:6-17
struct RhsExpGrowth : BuiltinRhs {
    static constexpr int ID = 5, D = 1, NP = 1;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        dydt[0] = (typename P::S)p[0] * y[0];
    }
};

// tests/ode/systems.rs:19-31
struct RhsLinear : BuiltinRhs {
    static constexpr int ID = 6, D = 1, NP = 2;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        dydt[0] = (S)p[0] + (S)p[1] * y[0];
    }
};

// tests/ode/systems.rs:33-46
struct RhsHarmonic : BuiltinRhs {
    static constexpr int ID = 7, D = 2, NP = 1;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        dydt[0] = y[1];
        dydt[1] = -(S)p[0] * y[0];
    }
};

// tests/ode/systems.rs:48-60
struct RhsLogistic : BuiltinRhs {
    static constexpr int ID = 8, D = 1, NP = 2;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        dydt[0] = (S)p[0] * y[0] * ((S)1 - y[0] / (S)p[1]);
    }
};

// tests/ode/systems.rs:155-173
struct RhsRobertson : BuiltinRhs {
    static constexpr int ID = 9, D = 3, NP = 0;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT*) {
        using S = typename P::S;
        S y1 = y[0], y2 = y[1], y3 = y[2];
        dydt[0] = (S)-0.04 * y1 + (S)1.0e4 * y2 * y3;
        dydt[1] = (S)0.04 * y1 - (S)1.0e4 * y2 * y3 - (S)3.0e7 * y2 * y2;
        dydt[2] = (S)3.0e7 * y2 * y2;
    }
};

// tests/ode/systems.rs:175-190
struct RhsHires : BuiltinRhs {
    static constexpr int ID = 10, D = 8, NP = 0;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT*) {
        using S = typename P::S;
        dydt[0] = (S)-1.71 * y[0] + (S)0.43 * y[1] + (S)8.32 * y[2] + (S)0.0007;
        dydt[1] = (S)1.71 * y[0] - (S)8.75 * y[1];
        dydt[2] = (S)-10.03 * y[2] + (S)0.43 * y[3] + (S)0.035 * y[4];
        dydt[3] = (S)8.32 * y[1] + (S)1.71 * y[2] - (S)1.12 * y[3];
        dydt[4] = (S)-1.745 * y[4] + (S)0.43 * y[5] + (S)0.43 * y[6];
        dydt[5] = (S)-280.0 * y[5] * y[7] + (S)0.69 * y[3] + (S)1.71 * y[4] - (S)0.43 * y[5] + (S)0.69 * y[6];
        dydt[6] = (S)280.0 * y[5] * y[7] - (S)1.81 * y[6];
        dydt[7] = (S)-280.0 * y[5] * y[7] + (S)1.81 * y[6];
    }
};

// tests/ode/systems.rs:103-120
struct RhsBrusselator : BuiltinRhs {
    static constexpr int ID = 11, D = 2, NP = 2;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        S a = (S)p[0], b = (S)p[1], y1 = y[0], y2 = y[1];
        dydt[0] = a + y1 * y1 * y2 - (b + (S)1) * y1;
        dydt[1] = b * y1 - y1 * y1 * y2;
    }
};

// tests/bvp/systems.rs:25-57 (pipe heat transfer): heat_loss_rate.powi(2) -> b*b.
struct RhsPipeHeat : BuiltinRhs {
    static constexpr int ID = 13, D = 2, NP = 2;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        const S b = (S)p[0], amb = (S)p[1];
        dydt[0] = y[1];
        dydt[1] = (b * b) * (y[0] - amb);
    }
};

// examples/ode/17_quadrature/main.rs:41-55: damped mass-spring system augmented with the energy
// dissipated by the damper, y = [x, v, W], p = [k, m, c].
struct RhsDampedQuadrature : BuiltinRhs {
    static constexpr int ID = 14, D = 3, NP = 3;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        const S k = (S)p[0], m = (S)p[1], c = (S)p[2];
        const S x = y[0], v = y[1];
        dydt[0] = v;
        dydt[1] = -(k / m) * x - (c / m) * v;
        dydt[2] = c * v * v;
    }
};

// tests/ode/systems.rs:122-153; powi(2) -> x*x, powi(3) -> x*(x*x) as LLVM expands them.
struct RhsCr3bp : BuiltinRhs {
    static constexpr int ID = 12, D = 6, NP = 1;
    template <class P, class PT>
    __device__ static __forceinline__ void diff(double, const typename P::S* y, typename P::S* dydt, const PT* p) {
        using S = typename P::S;
        S mu = (S)p[0];
        S rx = y[0], ry = y[1], rz = y[2], vx = y[3], vy = y[4], vz = y[5];
        S a = rx + mu, b = rx - (S)1 + mu;
        S r13 = sqrt(a * a + ry * ry + rz * rz);
        S r23 = sqrt(b * b + ry * ry + rz * rz);
        S c13 = r13 * (r13 * r13), c23 = r23 * (r23 * r23);
        dydt[0] = vx;
        dydt[1] = vy;
        dydt[2] = vz;
        dydt[3] = rx + (S)2 * vy - ((S)1 - mu) * (rx + mu) / c13 - mu * (rx - (S)1 + mu) / c23;
        dydt[4] = ry - (S)2 * vx - ((S)1 - mu) * ry / c13 - mu * ry / c23;
        dydt[5] = -((S)1 - mu) * rz / c13 - mu * rz / c23;
    }
};

}  // namespace degpu
