/*
 * degpu.h — C ABI of the GB300 ensemble explicit Runge–Kutta integrator.
 *
 * This is the drop-in boundary for the explicit Runge–Kutta path of the Rust crate
 * `differential-equations` v0.6.1.  One call solves many independent initial value problems
 * `dy/dt = f(t, y), y(t0) = y0` with RK4, DOPRI5 or DOP853, exactly as
 *
 *     IVP::ode(&system, t0, tf, y0)                         (src/ivp.rs:279)
 *        .method(ExplicitRungeKutta::dopri5().rtol(r).atol(a))  (src/ivp.rs:632, src/methods/erk/mod.rs:165-174)
 *        .t_eval(points)                                      (src/ivp.rs:656-660)
 *        .solve()                                             (src/ivp.rs:781-791 -> src/ode/solve_ivp.rs:116)
 *
 * would solve each of them, one instance at a time, on the CPU.
 *
 * Conventions
 *  - Plain C: pointers, sizes and POD structs only.  No exceptions cross the ABI.
 *  - Every array pointer in degpu_batch_in / degpu_batch_out is a DEVICE pointer for
 *    degpu_solve_ensemble and a HOST pointer for degpu_solve_ensemble_host.
 *  - State layout is structure-of-arrays: component c of instance i lives at [c * n + i].
 *    Dense output lives at [(e * d_max + c) * n + i] for evaluation point e.
 *  - The global return value says whether the call ran; per-instance failures are values in
 *    `status[i]`, mirroring `Error` (src/error.rs:13-40).  A failed instance never aborts the
 *    batch, exactly as one failed `solve()` does not affect another.
 *  - Calls are stream-ordered and asynchronous on `stream` (a cudaStream_t, NULL = default
 *    stream) unless the function says otherwise.
 */
#ifndef DEGPU_H
#define DEGPU_H

#if !defined(__CUDACC_RTC__)
#include <stddef.h>
#include <stdint.h>
#else
/* run-time compilation (NVRTC) has no C library headers */
typedef int int32_t;
typedef long long int64_t;
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Global status of a call. */
typedef enum {
    DEGPU_OK = 0,
    DEGPU_BAD_INPUT = 1,   /* a pointer, size or configuration value is invalid                */
    DEGPU_OOM = 2,         /* device memory could not be obtained                               */
    DEGPU_TIMEOUT = 3,     /* a bounded device-side wait gave up                                */
    DEGPU_CUDA_ERROR = 4,  /* a CUDA runtime / driver call failed                               */
    DEGPU_UNSUPPORTED = 5  /* the (method, family, precision, kernel) combination is not built */
} degpu_status;

/* Methods: constructors in src/methods/erk/fixed/mod.rs:69-75 (rk4),
 * src/methods/erk/dormandprince/mod.rs:45-58 (dop853, dopri5) and
 * src/methods/erk/adaptive/mod.rs:43-122 (the Adaptive family: embedded pair, infinity-norm
 * error, Stiffness after 100 consecutive rejections). rkf45 and cash_karp use cubic Hermite
 * dense output; Verner's pairs rkvPQRe (order P(Q), interpolant of order R; tableaus
 * src/tableau/verner.rs) evaluate extra stages on every accepted step and interpolate with
 * their own weights; rkv655e and rkv656e reuse their last stage (FSAL). */
typedef enum {
    DEGPU_RK4 = 0,
    DEGPU_DOPRI5 = 1,
    DEGPU_DOP853 = 2,
    DEGPU_RKF45 = 3,
    DEGPU_CASH_KARP = 4,
    DEGPU_RKV655E = 5,  /* 6(5), 9 stages + 1 dense stage   */
    DEGPU_RKV656E = 6,  /* 6(5), 9 stages + 3 dense stages  */
    DEGPU_RKV766E = 7,  /* 7(6), 10 stages + 3 dense stages */
    DEGPU_RKV767E = 8,  /* 7(6), 10 stages + 6 dense stages */
    DEGPU_RKV877E = 9,  /* 8(7), 13 stages + 4 dense stages */
    DEGPU_RKV878E = 10, /* 8(7), 13 stages + 8 dense stages */
    DEGPU_RKV988E = 11, /* 9(8), 16 stages + 5 dense stages */
    DEGPU_RKV989E = 12  /* 9(8), 16 stages + 10 dense stages */
} degpu_method;

/* Arithmetic of the solve.
 *  FP64_PARITY — every operation in the crate's order, no FMA contraction, correctly rounded
 *                pow/sin/cos: reproduces the crate's step counts and states bit for bit.
 *  FP64_FAST   — FP64 with FMA contraction and the fast CUDA math library.
 *  MIXED       — stage right-hand sides, stage combinations, the error norm, the step-size
 *                controller and the step size in FP32; y_{n+1} accumulated with Kahan
 *                compensation; t as an FP32 pair (about 48 bits, FP64 when output times,
 *                crossings or events need it; RK4: t and h in FP64).
 *                Instances whose rtol is below the method's mixed-precision bound
 *                (degpu_set_mixed_min_rtol) leave the FP32 stages: DOPRI5 and DOP853 on the Van
 *                der Pol, pendulum and Lorenz families and on FPU-beta chains run them with
 *                FP32-pair stages (about 48 bits: the state, stage states, right-hand sides and
 *                stage sums as unevaluated sums of two FP32 numbers, the step machinery as
 *                above), everything else in FP64_FAST.
 *  FP64_PLAIN  — FP64 with FMA contraction, refined hardware reciprocal and reciprocal square
 *                root, table-driven sin/cos (within one unit in the last place), and
 *                FP64_PARITY's correctly rounded controller power, so that every
 *                accept/reject decision follows the crate's unless contraction moves the error
 *                estimate across 1.  DOPRI5 and DOP853 on the Van der Pol, pendulum and Lorenz
 *                families, final states and output times.
 *  MIXED_FP64_CTRL — MIXED's FP32 stages and Kahan-compensated y, with the error norm, the
 *                controller's power, the accept decision and t in FP64 (the step size is an
 *                FP32 value, added to t in FP64).  Same families and methods as FP64_PLAIN, and
 *                the same mixed-precision bound as MIXED. */
typedef enum {
    DEGPU_FP64_PARITY = 0,
    DEGPU_FP64_FAST = 1,
    DEGPU_MIXED = 2,
    DEGPU_FP64_PLAIN = 3,
    DEGPU_MIXED_FP64_CTRL = 4
} degpu_precision;

/* Kernel layout. AUTO picks by method and dimension. */
typedef enum {
    DEGPU_KERNEL_AUTO = 0,
    DEGPU_KERNEL_THREAD = 1,      /* one system per thread, state and stages in registers          */
    DEGPU_KERNEL_WARP = 2,        /* one system per warp, lanes own components, stages in smem     */
    DEGPU_KERNEL_PERSISTENT = 3   /* persistent grid, device work queue, lane refill               */
} degpu_kernel;

/* DOP853 dense output: the crate's own fold (src/methods/erk/dormandprince/ordinary.rs:310-333)
 * or the published Hairer–Nørsett–Wanner continuous extension. */
typedef enum { DEGPU_DENSE_REFERENCE = 0, DEGPU_DENSE_HAIRER = 1 } degpu_dense_mode;

/* Per-instance result status; values mirror `Error` (src/error.rs:13-40). */
typedef enum {
    DEGPU_COMPLETE = 0,        /* Ok(Solution) with Status::Complete (src/ode/solve_ivp.rs:268-276) */
    DEGPU_ERR_BAD_INPUT = 1,   /* Error::BadInput  (src/utils.rs:60-157, src/ode/solve_ivp.rs:139-147) */
    DEGPU_ERR_MAX_STEPS = 2,   /* Error::MaxSteps  (dormandprince/ordinary.rs:82-92, fixed/ordinary.rs:64-75) */
    DEGPU_ERR_STEP_SIZE = 3,   /* Error::StepSize  (dormandprince/ordinary.rs:70-80)                   */
    DEGPU_ERR_STIFFNESS = 4,   /* Error::Stiffness (dormandprince/ordinary.rs:176-186)                 */
    DEGPU_INTERRUPTED = 5,     /* Ok(Solution) with Status::Interrupted: a terminal event stopped the
                                  solve (src/ode/solve_ivp.rs:254-259)                              */
    DEGPU_ERR_LINEAR_ALGEBRA = 6 /* Error::LinearAlgebra: a singular shooting Jacobian
                                    (src/methods/bvp/shooting/single.rs, lu_decomp)                 */
} degpu_instance_status;

/* Built-in right-hand sides (CUDA __device__ twins of `ODE::diff`, src/ode/ode.rs:20-44).
 * Parameters per instance are given in `params` as [p][n]. */
typedef enum {
    DEGPU_RHS_LORENZ = 1,       /* d=3, p=[sigma, rho, beta]        tests/ode/systems.rs:85-101   */
    DEGPU_RHS_VAN_DER_POL = 2,  /* d=2, p=[mu]                      tests/ode/systems.rs:66-78    */
    DEGPU_RHS_PENDULUM = 3,     /* d=2, p=[gamma, A, Omega]  damped driven pendulum, g/l = 1       */
    DEGPU_RHS_FPU_BETA = 4,     /* d=2m, p=[beta]  FPU-beta chain with fixed ends, y=[x_1..x_m,p_1..p_m] */
    DEGPU_RHS_EXP_GROWTH = 5,   /* d=1, p=[k]                       tests/ode/systems.rs:6-17     */
    DEGPU_RHS_LINEAR = 6,       /* d=1, p=[a, b]                    tests/ode/systems.rs:19-31    */
    DEGPU_RHS_HARMONIC = 7,     /* d=2, p=[k]                       tests/ode/systems.rs:33-46    */
    DEGPU_RHS_LOGISTIC = 8,     /* d=1, p=[k, m]                    tests/ode/systems.rs:48-60    */
    DEGPU_RHS_ROBERTSON = 9,    /* d=3, p=[]                        tests/ode/systems.rs:155-173  */
    DEGPU_RHS_HIRES = 10,       /* d=8, p=[]                        tests/ode/systems.rs:175-190  */
    DEGPU_RHS_BRUSSELATOR = 11, /* d=2, p=[a, b]                    tests/ode/systems.rs:103-120  */
    DEGPU_RHS_CR3BP = 12,       /* d=6, p=[mu]                      tests/ode/systems.rs:122-153  */
    DEGPU_RHS_PIPE_HEAT = 13,   /* d=2, p=[heat_loss_rate, ambient] tests/bvp/systems.rs:25-57    */
    DEGPU_RHS_DAMPED_QUADRATURE = 14, /* d=3, p=[k, m, c]  examples/ode/17_quadrature/main.rs:41-55 */
    DEGPU_RHS_NVRTC_BASE = 1000 /* ids >= this were returned by degpu_register_rhs_nvrtc          */
} degpu_rhs_id;

/* Solver settings: the fields and defaults of ExplicitRungeKutta (src/methods/erk/mod.rs:112-159)
 * and its builder setters (src/methods/erk/mod.rs:165-228).  `filter` is always the identity. */
typedef struct {
    int32_t method;        /* degpu_method                                                  */
    int32_t precision;     /* degpu_precision                                               */
    int32_t kernel;        /* degpu_kernel                                                  */
    int32_t dense_mode;    /* degpu_dense_mode                                              */
    double h0;             /* initial step; 0 = h_init heuristic (DP) or |tf-t0|/100 (RK4)  */
    double h_min;          /* default 0                                                     */
    double h_max;          /* default +inf                                                  */
    int64_t max_steps;     /* attempted-step cap, default 10 000                            */
    double safety_factor;  /* default 0.9                                                   */
    double min_scale;      /* default 0.2                                                   */
    double max_scale;      /* default 10                                                    */
} degpu_method_cfg;

/* The system being solved. */
typedef struct {
    int32_t rhs_id;    /* degpu_rhs_id for every instance (ignored when batch_in.family != NULL) */
    int32_t dim;       /* d, or the maximum d when batch_in.dims != NULL                         */
    int32_t n_params;  /* p                                                                      */
    int32_t reserved;
} degpu_problem;

typedef struct {
    int64_t n;               /* number of instances                                        */
    const double* t0;        /* [n]                                                          */
    const double* tf;        /* [n]                                                          */
    const double* y0;        /* [dim][n]                                                     */
    const double* params;    /* [n_params][n] (may be NULL when n_params == 0)               */
    const double* rtol;      /* [n] scalar Tolerance per instance (src/tolerance.rs:11-14)  */
    const double* atol;      /* [n]                                                          */
    const int32_t* dims;     /* [n] per-instance d (ragged ensembles) or NULL                */
    const int32_t* family;   /* [n] per-instance rhs id (mixed ensembles) or NULL            */
    const double* t_eval;    /* [n_eval] evaluation times shared by all instances, or NULL  */
    int32_t n_eval;          /* number of evaluation times (0 = no dense output)             */
    int32_t reserved;
    /* Per-component tolerances, Tolerance::Vector (src/tolerance.rs:11-14, indexed per component
     * by error_norm, src/traits.rs:394-410, and the initial step, src/methods/h_init.rs:76-82):
     * [dim][n], or NULL to use the scalar rtol[n] / atol[n].  Each may be given alone. */
    const double* rtol_vec;
    const double* atol_vec;
} degpu_batch_in;

typedef struct {
    double* y_final;     /* [dim][n] state at the end (or at the error, as Error{t, y} carries) */
    double* t_final;     /* [n]                                                                  */
    double* dense;       /* [n_eval][dim][n] or NULL; t_eval points the solve never reached stay NaN */
    int64_t* accepted;   /* [n] Steps.accepted (src/stats.rs, counted in src/ode/solve_ivp.rs:218-225) */
    int64_t* rejected;   /* [n] Steps.rejected                                                  */
    int64_t* fevals;     /* [n] Evals.function                                                  */
    int32_t* status;     /* [n] degpu_instance_status                                           */
} degpu_batch_out;

/* Fill `cfg` with the crate's defaults (src/methods/erk/mod.rs:112-159) for `method`. */
void degpu_default_cfg(degpu_method_cfg* cfg, int32_t method);

/* Mixed-precision bound of an adaptive method (no counterpart in the crate, which is FP64 only).
 * FP32 stage rounding puts a floor under the error: about 5e-7 relative on long Van der Pol
 * solves whatever the tolerance, and below rtol ~1e-9 the embedded error estimate stalls on the
 * noise and the controller keeps rejecting.  So in a DEGPU_MIXED solve an instance with
 * rtol < min_rtol leaves the FP32 stages: DOPRI5 (default bound 1e-6) and DOP853 (1e-7) run it
 * with FP32-pair stages, RKF45 and Cash-Karp (1e-9) in DEGPU_FP64_FAST arithmetic.  The choice
 * depends on the instance's own rtol only, so a result does not depend on the batch it is solved
 * in.  min_rtol = 0 disables the split.  RKF45 and Cash-Karp share one setting.  The setting is
 * process-wide and applies to solves launched after the call; the environment variable
 * DEGPU_MIXED_MIN_RTOL, read at the first solve, replaces every default.  RK4 (fixed step) has
 * no bound.  Returns DEGPU_BAD_INPUT for RK4, Verner's pairs, an unknown method, or a negative or
 * non-finite min_rtol. */
degpu_status degpu_set_mixed_min_rtol(int32_t method, double min_rtol);

/* The bound in force for `method` (0 for RK4 and unknown methods).  Verner's pairs return
 * +infinity: their stage sums carry coefficients up to 1.5e4, whose cancellation FP32 cannot
 * resolve, so a DEGPU_MIXED solve runs all their instances in DEGPU_FP64_FAST arithmetic. */
double degpu_mixed_min_rtol(int32_t method);

/* Dimension and parameter count of a built-in family (dim = -1 for variable-size families).
 * Returns DEGPU_BAD_INPUT for an unknown id. */
degpu_status degpu_rhs_info(int32_t rhs_id, int32_t* dim, int32_t* n_params);

/* Solve an ensemble, device pointers, stream-ordered.
 * Replaces, per instance i, `IVP::ode(&sys_i, t0[i], tf[i], y0_i).method(m).t_eval(t_eval).solve()`
 * (src/ivp.rs:279-791; src/ode/solve_ivp.rs:116-277).  Host-side validation of the arguments
 * happens before anything is launched; per-instance BadInput checks
 * (src/utils.rs:60-157, src/ode/solve_ivp.rs:139-147) are reported in status[i]. */
degpu_status degpu_solve_ensemble(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                  const degpu_batch_in* in, degpu_batch_out* out, void* stream);

/* Largest batch degpu_solve_ensemble_noalloc accepts. */
#define DEGPU_NOALLOC_MAX_INSTANCES 262144

/* degpu_solve_ensemble without any device memory allocation.  It has no counterpart in the
 * reference (the crate solves one problem per call on the CPU); it exists for callers that must
 * not allocate device memory while they run, such as an application that reserves the whole
 * device pool for itself at start-up or a latency-critical loop that cannot afford an allocator
 * call (cudaMalloc/cudaFree may synchronise the device).  The caller passes device inputs and
 * outputs as for degpu_solve_ensemble; the solve's work lists live in a fixed array of about
 * 4.2 MB inside the library (held by every GPU that loads it, until the process exits).
 *  - n must be <= DEGPU_NOALLOC_MAX_INSTANCES, otherwise DEGPU_BAD_INPUT and nothing runs.
 *  - The arguments are checked as degpu_solve_ensemble checks them (same DEGPU_BAD_INPUT cases).
 *  - Only the persistent solve of the Van der Pol, pendulum and Lorenz families, without dense
 *    output or per-instance dimensions (DEGPU_UNSUPPORTED otherwise).  With a device family map,
 *    dim and n_params must be >= 3 and out->status must be given; an instance of another family
 *    gets status BadInput and a NaN final state and time.
 *  - CUDA loads the library's device code, this array included, lazily: the first call on a
 *    device loads it there, and that is the one device allocation this entry point causes.
 *    Make that first call (any small batch) on each device before reserving the device's memory
 *    pool and before starting any stream capture; later calls allocate nothing.
 *  - Every call reuses the same array: calls that overlap on the GPU (other streams, other host
 *    threads) race and must be serialised by the caller. */
degpu_status degpu_solve_ensemble_noalloc(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                          const degpu_batch_in* in, degpu_batch_out* out, void* stream);

/* Same contract with HOST pointers: copies inputs to the device, solves, copies results back,
 * synchronizes.  This is the call a crate user's host code makes. */
degpu_status degpu_solve_ensemble_host(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                       const degpu_batch_in* in, degpu_batch_out* out);

/* Crossing detection: the crate's `.crossing(component, threshold, direction)` output
 * (CrossingSolout, src/solout/crossing.rs:200-330; IVP::crossing, src/ivp.rs:682-693).
 * After every accepted step, the sign of y[component] - threshold is compared with its value
 * at the previous step (the first value is taken at t0). On a change of sign that matches the
 * direction, the crossing time is located on the step's interpolant:
 *  - up to 10 Newton iterations with a finite-difference derivative;
 *  - the linear estimate between the two steps when those do not converge.
 * The time and the interpolated state are recorded. */
typedef enum { DEGPU_CROSS_BOTH = 0, DEGPU_CROSS_POSITIVE = 1, DEGPU_CROSS_NEGATIVE = -1 } degpu_crossing_direction;

typedef struct {
    int32_t component;   /* index of the monitored state component, 0 <= component < dim      */
    int32_t direction;   /* degpu_crossing_direction                                           */
    int32_t max_points;  /* capacity per instance of the outputs below (>= 0)                  */
    int32_t reserved;
    double threshold;
} degpu_crossing;

typedef struct {
    double* t;       /* [max_points][n] crossing times, in the order found; NaN past the count  */
    double* y;       /* [max_points][dim][n] interpolated states at those times                */
    int32_t* count;  /* [n] crossings found; can exceed max_points (the first ones are stored) */
} degpu_crossing_out;

/* degpu_solve_ensemble with crossing detection instead of output times (in->n_eval must be 0),
 * device pointers, stream-ordered. Built combinations (DEGPU_UNSUPPORTED otherwise):
 *  - RK4, DOPRI5, DOP853: Van der Pol, pendulum, Lorenz, harmonic oscillator, Brusselator, CR3BP,
 *    logistic and exponential growth, every precision;
 *  - RKF45, Cash-Karp: those eight families in FP64 parity; Van der Pol, pendulum and Lorenz in
 *    FP64 fast and mixed;
 *  - Verner's pairs: Van der Pol, pendulum, Lorenz and the harmonic oscillator in FP64 parity;
 *    the first three in FP64 fast and mixed (a mixed solve runs these pairs in FP64 fast).
 * The hyperplane and event entry points below build on the same kernels. */
degpu_status degpu_solve_ensemble_crossing(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                           const degpu_batch_in* in, const degpu_crossing* crossing,
                                           degpu_batch_out* out, degpu_crossing_out* crossing_out, void* stream);

/* Same with HOST pointers, synchronous (as degpu_solve_ensemble_host). */
degpu_status degpu_solve_ensemble_crossing_host(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                                const degpu_batch_in* in, const degpu_crossing* crossing,
                                                degpu_batch_out* out, degpu_crossing_out* crossing_out);

/* Hyperplane crossing detection: the crate's `.hyperplane_crossing(point, normal, extractor,
 * direction)` output (HyperplaneCrossingSolout, src/solout/hyperplane.rs; IVP::hyperplane_crossing,
 * src/ivp.rs:695-706). The extractor is a list of state components:
 * pos[j] = y[components[j]], j < dim. The monitored quantity is the signed distance
 * (pos - point) . normal, with the normal scaled to unit length when its norm exceeds the FP64
 * machine epsilon (as the crate's constructor does). Unlike component crossings, a step that
 * starts or ends exactly on the plane also counts as a crossing. The location search and the
 * outputs are those of degpu_solve_ensemble_crossing. */
#define DEGPU_HYPERPLANE_MAX_DIM 8

typedef struct {
    int32_t dim;         /* components extracted, 1 <= dim <= DEGPU_HYPERPLANE_MAX_DIM        */
    int32_t direction;   /* degpu_crossing_direction, on the signed distance                   */
    int32_t max_points;  /* capacity per instance of the outputs (>= 0)                        */
    int32_t reserved;
    int32_t components[DEGPU_HYPERPLANE_MAX_DIM]; /* extractor: state index of pos[j]          */
    double point[DEGPU_HYPERPLANE_MAX_DIM];       /* a point of the plane, in extracted space  */
    double normal[DEGPU_HYPERPLANE_MAX_DIM];      /* its normal (any length)                   */
} degpu_hyperplane;

/* degpu_solve_ensemble_crossing with a hyperplane instead of a component threshold; device
 * pointers, stream-ordered. Same families, methods and precisions. */
degpu_status degpu_solve_ensemble_hyperplane(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                             const degpu_batch_in* in, const degpu_hyperplane* plane,
                                             degpu_batch_out* out, degpu_crossing_out* crossing_out, void* stream);

/* Same with HOST pointers, synchronous. */
degpu_status degpu_solve_ensemble_hyperplane_host(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                                  const degpu_batch_in* in, const degpu_hyperplane* plane,
                                                  degpu_batch_out* out, degpu_crossing_out* crossing_out);

/* Event detection: the crate's `.event(&event)` (EventWrappedSolout, src/solout/event.rs:299-521;
 * IVP::event, src/ivp.rs:661-679). After every accepted step the event function g(t, y) at the
 * step's end is compared in sign with its previous value (the first value is taken at t0). On a
 * change of sign in `direction`, the event time is located by the crate's Brent–Dekker search on
 * the step's interpolant (at most 50 iterations, tolerance max(1e-14, 1e-12 |t|)). The event is
 * recorded unless it lies within 1e-14 of the last point of the crate's solution (the step's end
 * without output times, else the last output time or event), counted either way, and after
 * `terminate` counted events the instance stops with DEGPU_INTERRUPTED. The event functions are
 * the forms of the crate's examples and tests:
 *   DEGPU_EVENT_LINEAR   g = ((sum_j weights[j] y[components[j]]) + t_weight t) + offset
 *                        (e.g. `y[0] - 0.9 * m`, `t - 10.0`);
 *   DEGPU_EVENT_MAX_ABS  g = max_j |y[components[j]]| + offset
 *                        (e.g. `theta.abs().max(omega.abs()) - 0.01`). */
#define DEGPU_EVENT_MAX_TERMS 8
typedef enum { DEGPU_EVENT_LINEAR = 0, DEGPU_EVENT_MAX_ABS = 1 } degpu_event_kind;

typedef struct {
    int32_t kind;        /* degpu_event_kind                                                    */
    int32_t direction;   /* degpu_crossing_direction (EventConfig::direction)                   */
    int32_t terminate;   /* EventConfig::terminate: stop after this many events; 0 = never      */
    int32_t max_points;  /* capacity per instance of the event outputs (>= 0)                   */
    int32_t n_terms;     /* terms used: 0..8 for LINEAR, 1..8 for MAX_ABS                        */
    int32_t reserved;
    int32_t components[DEGPU_EVENT_MAX_TERMS]; /* state index of each term                      */
    double weights[DEGPU_EVENT_MAX_TERMS];     /* LINEAR: weight of each term                   */
    double t_weight;     /* LINEAR: weight of t                                                 */
    double offset;
} degpu_event;

/* degpu_solve_ensemble with event detection, device pointers, stream-ordered. Output times
 * (in->n_eval > 0) are the base output as in the crate (`.t_eval(..).event(..)`); the event
 * points go to event_out (laid out as degpu_crossing_out). Same families, methods and
 * precisions as degpu_solve_ensemble_crossing. */
degpu_status degpu_solve_ensemble_event(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                        const degpu_batch_in* in, const degpu_event* event, degpu_batch_out* out,
                                        degpu_crossing_out* event_out, void* stream);

/* Same with HOST pointers, synchronous. */
degpu_status degpu_solve_ensemble_event_host(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                             const degpu_batch_in* in, const degpu_event* event,
                                             degpu_batch_out* out, degpu_crossing_out* event_out);

/* Boundary value problems by shooting: the crate's `BVP::ode(&problem, t0, tf, y_guess)
 * .method(Shooting::single(erk) | Shooting::multiple(erk).segments(m)).solve()` (src/bvp.rs,
 * src/methods/bvp/shooting/{single,multiple}.rs) for every instance of a batch. Newton on the
 * shooting unknowns (the initial state; for multiple shooting the states at the m + 1 mesh nodes
 * t0 + (tf - t0) i / m) with a forward-difference Jacobian (step sqrt(eps) max(|u_j|, 1)) and the
 * crate's LU with partial pivoting; it stops when the residual's max norm is <= tolerance, then
 * solves the IVP from t0 with the converged initial state into the ordinary outputs (y_final =
 * y(tf), dense = the output times). Every IVP of every Newton iteration of the whole batch is one
 * ensemble solve on the device.
 * The boundary residual is r_i = y_side[component_i] - value_i (side 0: y(t0), 1: y(tf)), i < dim:
 * the form of every boundary function of the crate's tests and examples.
 * Per-instance status: COMPLETE; the status of a failing IVP; DEGPU_ERR_MAX_STEPS when Newton does
 * not converge in max_iterations; DEGPU_ERR_LINEAR_ALGEBRA for a singular Jacobian.
 * Multiple shooting needs one interval [t0, tf] for the whole batch. A DEGPU_MIXED configuration
 * runs its shots in DEGPU_FP64_FAST arithmetic: the Jacobian's perturbation (~1.5e-8 relative) is
 * below FP32 resolution. */
#define DEGPU_BVP_MAX_UNKNOWNS 64
typedef enum { DEGPU_BVP_SINGLE = 0, DEGPU_BVP_MULTIPLE = 1 } degpu_bvp_method;

typedef struct {
    int32_t method;          /* degpu_bvp_method                                               */
    int32_t segments;        /* multiple shooting: mesh segments m >= 1 (crate default 4)       */
    int32_t max_iterations;  /* Newton iterations (crate default 100)                          */
    int32_t reserved;
    double tolerance;        /* residual max-norm tolerance (crate default 1e-6)                */
    int32_t side[DEGPU_HYPERPLANE_MAX_DIM];      /* residual row i: 0 = y(t0), 1 = y(tf)       */
    int32_t component[DEGPU_HYPERPLANE_MAX_DIM]; /* state index of row i                       */
    double value[DEGPU_HYPERPLANE_MAX_DIM];      /* r_i = y_side[component] - value            */
} degpu_bvp;

typedef struct {
    double* y_a;          /* [dim][n] converged initial state (the solution's first point)     */
    int32_t* iterations;  /* [n] Newton iterations taken (Evals::newton)                        */
    int64_t* jacobian;    /* [n] Jacobian columns formed (Evals::jacobian)                      */
} degpu_bvp_out;

/* in->y0 holds the guesses; out->accepted / rejected / fevals receive the totals over every IVP
 * solved for the instance (the crate's Solution.steps / evals). HOST pointers, synchronous. */
degpu_status degpu_solve_bvp_host(const degpu_problem* problem, const degpu_method_cfg* cfg,
                                  const degpu_batch_in* in, const degpu_bvp* bvp, degpu_batch_out* out,
                                  degpu_bvp_out* bvp_out);

/* One evaluation of a built-in right-hand side for every instance (`ODE::diff`,
 * src/ode/ode.rs:20-44), device pointers: dydt[c*n+i] = f_i(t[i], y_i). */
degpu_status degpu_eval_rhs(int32_t rhs_id, int32_t precision, int64_t n, int32_t dim, int32_t n_params,
                            const double* t, const double* y, const double* params, double* dydt,
                            void* stream);

/* Register a right-hand side written as CUDA source and compiled at run time with NVRTC.
 * `source` must define
 *     template <class R> __device__ void <name>(R t, const R* y, R* dydt, const double* p);
 * (the shape of `ODE::diff(&self, t, &y, &mut dydt)`, src/ode/ode.rs:20-44, with the
 * system's fields passed as p[0..n_params)).  On success *rhs_id receives an id >= 1000
 * usable in degpu_problem.rhs_id.  Build log (on failure) goes to log[0..log_size). */
degpu_status degpu_register_rhs_nvrtc(const char* source, const char* name, int32_t dim, int32_t n_params,
                                      int32_t* rhs_id, char* log, size_t log_size);

/* Method-of-lines: 2-D Gray–Scott reaction–diffusion on a periodic nx*ny grid, advanced with
 * fixed-step RK4 (src/methods/erk/fixed/ordinary.rs:58-138) whose right-hand side is the
 * flux-form finite-difference semi-discretisation of src/pde/semi_discrete.rs:250-287 with a
 * periodic wrap.  u and v are [ny][nx] row-major device arrays, advanced in place by `steps`
 * steps of size dt.  precision: DEGPU_FP64_PARITY / DEGPU_FP64_FAST use the double arrays,
 * DEGPU_MIXED uses the float arrays (FP32 throughout). */
typedef struct {
    int32_t nx, ny;
    double dx;        /* grid spacing (both axes)           */
    double Du, Dv;    /* diffusivities                      */
    double F, k;      /* feed and kill rates                */
} degpu_gray_scott;

degpu_status degpu_gray_scott_rk4(const degpu_gray_scott* gs, int32_t precision, double t0, double dt,
                                  int64_t steps, void* u, void* v, void* stream);

/* One right-hand-side evaluation of the same semi-discretisation (u, v -> du, dv), FP64. */
degpu_status degpu_gray_scott_rhs(const degpu_gray_scott* gs, const double* u, const double* v,
                                  double* du, double* dv, void* stream);

/* Method of lines on a structured grid with the crate's faces: the semi-discretisation of
 * `MethodOfLines::finite_difference(grid).boundary(bc).discretize(&pde)` (SemiDiscretePde::diff,
 * src/pde/semi_discrete.rs:250-287; StructuredGrid, src/pde/grid.rs:23-145; BoundaryConditions,
 * src/pde/boundary.rs:11-94) for a built-in PDE, u_t = div(flux(t, x, u, grad u)) + source(t, x, u).
 * The state holds the fields of a node together, y[node * fields + c], node = i0 + nodes[0] i1
 * (axis 0 fastest), as the crate's Vec state does.  A node on a Dirichlet face has du/dt = 0.
 * A periodic face (not in the crate) wraps the neighbour around its axis; both faces of a
 * periodic axis must be periodic. */
#define DEGPU_MOL_MAX_FIELDS 4
#define DEGPU_MOL_MAX_PARAMS 8
typedef enum {
    DEGPU_PDE_DIFFUSION = 1,          /* flux_c = p[c] grad_c, no source; fields 1..4
                                         (HeatEquation, tests/pde/method_of_lines.rs:3-11)        */
    DEGPU_PDE_COUPLED_DIFFUSION = 2,  /* flux_c = p[c] grad_c, source (u1 - u0, u0 - u1); 2 fields
                                         (CoupledDiffusion, tests/pde/method_of_lines.rs:13-34)   */
    DEGPU_PDE_GRAY_SCOTT = 3          /* p = (Du, Dv, F, k); 2 fields (u, v)                    */
} degpu_pde_id;
typedef enum { DEGPU_BC_DIRICHLET = 0, DEGPU_BC_NEUMANN = 1, DEGPU_BC_PERIODIC = 2 } degpu_bc_kind;

typedef struct {
    int32_t pde_id;       /* degpu_pde_id                                                     */
    int32_t dims;         /* axes: 1 or 2                                                      */
    int32_t fields;       /* values per node (the PDE's local state length)                    */
    int32_t reserved;
    int32_t nodes[2];     /* nodes per axis (>= 2; nodes[1] ignored for one axis)              */
    double lower[2];      /* grid origin (StructuredGrid::uniform's lower corner)              */
    double dx[2];         /* node spacing per axis ((upper - lower) / (nodes - 1) for uniform) */
    int32_t bc_kind[2][2];   /* [axis][0 lower, 1 upper]: degpu_bc_kind                        */
    double bc_value[2][2][DEGPU_MOL_MAX_FIELDS]; /* Dirichlet value or Neumann gradient per field */
    double params[DEGPU_MOL_MAX_PARAMS];          /* the PDE's parameters                        */
} degpu_mol;

/* dydt = f(t, y), the semi-discrete right-hand side, on device arrays of nodes * fields values:
 * double for DEGPU_FP64_PARITY (the crate's operation order bit for bit), DEGPU_FP64_FAST and
 * DEGPU_FP64_PLAIN (FMA contraction); float for DEGPU_MIXED. */
degpu_status degpu_mol_rhs(const degpu_mol* mol, int32_t precision, double t, const void* y, void* dydt,
                           void* stream);

/* `IVP::pde(..).space(..).method(ExplicitRungeKutta::rk4(h)).solve()` from t0 to tf: the crate's
 * fixed RK4 steps (src/methods/erk/fixed/ordinary.rs:58-138) under its driver loop
 * (src/ode/solve_ivp.rs:138-277: the last step is shortened to end at tf), y advanced in place.
 * *steps receives the number of steps taken.  Precision as degpu_mol_rhs. */
degpu_status degpu_mol_rk4(const degpu_mol* mol, int32_t precision, double t0, double tf, double h, void* y,
                           int64_t* steps, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Serving: continuous batching of ensemble solves.
 *
 * The crate solves one IVP per call, synchronously (src/ivp.rs:781-791); a server built on it
 * would queue whole solves.  Here requests (each an ensemble, as degpu_solve_ensemble_host takes
 * it) are admitted as device memory frees up, under a memory budget, in arrival order; every
 * admitted request keeps its instances' solver state (t, h, y, derivative, counters, controller
 * state) resident on the device and advances in bounded rounds of a persistent kernel on its own
 * stream, so requests that arrive while others run join at the next round and their work overlaps
 * on the GPU.  A request's results do not depend on what else is in flight.
 * --------------------------------------------------------------------------------------------- */
typedef struct degpu_server degpu_server;

typedef struct {
    uint64_t memory_budget_bytes;  /* device memory admitted requests may hold (0 = 150 GB)          */
    int32_t max_active;            /* requests resident at once (0 = 64)                             */
    int32_t round_budget;          /* driver iterations per instance per round (0 = 512)             */
} degpu_server_cfg;

/* Start a server (a scheduler thread on the current device). */
degpu_status degpu_server_create(const degpu_server_cfg* cfg, degpu_server** server);

/* Queue a request.  `in` and `out` are HOST pointers that must stay valid until the request is
 * done; the call copies nothing yet and returns at once with the request's id. */
degpu_status degpu_server_submit(degpu_server* server, const degpu_problem* problem, const degpu_method_cfg* cfg,
                                 const degpu_batch_in* in, degpu_batch_out* out, uint64_t* request_id);

/* Non-blocking: *done = 1 once the outputs are in `out`; *latency_ms = submit-to-done time.
 * The return value is the request's own status (DEGPU_OK, or why it failed) once done. */
degpu_status degpu_server_poll(degpu_server* server, uint64_t request_id, int32_t* done, double* latency_ms);

/* Block until the request is done. */
degpu_status degpu_server_wait(degpu_server* server, uint64_t request_id, double* latency_ms);

/* Drain every queued and running request, stop the scheduler and release the device memory. */
degpu_status degpu_server_destroy(degpu_server* server);

/* Human-readable message for a status. */
const char* degpu_status_string(degpu_status s);

/* Library version string. */
const char* degpu_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DEGPU_H */
