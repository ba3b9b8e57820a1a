// degpu_abi.cu — the extern "C" boundary (include/degpu.h) over the ensemble kernels.
//
// Host-side responsibilities, before any launch:
//  - argument validation (null pointers, sizes, enum ranges) -> DEGPU_BAD_INPUT;
//  - TEvalSolout::new's sort of the requested times (src/solout/t_eval.rs:154-171), done once
//    for the batch, with the permutation back to the caller's order;
//  - grouping of a mixed-family batch into one work list per family, and of a mixed-precision
//    batch into FP32-stage and FP64 lists by the instances' rtol (degpu_set_mixed_min_rtol);
//  - choice of the kernel layout.
// Per-instance checks (BadInput of src/utils.rs:60-157) run on the device and are reported in
// status[i].
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <vector>

#include "registry.cuh"
#include "side_paths.cuh"

namespace degpu {

std::map<VariantKey, EnsLaunchFn>& ens_registry() {
    static std::map<VariantKey, EnsLaunchFn> m;
    return m;
}
std::map<VariantKey, EnsLaunchFn>& cross_registry() {
    static std::map<VariantKey, EnsLaunchFn> m;
    return m;
}
std::map<VariantKey, RoundOps>& round_registry() {
    static std::map<VariantKey, RoundOps> m;
    return m;
}
std::map<std::pair<int, int>, RhsLaunchFn>& rhs_registry() {
    static std::map<std::pair<int, int>, RhsLaunchFn> m;
    return m;
}

int device_sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

void ensure_registered() {
    static std::once_flag once;
    std::call_once(once, []() {
        register_parity_main();
        register_parity_tests();
        register_fast();
        register_mixed();
        register_parity_multi();
        register_multi_fast_mixed();
        register_multi_cross();
        register_multi_embedded();
        register_cross_parity();
        register_cross_fast_mixed();
        register_cross_embedded_parity();
        register_cross_embedded_fast_mixed();
        register_embedded_parity();
        register_embedded_fast_mixed();
        register_verner65_parity();
        register_verner76_parity();
        register_verner87_parity();
        register_verner98_parity();
        register_verner65_fast();
        register_verner76_fast();
        register_verner87_fast();
        register_verner98_fast();
        register_verner_cross65_parity();
        register_verner_cross76_parity();
        register_verner_cross87_parity();
        register_verner_cross98_parity();
        register_verner_cross6576_fast();
        register_verner_cross8798_fast();
        register_plain();
        register_mixed_f64ctrl();
        register_mixed_pair();
        register_round_dense_parity();
        register_round_dense_fast_mixed();
        register_groups();
        register_mixed_pair853();
    });
}

// Stream-ordered scratch allocations released at the end of a call.
struct Scratch {
    cudaStream_t s;
    std::vector<void*> ptrs;
    explicit Scratch(cudaStream_t st) : s(st) {}
    template <class T>
    T* alloc(size_t count) {
        void* p = nullptr;
        if (count == 0) count = 1;
        if (cudaMallocAsync(&p, count * sizeof(T), s) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (T*)p;
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
    }
};

static bool valid_method(int m) { return m >= DEGPU_RK4 && m <= DEGPU_RKV989E; }

// Slot of the mixed-precision bound a method uses: DOPRI5, DOP853, or the other order-5 pairs.
static int bound_slot(int m) { return m == DEGPU_DOPRI5 ? 0 : (m == DEGPU_DOP853 ? 1 : 2); }

// Mixed-precision bounds, by slot (DOPRI5, DOP853, RKF45 / Cash-Karp): the rtol below which an
// instance of a mixed solve leaves the FP32 stages.
//  - DOPRI5 1e-6, and below it FP32-pair stages.  FP32 stage rounding puts a floor of about 5e-7
//    (Van der Pol) under the error against an rtol = atol = 1e-13 solution, whatever the
//    tolerance; measured per rtol decade on the uneven Van der Pol / pendulum / Lorenz ensemble,
//    the FP32 stages match FP64's error at rtol >= 1e-6 (Van der Pol median 1.26e-5 against
//    1.16e-5, pendulum 5.2e-6 against 6.0e-6) and miss it below (1e-7..1e-6: 1.7e-6 against 1.0e-6;
//    1e-9..1e-8: 5.2e-7 against 6.1e-9).  Pair stages carry 48 bits.
//  - DOP853 1e-7 and RKF45 / Cash-Karp 1e-9, and below them FP64.  Below the FP32 rounding level
//    of the stage states the error estimate has a noise floor and the step count climbs
//    (FP32-stage steps / FP64 steps, share of instances ending in MaxSteps at the crate's
//    10 000-step cap): DOPRI5 1e-8: 1.03-1.18x, none; 1e-9: 1.6-3.2x, up to 39%; 1e-10: 1.7-11x,
//    53-96%; DOP853 1e-7: 1.14-1.46x, none; 1e-8: 4.8-21x, up to 53%.
static constexpr double MIXED_MIN_RTOL[3] = {1e-6, 1e-7, 1e-9};

static std::atomic<double>& mixed_bound(int slot) {
    static std::atomic<double> b[3];
    static std::once_flag once;
    std::call_once(once, []() {
        double v[3] = {MIXED_MIN_RTOL[0], MIXED_MIN_RTOL[1], MIXED_MIN_RTOL[2]};
        if (const char* e = getenv("DEGPU_MIXED_MIN_RTOL")) {
            char* end = nullptr;
            double x = strtod(e, &end);
            if (end != e && std::isfinite(x) && x >= 0.0) v[0] = v[1] = v[2] = x;
        }
        for (int q = 0; q < 3; ++q) b[q].store(v[q]);
    });
    return b[slot];
}

double mixed_split(const degpu_method_cfg* cfg) {
    if (!(cfg->precision == DEGPU_MIXED || cfg->precision == DEGPU_MIXED_FP64_CTRL) || cfg->method == DEGPU_RK4)
        return 0.0;
    // Verner's pairs: their stage sums carry coefficients up to 1.5e4 (RKV877e), whose
    // cancellation FP32 cannot resolve, so every instance of a mixed solve runs in FP64
    if (cfg->method >= DEGPU_RKV655E) return INFINITY;
    return mixed_bound(bound_slot(cfg->method)).load();
}

int mixed_low_precision(const degpu_method_cfg* cfg) {
    const bool mixed = cfg->precision == DEGPU_MIXED || cfg->precision == DEGPU_MIXED_FP64_CTRL;
    return (mixed && (cfg->method == DEGPU_DOPRI5 || cfg->method == DEGPU_DOP853)) ? PrecMixedPair::ID
                                                                                 : DEGPU_FP64_FAST;
}

static bool valid_prec(int p) { return p >= DEGPU_FP64_PARITY && p <= DEGPU_MIXED_FP64_CTRL; }

static void builtin_info(int id, int& dim, int& np) {
    switch (id) {
        case DEGPU_RHS_LORENZ: dim = 3; np = 3; return;
        case DEGPU_RHS_VAN_DER_POL: dim = 2; np = 1; return;
        case DEGPU_RHS_PENDULUM: dim = 2; np = 3; return;
        case DEGPU_RHS_FPU_BETA: dim = -1; np = 1; return;
        case DEGPU_RHS_EXP_GROWTH: dim = 1; np = 1; return;
        case DEGPU_RHS_LINEAR: dim = 1; np = 2; return;
        case DEGPU_RHS_HARMONIC: dim = 2; np = 1; return;
        case DEGPU_RHS_LOGISTIC: dim = 1; np = 2; return;
        case DEGPU_RHS_ROBERTSON: dim = 3; np = 0; return;
        case DEGPU_RHS_HIRES: dim = 8; np = 0; return;
        case DEGPU_RHS_BRUSSELATOR: dim = 2; np = 2; return;
        case DEGPU_RHS_CR3BP: dim = 6; np = 1; return;
        case DEGPU_RHS_PIPE_HEAT: dim = 2; np = 2; return;
        case DEGPU_RHS_DAMPED_QUADRATURE: dim = 3; np = 3; return;
        default: dim = 0; np = -1; return;
    }
}

// Kernel arguments of a solve: inputs, outputs and settings (no work list yet).
static EnsArgs make_args(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                         degpu_batch_out* out) {
    EnsArgs a{};
    a.n = in->n;
    a.t0 = in->t0;
    a.tf = in->tf;
    a.y0 = in->y0;
    a.params = in->params;
    a.rtol = in->rtol;
    a.atol = in->atol;
    a.rtol_vec = in->rtol_vec;
    a.atol_vec = in->atol_vec;
    a.n_eval = (in->n_eval > 0 && in->t_eval) ? in->n_eval : 0;
    a.dmax = pb->dim;
    a.y_final = out->y_final;
    a.t_final = out->t_final;
    a.dense = out->dense;
    a.accepted = out->accepted;
    a.rejected = out->rejected;
    a.fevals = out->fevals;
    a.status = out->status;
    a.h0 = cfg->h0;
    a.h_min = cfg->h_min;
    a.h_max = cfg->h_max;
    a.max_steps = cfg->max_steps;
    a.safety = cfg->safety_factor;
    a.min_scale = cfg->min_scale;
    a.max_scale = cfg->max_scale;
    a.safety_f = (float)a.safety;
    a.min_scale_f = (float)a.min_scale;
    a.max_scale_f = (float)a.max_scale;
    a.dense_mode = cfg->dense_mode;
    a.n_params = pb->n_params;
    return a;
}

// The requested output times: TEvalSolout::new's stable ascending sort (descending instances walk
// it backwards), uploaded with its permutation; every output starts as NaN, so points the solve
// never reaches stay NaN. Without a dense output array there are no output times.
static degpu_status prepare_t_eval(EnsArgs& a, const degpu_problem* pb, const degpu_batch_in* in,
                                   degpu_batch_out* out, const double* t_eval_host, Scratch& scratch,
                                   cudaStream_t s) {
    if (a.n_eval > 0 && !out->dense) a.n_eval = 0;
    if (a.n_eval == 0) return DEGPU_OK;
    std::vector<int32_t> perm(a.n_eval);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int32_t x, int32_t y) { return t_eval_host[x] < t_eval_host[y]; });
    std::vector<double> sorted(a.n_eval);
    for (int e = 0; e < a.n_eval; ++e) sorted[e] = t_eval_host[perm[e]];
    double* d_t = scratch.alloc<double>(a.n_eval);
    int32_t* d_p = scratch.alloc<int32_t>(a.n_eval);
    if (!d_t || !d_p) return DEGPU_OOM;
    if (cudaMemcpyAsync(d_t, sorted.data(), a.n_eval * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(d_p, perm.data(), a.n_eval * sizeof(int32_t), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return DEGPU_CUDA_ERROR;
    a.t_eval = d_t;
    a.eval_perm = d_p;
    // the host vectors must outlive the async copies
    if (cudaStreamSynchronize(s) != cudaSuccess) return DEGPU_CUDA_ERROR;
    // 0xFF bytes form a quiet NaN
    const size_t bytes = (size_t)in->n_eval * pb->dim * in->n * sizeof(double);
    if (cudaMemsetAsync(out->dense, 0xFF, bytes, s) != cudaSuccess) return DEGPU_CUDA_ERROR;
    return DEGPU_OK;
}

// Core of degpu_solve_ensemble.  `family_host` / `t_eval_host` are host copies of the
// corresponding device arrays (or NULL when absent).
static degpu_status solve_impl(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                               degpu_batch_out* out, cudaStream_t s, const int32_t* family_host,
                               const double* t_eval_host, const int32_t* dims_host) {
    ensure_registered();
    const int64_t n = in->n;
    if (n == 0) return DEGPU_OK;
    Scratch scratch(s);

    EnsArgs a = make_args(pb, cfg, in, out);
    {
        degpu_status st = prepare_t_eval(a, pb, in, out, t_eval_host, scratch, s);
        if (st != DEGPU_OK) return st;
    }
    const bool dense = a.n_eval > 0;

    // ragged (per-instance dimension) problems go to the warp-per-system kernel
    if (pb->rhs_id == DEGPU_RHS_FPU_BETA) {
        return group_solve(pb, cfg, a, in->dims, s);
    }

    int kernel_sel = cfg->kernel;
    if (kernel_sel == DEGPU_KERNEL_AUTO)
        kernel_sel = (cfg->method != DEGPU_RK4 && n >= 32768) ? DEGPU_KERNEL_PERSISTENT : DEGPU_KERNEL_THREAD;

    // solves of the production families (Van der Pol, pendulum, Lorenz) run over longest-first
    // work lists: one multi-family persistent launch, or one run-to-completion launch per list
    {
        auto prod = [](int id) {
            return id == DEGPU_RHS_VAN_DER_POL || id == DEGPU_RHS_PENDULUM || id == DEGPU_RHS_LORENZ;
        };
        bool seen[3] = {false, false, false};
        bool ok = true;
        auto note = [&](int id) {
            if (!prod(id)) ok = false;
            else seen[id == DEGPU_RHS_VAN_DER_POL ? 0 : id == DEGPU_RHS_PENDULUM ? 1 : 2] = true;
        };
        if (family_host) {
            for (int64_t i = 0; i < n && ok; ++i) note(family_host[i]);
        } else {
            note(pb->rhs_id);
        }
        const int ids[3] = {DEGPU_RHS_VAN_DER_POL, DEGPU_RHS_PENDULUM, DEGPU_RHS_LORENZ};
        for (int f = 0; f < 3 && ok; ++f) {
            if (!seen[f]) continue;
            int dim, np;
            builtin_info(ids[f], dim, np);
            if (dim > pb->dim || np > pb->n_params) return DEGPU_BAD_INPUT;
        }
        if (ok) {
            EnsArgs ma = a;
            ma.count = n;
            const int32_t* fam_dev = family_host ? in->family : nullptr;
            if (kernel_sel == DEGPU_KERNEL_PERSISTENT && multi_registry().count({cfg->method, cfg->precision, dense ? 1 : 0}))
                return multi_solve(cfg, ma, fam_dev, pb->rhs_id, dense, s);
            return sorted_thread_solve(cfg, ma, fam_dev, pb->rhs_id, dense, s);
        }
    }

    // work lists per (family, precision): a mixed solve sends instances with rtol below the
    // mixed-precision bound to the FP64_FAST variant
    struct WorkList {
        int family, precision;
        bool all;  // every instance of the batch, no index list
        std::vector<int64_t> idx;
    };
    std::vector<WorkList> groups;
    const double split = mixed_split(cfg);
    std::vector<double> rtol_host;
    if (split > 0.0) {
        rtol_host.resize(n);
        if (cudaMemcpyAsync(rtol_host.data(), in->rtol, n * sizeof(double), cudaMemcpyDeviceToHost, s) !=
                cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return DEGPU_CUDA_ERROR;
    }
    if (family_host || split > 0.0) {
        std::map<std::pair<int, int>, std::vector<int64_t>> by;
        for (int64_t i = 0; i < n; ++i) {
            const int fam = family_host ? family_host[i] : pb->rhs_id;
            int prec = cfg->precision;
            if (split > 0.0 && rtol_host[i] < split) {
                prec = mixed_low_precision(cfg);
                if (!ens_registry().count(VariantKey{cfg->method, fam, prec, dense ? 1 : 0})) prec = DEGPU_FP64_FAST;
            }
            by[{fam, prec}].push_back(i);
        }
        for (auto& kv : by) groups.push_back(WorkList{kv.first.first, kv.first.second, false, std::move(kv.second)});
    } else {
        groups.push_back(WorkList{pb->rhs_id, cfg->precision, true, {}});
    }

    int kernel = cfg->kernel;
    if (kernel == DEGPU_KERNEL_AUTO) kernel = (cfg->method != DEGPU_RK4 && n >= 32768) ? DEGPU_KERNEL_PERSISTENT
                                                                                        : DEGPU_KERNEL_THREAD;
    if (kernel == DEGPU_KERNEL_WARP) kernel = DEGPU_KERNEL_THREAD;  // fixed-size families: one system per thread

    for (auto& g : groups) {
        int dim, np;
        builtin_info(g.family, dim, np);
        if (np < 0) return DEGPU_BAD_INPUT;
        if (dim > pb->dim || np > pb->n_params) return DEGPU_BAD_INPUT;
        auto it = ens_registry().find(VariantKey{cfg->method, g.family, g.precision, dense ? 1 : 0});
        if (it == ens_registry().end()) return DEGPU_UNSUPPORTED;
        EnsArgs ga = a;
        if (!g.all) {
            int64_t* d_idx = scratch.alloc<int64_t>(g.idx.size());
            if (!d_idx) return DEGPU_OOM;
            if (cudaMemcpyAsync(d_idx, g.idx.data(), g.idx.size() * sizeof(int64_t), cudaMemcpyHostToDevice, s) !=
                cudaSuccess)
                return DEGPU_CUDA_ERROR;
            ga.index = d_idx;
            ga.count = (int64_t)g.idx.size();
        } else {
            ga.index = nullptr;
            ga.count = n;
        }
        if (kernel == DEGPU_KERNEL_PERSISTENT) {
            unsigned long long* tk = scratch.alloc<unsigned long long>(1);
            if (!tk) return DEGPU_OOM;
            if (cudaMemsetAsync(tk, 0, sizeof(unsigned long long), s) != cudaSuccess) return DEGPU_CUDA_ERROR;
            ga.ticket = tk;
        }
        cudaError_t e = it->second(ga, kernel, s);
        if (e != cudaSuccess) return DEGPU_CUDA_ERROR;
    }
    if (!(groups.size() == 1 && groups[0].all)) {
        // index lists were copied from host vectors that die with this call
        if (cudaStreamSynchronize(s) != cudaSuccess) return DEGPU_CUDA_ERROR;
    }
    return DEGPU_OK;
}

degpu_status validate_solve_args(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                 const degpu_batch_out* out) {
    if (!pb || !cfg || !in || !out) return DEGPU_BAD_INPUT;
    if (in->n < 0) return DEGPU_BAD_INPUT;
    if (in->n == 0) return DEGPU_OK;
    if (!valid_method(cfg->method) || !valid_prec(cfg->precision)) return DEGPU_BAD_INPUT;
    if (cfg->kernel < DEGPU_KERNEL_AUTO || cfg->kernel > DEGPU_KERNEL_PERSISTENT) return DEGPU_BAD_INPUT;
    if (pb->dim <= 0 || pb->n_params < 0) return DEGPU_BAD_INPUT;
    if (!in->t0 || !in->tf || !in->y0 || !in->rtol || !in->atol) return DEGPU_BAD_INPUT;
    if (pb->n_params > 0 && !in->params) return DEGPU_BAD_INPUT;
    if (!out->y_final) return DEGPU_BAD_INPUT;
    if (in->n_eval < 0 || (in->n_eval > 0 && !in->t_eval)) return DEGPU_BAD_INPUT;
    if (cfg->max_steps < 0) return DEGPU_BAD_INPUT;
    if (!in->family) {
        int dim, np;
        builtin_info(pb->rhs_id, dim, np);
        if (np < 0 && pb->rhs_id >= DEGPU_RHS_NVRTC_BASE) {
            int32_t d32 = 0, p32 = 0;
            if (nvrtc_rhs_info(pb->rhs_id, &d32, &p32) != DEGPU_OK) return DEGPU_BAD_INPUT;
            dim = d32;
            np = p32;
        }
        if (np < 0) return DEGPU_BAD_INPUT;
        if (dim > 0 && dim != pb->dim) return DEGPU_BAD_INPUT;
        if (np > pb->n_params) return DEGPU_BAD_INPUT;
        if (dim < 0 && !in->dims) return DEGPU_BAD_INPUT;
    }
    return DEGPU_OK;
}

// What a crossing- or event-detection solve monitors: a component against a threshold
// (degpu_crossing, mode 0), the signed distance to a hyperplane (degpu_hyperplane, mode 1) or an
// event function (degpu_event, mode 2).
struct CrossSpec {
    int32_t mode = 0, comp = 0, dir = 0, max_points = 0;
    double value = 0.0;  // threshold; plane: sum |point_j normal_j|; event: offset
    int32_t dim = 0;     // terms
    int32_t comps[DEGPU_HYPERPLANE_MAX_DIM] = {};
    double point[DEGPU_HYPERPLANE_MAX_DIM] = {}, normal[DEGPU_HYPERPLANE_MAX_DIM] = {};  // event: weights in normal
    int32_t event_kind = 0, terminate = 0;
    double t_weight = 0.0;
    int32_t max_comp = 0;  // largest state index read
};

static bool make_spec(const degpu_crossing* cr, int32_t dim, CrossSpec& sp) {
    if (cr->component < 0 || cr->component >= dim || cr->max_points < 0) return false;
    if (cr->direction < -1 || cr->direction > 1) return false;
    sp.comp = sp.max_comp = cr->component;
    sp.dir = cr->direction;
    sp.max_points = cr->max_points;
    sp.value = cr->threshold;
    return true;
}

// HyperplaneCrossingSolout::new (src/solout/hyperplane.rs): the normal is scaled by 1/|normal|
// when |normal| exceeds the FP64 epsilon, |normal|^2 folded from zero in component order
// (src/traits.rs:574-576). Host code is compiled without multiply-add contraction, so the scaled
// normal is the crate's to the bit.
static bool make_spec(const degpu_hyperplane* hp, int32_t dim, CrossSpec& sp) {
    if (hp->dim < 1 || hp->dim > DEGPU_HYPERPLANE_MAX_DIM || hp->max_points < 0) return false;
    if (hp->direction < -1 || hp->direction > 1) return false;
    sp.mode = 1;
    sp.dir = hp->direction;
    sp.max_points = hp->max_points;
    sp.dim = hp->dim;
    double nn = 0.0;
    for (int j = 0; j < hp->dim; ++j) {
        if (hp->components[j] < 0 || hp->components[j] >= dim) return false;
        sp.comps[j] = hp->components[j];
        sp.max_comp = std::max(sp.max_comp, hp->components[j]);
        sp.point[j] = hp->point[j];
        sp.normal[j] = hp->normal[j];
        const double sq = hp->normal[j] * hp->normal[j];
        nn = nn + sq;
    }
    const double norm = std::sqrt(nn);
    if (norm > 2.220446049250313e-16) {
        const double inv = 1.0 / norm;
        for (int j = 0; j < hp->dim; ++j) sp.normal[j] = sp.normal[j] * inv;
    }
    double scale = 0.0;
    for (int j = 0; j < hp->dim; ++j) scale += std::fabs(sp.point[j] * sp.normal[j]);
    sp.value = scale;
    return true;
}

// EventWrappedSolout's event (src/solout/event.rs:299-521) in one of the two built-in forms.
static bool make_spec(const degpu_event* ev, int32_t dim, CrossSpec& sp) {
    if (ev->kind != DEGPU_EVENT_LINEAR && ev->kind != DEGPU_EVENT_MAX_ABS) return false;
    const int32_t min_terms = ev->kind == DEGPU_EVENT_MAX_ABS ? 1 : 0;
    if (ev->n_terms < min_terms || ev->n_terms > DEGPU_EVENT_MAX_TERMS) return false;
    if (ev->max_points < 0 || ev->terminate < 0 || ev->direction < -1 || ev->direction > 1) return false;
    sp.mode = 2;
    sp.dir = ev->direction;
    sp.max_points = ev->max_points;
    sp.dim = ev->n_terms;
    sp.event_kind = ev->kind;
    sp.terminate = ev->terminate;
    sp.t_weight = ev->t_weight;
    sp.value = ev->offset;
    for (int j = 0; j < ev->n_terms; ++j) {
        if (ev->components[j] < 0 || ev->components[j] >= dim) return false;
        sp.comps[j] = ev->components[j];
        sp.max_comp = std::max(sp.max_comp, ev->components[j]);
        sp.normal[j] = ev->weights[j];
    }
    return true;
}

// degpu_solve_ensemble_crossing / _hyperplane / _event: one run-to-completion detection launch
// per (family, precision) work list.
static degpu_status crossing_impl(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                  const CrossSpec& cr, degpu_batch_out* out, degpu_crossing_out* co,
                                  const double* t_eval_host, cudaStream_t s) {
    const int64_t n = in->n;
    Scratch scratch(s);
    std::vector<int32_t> fam_host;
    if (in->family) {
        fam_host.resize(n);
        if (cudaMemcpyAsync(fam_host.data(), in->family, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s) !=
                cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return DEGPU_CUDA_ERROR;
    }
    const double split = mixed_split(cfg);
    std::vector<double> rtol_host;
    if (split > 0.0) {
        rtol_host.resize(n);
        if (cudaMemcpyAsync(rtol_host.data(), in->rtol, n * sizeof(double), cudaMemcpyDeviceToHost, s) !=
                cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return DEGPU_CUDA_ERROR;
    }
    std::map<std::pair<int, int>, std::vector<int64_t>> lists;
    for (int64_t i = 0; i < n; ++i) {
        const int fam = in->family ? fam_host[i] : pb->rhs_id;
        int prec = cfg->precision;
        if (split > 0.0 && rtol_host[i] < split) {
            // the tight class: FP32-pair stages where built for this family, else FP64 fast
            prec = mixed_low_precision(cfg);
            if (!cross_registry().count(VariantKey{cfg->method, fam, prec, 1})) prec = DEGPU_FP64_FAST;
        }
        lists[{fam, prec}].push_back(i);
    }
    for (auto& kv : lists) {
        int dim, np;
        builtin_info(kv.first.first, dim, np);
        if (np < 0 || dim > pb->dim || np > pb->n_params || cr.max_comp >= dim) return DEGPU_BAD_INPUT;
        if (cross_registry().find(VariantKey{cfg->method, kv.first.first, kv.first.second, 1}) ==
            cross_registry().end())
            return DEGPU_UNSUPPORTED;
    }
    EnsArgs a = make_args(pb, cfg, in, out);
    if (cr.mode == 2) {  // events keep the output times as their base output
        degpu_status st = prepare_t_eval(a, pb, in, out, t_eval_host, scratch, s);
        if (st != DEGPU_OK) return st;
    } else {
        a.n_eval = 0;
    }
    a.cross_comp = cr.comp;
    a.cross_dir = cr.dir;
    a.cross_max = cr.max_points;
    a.cross_value = cr.value;
    a.cross_t = co->t;
    a.cross_y = co->y;
    a.cross_count = co->count;
    a.cross_mode = cr.mode;
    a.n_terms = cr.dim;
    a.event_kind = cr.event_kind;
    a.event_terminate = cr.terminate;
    a.event_tw = cr.t_weight;
    a.cross_value_f = (float)cr.value;
    a.event_tw_f = (float)cr.t_weight;
    for (int j = 0; j < DEGPU_HYPERPLANE_MAX_DIM; ++j) {
        a.term_comp[j] = cr.comps[j];
        a.term_a[j] = cr.point[j];
        a.term_w[j] = cr.normal[j];
        a.term_a_f[j] = (float)cr.point[j];
        a.term_w_f[j] = (float)cr.normal[j];
    }
    if (cr.max_points > 0) {
        // 0xFF bytes form a quiet NaN: slots past an instance's count stay NaN
        const size_t m = (size_t)cr.max_points * n;
        if (cudaMemsetAsync(co->t, 0xFF, m * sizeof(double), s) != cudaSuccess ||
            cudaMemsetAsync(co->y, 0xFF, m * pb->dim * sizeof(double), s) != cudaSuccess)
            return DEGPU_CUDA_ERROR;
    }
    // the production families go through the longest-first plan lists (lanes of a warp get
    // instances of similar cost); others through host-built lists
    bool prod = true;
    for (auto& kv : lists) {
        const int f = kv.first.first;
        prod = prod && (f == DEGPU_RHS_VAN_DER_POL || f == DEGPU_RHS_PENDULUM || f == DEGPU_RHS_LORENZ);
    }
    if (prod) {
        EnsArgs ma = a;
        ma.count = n;
        // the persistent multi-family kernel where it is built (fast and mixed DOPRI5 / DOP853),
        // else one run-to-completion launch per (precision, family) list
        if (multi_registry().count({cfg->method, cfg->precision, 2}))
            return multi_solve(cfg, ma, in->family, pb->rhs_id, true, s, true);
        return sorted_thread_solve(cfg, ma, in->family, pb->rhs_id, true, s, true);
    }
    for (auto& kv : lists) {
        EnsArgs ga = a;
        if (lists.size() > 1 || in->family) {
            int64_t* d_idx = scratch.alloc<int64_t>(kv.second.size());
            if (!d_idx) return DEGPU_OOM;
            if (cudaMemcpyAsync(d_idx, kv.second.data(), kv.second.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                                s) != cudaSuccess)
                return DEGPU_CUDA_ERROR;
            ga.index = d_idx;
            ga.count = (int64_t)kv.second.size();
        } else {
            ga.index = nullptr;
            ga.count = n;
        }
        auto it = cross_registry().find(VariantKey{cfg->method, kv.first.first, kv.first.second, 1});
        if (it->second(ga, DEGPU_KERNEL_THREAD, s) != cudaSuccess) return DEGPU_CUDA_ERROR;
    }
    // the index lists came from host vectors that die with this call
    if (cudaStreamSynchronize(s) != cudaSuccess) return DEGPU_CUDA_ERROR;
    return DEGPU_OK;
}

// Shared body of the device-pointer crossing entry points.
template <class Spec>
static degpu_status crossing_entry(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                   const Spec* sd, degpu_batch_out* out, degpu_crossing_out* co, cudaStream_t s) {
    if (!sd || !co) return DEGPU_BAD_INPUT;
    degpu_status v = validate_solve_args(pb, cfg, in, out);
    if (v != DEGPU_OK || in->n == 0) return v;
    CrossSpec cr;
    if (!make_spec(sd, pb->dim, cr)) return DEGPU_BAD_INPUT;
    // output times are the base output of events only (crossings replace them)
    if ((in->n_eval > 0 && cr.mode != 2) || in->dims || pb->rhs_id >= DEGPU_RHS_NVRTC_BASE) return DEGPU_UNSUPPORTED;
    if (!co->count || (cr.max_points > 0 && (!co->t || !co->y))) return DEGPU_BAD_INPUT;
    ensure_registered();
    std::vector<double> te;
    if (in->n_eval > 0 && out->dense) {
        te.resize(in->n_eval);
        if (cudaMemcpyAsync(te.data(), in->t_eval, in->n_eval * sizeof(double), cudaMemcpyDeviceToHost, s) !=
                cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return DEGPU_CUDA_ERROR;
    }
    return crossing_impl(pb, cfg, in, cr, out, co, te.empty() ? nullptr : te.data(), s);
}

// Shared body of the host-pointer crossing entry points: copies in, solves, copies back.
template <class Spec>
static degpu_status crossing_host_entry(const degpu_problem* pb, const degpu_method_cfg* cfg,
                                        const degpu_batch_in* in, const Spec* sd, degpu_batch_out* out,
                                        degpu_crossing_out* co) {
    if (!sd || !co) return DEGPU_BAD_INPUT;
    degpu_status v = validate_solve_args(pb, cfg, in, out);
    if (v != DEGPU_OK || in->n == 0) return v;
    CrossSpec cr;
    if (!make_spec(sd, pb->dim, cr)) return DEGPU_BAD_INPUT;
    if ((in->n_eval > 0 && cr.mode != 2) || in->dims || pb->rhs_id >= DEGPU_RHS_NVRTC_BASE) return DEGPU_UNSUPPORTED;
    if (!co->count || (cr.max_points > 0 && (!co->t || !co->y))) return DEGPU_BAD_INPUT;
    ensure_registered();
    const size_t ne = (in->n_eval > 0 && out->dense) ? (size_t)in->n_eval : 0;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return DEGPU_CUDA_ERROR;
    degpu_status st = DEGPU_OK;
    {
        const int64_t n = in->n;
        const size_t d = (size_t)pb->dim, np = (size_t)pb->n_params, m = (size_t)cr.max_points;
        Scratch sc(s);
        degpu_batch_in din = *in;
        degpu_batch_out dout{};
        degpu_crossing_out dco{};
        auto up = [&](const void* src, size_t bytes) -> void* {
            if (!src) return nullptr;
            void* p = sc.alloc<char>(bytes);
            if (p) cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, s);
            return p;
        };
        din.t0 = (const double*)up(in->t0, n * 8);
        din.tf = (const double*)up(in->tf, n * 8);
        din.y0 = (const double*)up(in->y0, d * n * 8);
        din.params = np > 0 ? (const double*)up(in->params, np * n * 8) : nullptr;
        din.rtol = (const double*)up(in->rtol, n * 8);
        din.atol = (const double*)up(in->atol, n * 8);
        din.rtol_vec = (const double*)up(in->rtol_vec, d * n * 8);
        din.atol_vec = (const double*)up(in->atol_vec, d * n * 8);
        din.family = in->family ? (const int32_t*)up(in->family, n * 4) : nullptr;
        din.t_eval = ne > 0 ? (const double*)up(in->t_eval, ne * 8) : nullptr;
        din.n_eval = (int32_t)ne;
        dout.y_final = sc.alloc<double>(d * n);
        dout.t_final = out->t_final ? sc.alloc<double>(n) : nullptr;
        dout.dense = ne > 0 ? sc.alloc<double>(ne * d * n) : nullptr;
        dout.accepted = out->accepted ? sc.alloc<int64_t>(n) : nullptr;
        dout.rejected = out->rejected ? sc.alloc<int64_t>(n) : nullptr;
        dout.fevals = out->fevals ? sc.alloc<int64_t>(n) : nullptr;
        dout.status = out->status ? sc.alloc<int32_t>(n) : nullptr;
        dco.t = m > 0 ? sc.alloc<double>(m * n) : nullptr;
        dco.y = m > 0 ? sc.alloc<double>(m * d * n) : nullptr;
        dco.count = sc.alloc<int32_t>(n);
        if (!din.t0 || !din.tf || !din.y0 || !din.rtol || !din.atol || !dout.y_final || !dco.count ||
            (m > 0 && (!dco.t || !dco.y)) || (ne > 0 && (!din.t_eval || !dout.dense)) ||
            (in->rtol_vec && !din.rtol_vec) || (in->atol_vec && !din.atol_vec)) {
            st = DEGPU_OOM;
        } else {
            st = crossing_impl(pb, cfg, &din, cr, &dout, &dco, ne > 0 ? in->t_eval : nullptr, s);
        }
        if (st == DEGPU_OK) {
            auto down = [&](void* dst, const void* src, size_t bytes) {
                if (dst && src) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
            };
            down(out->y_final, dout.y_final, d * n * 8);
            down(out->t_final, dout.t_final, n * 8);
            down(out->dense, dout.dense, ne * d * n * 8);
            down(out->accepted, dout.accepted, n * 8);
            down(out->rejected, dout.rejected, n * 8);
            down(out->fevals, dout.fevals, n * 8);
            down(out->status, dout.status, n * 4);
            down(co->t, dco.t, m * n * 8);
            down(co->y, dco.y, m * d * n * 8);
            down(co->count, dco.count, n * 4);
        }
        if (cudaStreamSynchronize(s) != cudaSuccess && st == DEGPU_OK) st = DEGPU_CUDA_ERROR;
    }
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return st;
}

}  // namespace degpu

using namespace degpu;

extern "C" {

void degpu_default_cfg(degpu_method_cfg* cfg, int32_t method) {
    if (!cfg) return;
    cfg->method = method;
    cfg->precision = DEGPU_FP64_PARITY;
    cfg->kernel = DEGPU_KERNEL_AUTO;
    cfg->dense_mode = DEGPU_DENSE_REFERENCE;
    cfg->h0 = 0.0;
    cfg->h_min = 0.0;
    cfg->h_max = INFINITY;
    cfg->max_steps = 10000;
    cfg->safety_factor = 0.9;
    cfg->min_scale = 0.2;
    cfg->max_scale = 10.0;
}

degpu_status degpu_set_mixed_min_rtol(int32_t method, double min_rtol) {
    if (method != DEGPU_DOPRI5 && method != DEGPU_DOP853 && method != DEGPU_RKF45 && method != DEGPU_CASH_KARP)
        return DEGPU_BAD_INPUT;
    if (!std::isfinite(min_rtol) || min_rtol < 0.0) return DEGPU_BAD_INPUT;
    mixed_bound(bound_slot(method)).store(min_rtol);
    return DEGPU_OK;
}

double degpu_mixed_min_rtol(int32_t method) {
    if (!valid_method(method) || method == DEGPU_RK4) return 0.0;
    if (method >= DEGPU_RKV655E) return INFINITY;
    return mixed_bound(bound_slot(method)).load();
}

degpu_status degpu_rhs_info(int32_t rhs_id, int32_t* dim, int32_t* n_params) {
    int d, np;
    builtin_info(rhs_id, d, np);
    if (np < 0) {
        if (rhs_id >= DEGPU_RHS_NVRTC_BASE) return nvrtc_rhs_info(rhs_id, dim, n_params);
        return DEGPU_BAD_INPUT;
    }
    if (dim) *dim = d;
    if (n_params) *n_params = np;
    return DEGPU_OK;
}

degpu_status degpu_solve_ensemble(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                  degpu_batch_out* out, void* stream) {
    degpu_status v = validate_solve_args(pb, cfg, in, out);
    if (v != DEGPU_OK || in->n == 0) return v;
    cudaStream_t s = (cudaStream_t)stream;
    if (pb->rhs_id >= DEGPU_RHS_NVRTC_BASE) return nvrtc_solve(pb, cfg, in, out, s);
    // small host copies: the family map and the requested times
    std::vector<int32_t> fam;
    std::vector<double> te;
    if (in->family) {
        fam.resize(in->n);
        if (cudaMemcpyAsync(fam.data(), in->family, in->n * sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return DEGPU_CUDA_ERROR;
    }
    if (in->n_eval > 0) {
        te.resize(in->n_eval);
        if (cudaMemcpyAsync(te.data(), in->t_eval, in->n_eval * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return DEGPU_CUDA_ERROR;
    }
    if ((in->family || in->n_eval > 0) && cudaStreamSynchronize(s) != cudaSuccess) return DEGPU_CUDA_ERROR;
    return solve_impl(pb, cfg, in, out, s, in->family ? fam.data() : nullptr, in->n_eval > 0 ? te.data() : nullptr,
                      nullptr);
}

degpu_status degpu_solve_ensemble_crossing(const degpu_problem* pb, const degpu_method_cfg* cfg,
                                           const degpu_batch_in* in, const degpu_crossing* cr, degpu_batch_out* out,
                                           degpu_crossing_out* co, void* stream) {
    return crossing_entry(pb, cfg, in, cr, out, co, (cudaStream_t)stream);
}

degpu_status degpu_solve_ensemble_crossing_host(const degpu_problem* pb, const degpu_method_cfg* cfg,
                                                const degpu_batch_in* in, const degpu_crossing* cr,
                                                degpu_batch_out* out, degpu_crossing_out* co) {
    return crossing_host_entry(pb, cfg, in, cr, out, co);
}

degpu_status degpu_solve_ensemble_hyperplane(const degpu_problem* pb, const degpu_method_cfg* cfg,
                                             const degpu_batch_in* in, const degpu_hyperplane* hp,
                                             degpu_batch_out* out, degpu_crossing_out* co, void* stream) {
    return crossing_entry(pb, cfg, in, hp, out, co, (cudaStream_t)stream);
}

degpu_status degpu_solve_ensemble_event(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                        const degpu_event* ev, degpu_batch_out* out, degpu_crossing_out* co,
                                        void* stream) {
    return crossing_entry(pb, cfg, in, ev, out, co, (cudaStream_t)stream);
}

degpu_status degpu_solve_ensemble_event_host(const degpu_problem* pb, const degpu_method_cfg* cfg,
                                             const degpu_batch_in* in, const degpu_event* ev, degpu_batch_out* out,
                                             degpu_crossing_out* co) {
    return crossing_host_entry(pb, cfg, in, ev, out, co);
}

degpu_status degpu_solve_ensemble_hyperplane_host(const degpu_problem* pb, const degpu_method_cfg* cfg,
                                                  const degpu_batch_in* in, const degpu_hyperplane* hp,
                                                  degpu_batch_out* out, degpu_crossing_out* co) {
    return crossing_host_entry(pb, cfg, in, hp, out, co);
}

degpu_status degpu_solve_ensemble_host(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                       degpu_batch_out* out) {
    degpu_status v = validate_solve_args(pb, cfg, in, out);
    if (v != DEGPU_OK || in->n == 0) return v;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return DEGPU_CUDA_ERROR;
    degpu_status st = DEGPU_OK;
    {
        const int64_t n = in->n;
        const int d = pb->dim, np = pb->n_params, m = in->n_eval;
        Scratch sc(s);
        degpu_batch_in din = *in;
        degpu_batch_out dout{};
        auto up = [&](const void* src, size_t bytes) -> void* {
            if (!src) return nullptr;
            void* p = sc.alloc<char>(bytes);
            if (!p) return nullptr;
            cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, s);
            return p;
        };
        din.t0 = (const double*)up(in->t0, n * 8);
        din.tf = (const double*)up(in->tf, n * 8);
        din.y0 = (const double*)up(in->y0, (size_t)d * n * 8);
        din.params = np > 0 ? (const double*)up(in->params, (size_t)np * n * 8) : nullptr;
        din.rtol = (const double*)up(in->rtol, n * 8);
        din.atol = (const double*)up(in->atol, n * 8);
        din.rtol_vec = (const double*)up(in->rtol_vec, (size_t)d * n * 8);
        din.atol_vec = (const double*)up(in->atol_vec, (size_t)d * n * 8);
        din.dims = in->dims ? (const int32_t*)up(in->dims, n * 4) : nullptr;
        din.family = in->family ? (const int32_t*)up(in->family, n * 4) : nullptr;
        din.t_eval = m > 0 ? (const double*)up(in->t_eval, (size_t)m * 8) : nullptr;
        dout.y_final = sc.alloc<double>((size_t)d * n);
        dout.t_final = out->t_final ? sc.alloc<double>(n) : nullptr;
        dout.dense = (m > 0 && out->dense) ? sc.alloc<double>((size_t)m * d * n) : nullptr;
        dout.accepted = out->accepted ? sc.alloc<int64_t>(n) : nullptr;
        dout.rejected = out->rejected ? sc.alloc<int64_t>(n) : nullptr;
        dout.fevals = out->fevals ? sc.alloc<int64_t>(n) : nullptr;
        dout.status = out->status ? sc.alloc<int32_t>(n) : nullptr;
        if (!din.t0 || !din.tf || !din.y0 || !din.rtol || !din.atol || !dout.y_final ||
            (in->rtol_vec && !din.rtol_vec) || (in->atol_vec && !din.atol_vec)) {
            st = DEGPU_OOM;
        } else if (pb->rhs_id >= DEGPU_RHS_NVRTC_BASE) {
            st = nvrtc_solve(pb, cfg, &din, &dout, s);
        } else {
            st = solve_impl(pb, cfg, &din, &dout, s, in->family, m > 0 ? in->t_eval : nullptr, in->dims);
        }
        if (st == DEGPU_OK) {
            auto down = [&](void* dst, const void* src, size_t bytes) {
                if (dst && src) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
            };
            down(out->y_final, dout.y_final, (size_t)d * n * 8);
            down(out->t_final, dout.t_final, n * 8);
            down(out->dense, dout.dense, (size_t)m * d * n * 8);
            down(out->accepted, dout.accepted, n * 8);
            down(out->rejected, dout.rejected, n * 8);
            down(out->fevals, dout.fevals, n * 8);
            down(out->status, dout.status, n * 4);
        }
        if (cudaStreamSynchronize(s) != cudaSuccess && st == DEGPU_OK) st = DEGPU_CUDA_ERROR;
    }
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return st;
}

degpu_status degpu_eval_rhs(int32_t rhs_id, int32_t precision, int64_t n, int32_t dim, int32_t n_params,
                            const double* t, const double* y, const double* params, double* dydt, void* stream) {
    ensure_registered();
    if (n < 0 || !t || !y || !dydt || !valid_prec(precision)) return DEGPU_BAD_INPUT;
    int d, np;
    builtin_info(rhs_id, d, np);
    if (np < 0 || d != dim || np > n_params || (np > 0 && !params)) return DEGPU_BAD_INPUT;
    auto it = rhs_registry().find({rhs_id, precision});
    if (it == rhs_registry().end()) return DEGPU_UNSUPPORTED;
    return it->second(n, t, y, params, dydt, (cudaStream_t)stream) == cudaSuccess ? DEGPU_OK : DEGPU_CUDA_ERROR;
}

const char* degpu_status_string(degpu_status s) {
    switch (s) {
        case DEGPU_OK: return "ok";
        case DEGPU_BAD_INPUT: return "bad input";
        case DEGPU_OOM: return "out of device memory";
        case DEGPU_TIMEOUT: return "device wait timed out";
        case DEGPU_CUDA_ERROR: return "CUDA error";
        case DEGPU_UNSUPPORTED: return "unsupported combination";
    }
    return "unknown status";
}

const char* degpu_version(void) { return "degpu 0.1.0 (sm_103a)"; }

}  // extern "C"
