// oracle.cpp — TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline).
//
// C ABI of the CPU restatement in oracle.hpp.  The ensemble entry point mirrors
// degpu_solve_ensemble (include/degpu.h) with HOST pointers and solves one crate-style IVP per
// instance, statically chunked over `threads` std::threads — the "one crate solve per instance,
// looped over all host threads" baseline.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <thread>

#include "oracle.hpp"
#include "oracle_bvp.hpp"
#include "oracle_mol.hpp"

#if defined(__x86_64__) || defined(__i386__)
#include <quadmath.h>
typedef __float128 qreal_t;
static inline qreal_t q_pow(qreal_t x, qreal_t y) { return powq(x, y); }
static inline qreal_t q_sin(qreal_t x) { return sinq(x); }
static inline qreal_t q_cos(qreal_t x) { return cosq(x); }
#else
static_assert(LDBL_MANT_DIG == 113, "the correctly rounded oracle mode needs binary128 long double");
typedef long double qreal_t;
static inline qreal_t q_pow(qreal_t x, qreal_t y) { return powl(x, y); }
static inline qreal_t q_sin(qreal_t x) { return sinl(x); }
static inline qreal_t q_cos(qreal_t x) { return cosl(x); }
#endif

namespace oracle {
// A binary128 evaluation (113-bit significand, error of a few units in its last place) rounded
// once to binary64 gives the correctly rounded double except when the exact value lies within
// ~2^-58 ulp of a rounding boundary.
double cr_pow(double x, double y) { return (double)q_pow((qreal_t)x, (qreal_t)y); }
double cr_sin(double x) { return (double)q_sin((qreal_t)x); }
double cr_cos(double x) { return (double)q_cos((qreal_t)x); }
}  // namespace oracle

using namespace oracle;

// Runs body(i) for i in [0, n) on `threads` host threads with dynamic chunks (instances differ
// widely in cost).
template <class Body>
static void for_instances(int64_t n, int threads, Body body) {
    if (threads <= 1 || n < 2) {
        for (int64_t i = 0; i < n; ++i) body(i);
        return;
    }
    std::atomic<int64_t> next{0};
    const int64_t chunk = 16;
    std::vector<std::thread> pool;
    for (int w = 0; w < threads; ++w)
        pool.emplace_back([&]() {
            for (;;) {
                int64_t s = next.fetch_add(chunk);
                if (s >= n) break;
                int64_t e = std::min(n, s + chunk);
                for (int64_t i = s; i < e; ++i) body(i);
            }
        });
    for (auto& t : pool) t.join();
}

extern "C" {

// Scalar math, exposed for tests of the math policy.
double oracle_cr_pow(double x, double y) { return cr_pow(x, y); }
double oracle_cr_sin(double x) { return cr_sin(x); }
double oracle_cr_cos(double x) { return cr_cos(x); }
double oracle_libm_pow(double x, double y) { return std::pow(x, y); }
double oracle_libm_sin(double x) { return std::sin(x); }
double oracle_libm_cos(double x) { return std::cos(x); }

void oracle_cr_pow_batch(const double* x, const double* y, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = cr_pow(x[i], y[i]);
}
void oracle_cr_sincos_batch(const double* x, double* s, double* c, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        s[i] = cr_sin(x[i]);
        c[i] = cr_cos(x[i]);
    }
}
void oracle_libm_pow_batch(const double* x, const double* y, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = std::pow(x[i], y[i]);
}

// Solve one instance i of the batch into the outputs.
// The Tolerance of instance i: the per-component column of `vec` ([d][n]) when given, else the
// scalar `scalar[i]` (src/tolerance.rs:11-14).
static Tolerance tolerance_of(const double* scalar, const double* vec, int64_t n, int64_t i, int d) {
    Tolerance t(scalar[i]);
    if (vec) {
        t.vec.resize(d);
        for (int c = 0; c < d; ++c) t.vec[c] = vec[(int64_t)c * n + i];
    }
    return t;
}

static void solve_instance(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                           degpu_batch_out* out, int64_t i, const Math& math, const CrossingSolout* proto = nullptr,
                           int64_t max_points = 0, degpu_crossing_out* co = nullptr,
                           const EventSolout* eproto = nullptr) {
    const int64_t n = in->n;
    int rhs = in->family ? in->family[i] : pb->rhs_id;
    // per-instance dimension: given explicitly (ragged batches) or the family's own
    int fam_dim, fam_np;
    builtin_info(rhs, fam_dim, fam_np);
    int d = in->dims ? in->dims[i] : (fam_dim > 0 ? fam_dim : pb->dim);
    int dmax = pb->dim;
    State y0(d);
    for (int c = 0; c < d; ++c) y0[c] = in->y0[(int64_t)c * n + i];
    std::vector<double> p(pb->n_params);
    for (int q = 0; q < pb->n_params; ++q) p[q] = in->params[(int64_t)q * n + i];
    BuiltinOde ode(rhs, d, p, math);
    Settings set;
    set.rtol = tolerance_of(in->rtol, in->rtol_vec, n, i, d);
    set.atol = tolerance_of(in->atol, in->atol_vec, n, i, d);
    set.h0 = cfg->h0;
    set.h_min = cfg->h_min;
    set.h_max = cfg->h_max;
    set.max_steps = cfg->max_steps;
    set.safety_factor = cfg->safety_factor;
    set.min_scale = cfg->min_scale;
    set.max_scale = cfg->max_scale;
    std::vector<double> te;
    const std::vector<double>* tep = nullptr;
    if (in->n_eval > 0 && in->t_eval) {
        te.assign(in->t_eval, in->t_eval + in->n_eval);
        tep = &te;
    }
    CrossingSolout cs;
    if (proto) cs = *proto;
    EventSolout es;
    if (eproto) es = *eproto;
    Result r = solve_one(cfg->method, ode, in->t0[i], in->tf[i], y0, set, math, tep,
                         cfg->dense_mode == DEGPU_DENSE_HAIRER, proto ? &cs : nullptr, eproto ? &es : nullptr);
    if ((proto || eproto) && co) {
        const std::vector<double>& pt = proto ? cs.t : es.t;
        const std::vector<State>& py = proto ? cs.y : es.y;
        const int64_t m = max_points;
        co->count[i] = (int32_t)pt.size();
        for (int64_t k = 0; k < m; ++k) {
            const bool have = (size_t)k < pt.size();
            co->t[k * n + i] = have ? pt[k] : NAN;
            for (int c = 0; c < dmax; ++c)
                co->y[(k * dmax + c) * n + i] = (have && c < d) ? py[k][c] : NAN;
        }
    }
    for (int c = 0; c < d; ++c) out->y_final[(int64_t)c * n + i] = r.y_final.size() == (size_t)d ? r.y_final[c] : NAN;
    for (int c = d; c < dmax; ++c) out->y_final[(int64_t)c * n + i] = 0.0;
    if (out->t_final) out->t_final[i] = r.t_final;
    if (out->accepted) out->accepted[i] = r.accepted;
    if (out->rejected) out->rejected[i] = r.rejected;
    if (out->fevals) out->fevals[i] = r.fevals;
    if (out->status) out->status[i] = r.outcome.status;
    if (out->dense && tep) {
        for (int e = 0; e < in->n_eval; ++e)
            for (int c = 0; c < dmax; ++c) {
                // rows beyond the instance's dimension are never written: they keep the NaN fill
                double v = (c < d && (size_t)e < r.dense.size()) ? r.dense[e][c] : NAN;
                out->dense[((int64_t)e * dmax + c) * n + i] = v;
            }
    }
}

// Crossing detection (CrossingSolout) for every instance; outputs laid out as
// degpu_solve_ensemble_crossing's.  Returns 0 on success, 1 on bad input.
int oracle_solve_ensemble_crossing(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                   const degpu_crossing* cr, degpu_batch_out* out, degpu_crossing_out* co,
                                   int threads, int math_mode) {
    if (!pb || !cfg || !in || !out || !cr || !co || in->n < 0 || !out->y_final || in->n_eval > 0) return 1;
    if (cr->component < 0 || cr->component >= pb->dim || cr->max_points < 0) return 1;
    Math math;
    math.mode = math_mode == 0 ? MathMode::Libm : MathMode::CorrectlyRounded;
    CrossingSolout proto;
    proto.comp = cr->component;
    proto.threshold = cr->threshold;
    proto.direction = cr->direction;
    for_instances(in->n, threads,
                  [&](int64_t i) { solve_instance(pb, cfg, in, out, i, math, &proto, cr->max_points, co); });
    return 0;
}

// Hyperplane crossing detection (HyperplaneCrossingSolout) for every instance; outputs laid out
// as degpu_solve_ensemble_hyperplane's.  Returns 0 on success, 1 on bad input.
int oracle_solve_ensemble_hyperplane(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                     const degpu_hyperplane* hp, degpu_batch_out* out, degpu_crossing_out* co,
                                     int threads, int math_mode) {
    if (!pb || !cfg || !in || !out || !hp || !co || in->n < 0 || !out->y_final || in->n_eval > 0) return 1;
    if (hp->dim < 1 || hp->dim > DEGPU_HYPERPLANE_MAX_DIM || hp->max_points < 0) return 1;
    std::vector<int> comps(hp->components, hp->components + hp->dim);
    for (int c : comps)
        if (c < 0 || c >= pb->dim) return 1;
    Math math;
    math.mode = math_mode == 0 ? MathMode::Libm : MathMode::CorrectlyRounded;
    CrossingSolout proto;
    proto.direction = hp->direction;
    proto.set_plane(comps, std::vector<double>(hp->point, hp->point + hp->dim),
                    std::vector<double>(hp->normal, hp->normal + hp->dim));
    for_instances(in->n, threads,
                  [&](int64_t i) { solve_instance(pb, cfg, in, out, i, math, &proto, hp->max_points, co); });
    return 0;
}

// Event detection (EventWrappedSolout over the output times, or over DefaultSolout when there are
// none) for every instance; event points laid out as degpu_solve_ensemble_event's.  Returns 0 on
// success, 1 on bad input.
int oracle_solve_ensemble_event(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                const degpu_event* ev, degpu_batch_out* out, degpu_crossing_out* co, int threads,
                                int math_mode) {
    if (!pb || !cfg || !in || !out || !ev || !co || in->n < 0 || !out->y_final) return 1;
    if (ev->kind != DEGPU_EVENT_LINEAR && ev->kind != DEGPU_EVENT_MAX_ABS) return 1;
    if (ev->n_terms < (ev->kind == DEGPU_EVENT_MAX_ABS ? 1 : 0) || ev->n_terms > DEGPU_EVENT_MAX_TERMS) return 1;
    if (ev->max_points < 0 || ev->terminate < 0 || ev->direction < -1 || ev->direction > 1) return 1;
    EventSolout proto;
    proto.kind = ev->kind;
    proto.direction = ev->direction;
    proto.terminate = ev->terminate;
    proto.t_weight = ev->t_weight;
    proto.offset = ev->offset;
    for (int j = 0; j < ev->n_terms; ++j) {
        if (ev->components[j] < 0 || ev->components[j] >= pb->dim) return 1;
        proto.comp.push_back(ev->components[j]);
        proto.w.push_back(ev->weights[j]);
    }
    Math math;
    math.mode = math_mode == 0 ? MathMode::Libm : MathMode::CorrectlyRounded;
    for_instances(in->n, threads, [&](int64_t i) {
        solve_instance(pb, cfg, in, out, i, math, nullptr, ev->max_points, co, &proto);
    });
    return 0;
}

// Boundary value problems by shooting (SingleShooting / MultipleShooting) for every instance;
// outputs laid out as degpu_solve_bvp_host's.  Returns 0 on success, 1 on bad input.
int oracle_solve_bvp(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                     const degpu_bvp* bvp, degpu_batch_out* out, degpu_bvp_out* bo, int threads, int math_mode) {
    if (!pb || !cfg || !in || !out || !bvp || !bo || in->n < 0 || !out->y_final) return 1;
    const int dim = pb->dim;
    if (dim < 1 || dim > DEGPU_HYPERPLANE_MAX_DIM) return 1;
    BvpSpec spec;
    spec.method = bvp->method;
    spec.segments = bvp->segments;
    spec.max_iterations = bvp->max_iterations;
    spec.tolerance = bvp->tolerance;
    for (int i = 0; i < dim; ++i) {
        if (bvp->side[i] < 0 || bvp->side[i] > 1 || bvp->component[i] < 0 || bvp->component[i] >= dim) return 1;
        spec.side.push_back(bvp->side[i]);
        spec.comp.push_back(bvp->component[i]);
        spec.value.push_back(bvp->value[i]);
    }
    Math math;
    math.mode = math_mode == 0 ? MathMode::Libm : MathMode::CorrectlyRounded;
    const int64_t n = in->n;
    std::vector<double> te;
    if (in->n_eval > 0 && in->t_eval) te.assign(in->t_eval, in->t_eval + in->n_eval);
    for_instances(n, threads, [&](int64_t i) {
        int fam_dim, fam_np;
        builtin_info(pb->rhs_id, fam_dim, fam_np);
        State guess(dim);
        for (int c = 0; c < dim; ++c) guess[c] = in->y0[(int64_t)c * n + i];
        std::vector<double> p(pb->n_params);
        for (int q = 0; q < pb->n_params; ++q) p[q] = in->params[(int64_t)q * n + i];
        BuiltinOde ode(pb->rhs_id, dim, p, math);
        BvpSolver sv{cfg->method, ode, Settings{}, math, cfg->dense_mode == DEGPU_DENSE_HAIRER, BvpResult{}};
        sv.set.rtol = tolerance_of(in->rtol, in->rtol_vec, n, i, dim);
        sv.set.atol = tolerance_of(in->atol, in->atol_vec, n, i, dim);
        sv.set.h0 = cfg->h0;
        sv.set.h_min = cfg->h_min;
        sv.set.h_max = cfg->h_max;
        sv.set.max_steps = cfg->max_steps;
        sv.set.safety_factor = cfg->safety_factor;
        sv.set.min_scale = cfg->min_scale;
        sv.set.max_scale = cfg->max_scale;
        const std::vector<double>* tep = te.empty() ? nullptr : &te;
        if (spec.method == DEGPU_BVP_MULTIPLE)
            sv.multiple(spec, in->t0[i], in->tf[i], guess, tep);
        else
            sv.single(spec, in->t0[i], in->tf[i], guess, tep);
        const BvpResult& r = sv.out;
        const Result& f = r.final;
        for (int c = 0; c < dim; ++c) {
            out->y_final[(int64_t)c * n + i] = f.y_final.size() == (size_t)dim ? f.y_final[c] : NAN;
            bo->y_a[(int64_t)c * n + i] = r.status == DEGPU_COMPLETE ? r.y_a[c] : NAN;
        }
        if (out->t_final) out->t_final[i] = f.t_final;
        if (out->accepted) out->accepted[i] = r.accepted;
        if (out->rejected) out->rejected[i] = r.rejected;
        if (out->fevals) out->fevals[i] = r.fevals;
        if (out->status) out->status[i] = r.status;
        if (bo->iterations) bo->iterations[i] = (int32_t)r.iterations;
        if (bo->jacobian) bo->jacobian[i] = r.jacobian;
        if (out->dense && tep) {
            for (int e = 0; e < in->n_eval; ++e)
                for (int c = 0; c < dim; ++c) {
                    const bool have = r.status == DEGPU_COMPLETE && (size_t)e < f.dense.size();
                    out->dense[((int64_t)e * dim + c) * n + i] = have ? f.dense[e][c] : NAN;
                }
        }
    });
    return 0;
}

// Solve instances [0, n) of the batch with `threads` host threads.  math_mode: 0 libm, 1 cr.
// Returns 0 on success, 1 on bad input.
int oracle_solve_ensemble(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                          degpu_batch_out* out, int threads, int math_mode) {
    if (!pb || !cfg || !in || !out || in->n < 0 || !out->y_final) return 1;
    Math math;
    math.mode = math_mode == 0 ? MathMode::Libm : MathMode::CorrectlyRounded;
    int64_t n = in->n;
    if (threads <= 1 || n < 2) {
        for (int64_t i = 0; i < n; ++i) solve_instance(pb, cfg, in, out, i, math);
        return 0;
    }
    // dynamic chunking: instances differ widely in cost
    std::atomic<int64_t> next{0};
    const int64_t chunk = 16;
    std::vector<std::thread> pool;
    for (int w = 0; w < threads; ++w)
        pool.emplace_back([&]() {
            for (;;) {
                int64_t s = next.fetch_add(chunk);
                if (s >= n) break;
                int64_t e = std::min(n, s + chunk);
                for (int64_t i = s; i < e; ++i) solve_instance(pb, cfg, in, out, i, math);
            }
        });
    for (auto& t : pool) t.join();
    return 0;
}

// One RHS evaluation per instance (same layout as degpu_eval_rhs).
int oracle_eval_rhs(int32_t rhs_id, int64_t n, int32_t dim, int32_t n_params, const double* t, const double* y,
                    const double* params, double* dydt, int math_mode) {
    Math math;
    math.mode = math_mode == 0 ? MathMode::Libm : MathMode::CorrectlyRounded;
    for (int64_t i = 0; i < n; ++i) {
        std::vector<double> p(n_params);
        for (int q = 0; q < n_params; ++q) p[q] = params[(int64_t)q * n + i];
        BuiltinOde ode(rhs_id, dim, p, math);
        State yy(dim), dd(dim, 0.0);
        for (int c = 0; c < dim; ++c) yy[c] = y[(int64_t)c * n + i];
        ode.diff(t[i], yy, dd);
        for (int c = 0; c < dim; ++c) dydt[(int64_t)c * n + i] = dd[c];
    }
    return 0;
}


// ---------------------------------------------------------------------------------------------
// Method of lines (oracle_mol.hpp)
// ---------------------------------------------------------------------------------------------
static Bc make_bc(int kind, const double* val, int L) {
    Bc b;
    b.kind = kind == 0 ? BcKind::Dirichlet : kind == 1 ? BcKind::Neumann : BcKind::Periodic;
    if (val)
        b.value.assign(val, val + L);
    else
        b.value.assign(L, 0.0);
    return b;
}

// Threaded evaluation of SemiDiscrete::diff: nodes are independent, so splitting the node loop
// across threads gives bit-identical results.
static void mol_diff_threaded(const SemiDiscrete& sd, double t, const State& y, State& dydt, int threads) {
    if (threads <= 1) {
        sd.diff(t, y, dydt);
        return;
    }
    size_t N = sd.len();
    std::vector<std::thread> pool;
    for (int w = 0; w < threads; ++w)
        pool.emplace_back([&, w]() {
            size_t s = N * w / threads, e = N * (w + 1) / threads;
            for (size_t node = s; node < e; ++node) {
                // same per-node body as SemiDiscrete::diff
                const int L = sd.L;
                if (sd.dirichlet_mask[node]) {
                    for (int c = 0; c < L; ++c) dydt[node * L + c] = 0.0;
                    continue;
                }
                double x[2];
                sd.point(node, x);
                State der(L, 0.0);
                sd.pde->source(t, x, &y[node * L], der.data(), L);
                for (int a = 0; a < sd.D; ++a) {
                    State flo = sd.fd_flux(t, y, node, a, -1);
                    State fhi = sd.fd_flux(t, y, node, a, +1);
                    for (int c = 0; c < L; ++c) der[c] = der[c] + (fhi[c] - flo[c]) / sd.dx[a];
                }
                for (int c = 0; c < L; ++c) dydt[node * L + c] = der[c];
            }
        });
    for (auto& th : pool) th.join();
}

struct ThreadedOde : Ode {
    const SemiDiscrete* sd;
    int threads;
    void diff(double t, const State& y, State& dydt) const override { mol_diff_threaded(*sd, t, y, dydt, threads); }
};

// 1-D heat equation (tests/pde/method_of_lines.rs:3-11) on StructuredGrid::uniform([lo],[hi],[n]).
// bc kinds: 0 Dirichlet, 1 Neumann.  dydt = SemiDiscretePde::diff(0, y).
int oracle_heat1d_diff(double alpha, int n, double lo, double hi, int lo_kind, double lo_val, int hi_kind,
                       double hi_val, const double* y, double* dydt) {
    HeatPde pde(alpha);
    SemiDiscrete sd;
    sd.pde = &pde;
    sd.D = 1;
    sd.L = 1;
    sd.nodes = {n, 1};
    sd.lower = {lo, 0.0};
    sd.dx = {(hi - lo) / (double)(n - 1), 1.0};
    sd.lo_bc[0] = make_bc(lo_kind, &lo_val, 1);
    sd.hi_bc[0] = make_bc(hi_kind, &hi_val, 1);
    sd.build_mask();
    State yy(y, y + n), dd(n, 0.0);
    sd.diff(0.0, yy, dd);
    for (int i = 0; i < n; ++i) dydt[i] = dd[i];
    return 0;
}

// Coupled diffusion vector field (tests/pde/method_of_lines.rs:13-34,115-140), 1-D, L = 2,
// y interleaved [node*2 + c].
int oracle_coupled1d_diff(double d0, double d1, int n, double lo, double hi, const double* lo_val,
                          const double* hi_val, const double* y, double* dydt) {
    CoupledDiffusionPde pde;
    pde.d0 = d0;
    pde.d1 = d1;
    SemiDiscrete sd;
    sd.pde = &pde;
    sd.D = 1;
    sd.L = 2;
    sd.nodes = {n, 1};
    sd.lower = {lo, 0.0};
    sd.dx = {(hi - lo) / (double)(n - 1), 1.0};
    sd.lo_bc[0] = make_bc(0, lo_val, 2);
    sd.hi_bc[0] = make_bc(0, hi_val, 2);
    sd.build_mask();
    State yy(y, y + 2 * n), dd(2 * n, 0.0);
    sd.diff(0.0, yy, dd);
    for (int i = 0; i < 2 * n; ++i) dydt[i] = dd[i];
    return 0;
}

// Heat equation solved through the full driver with RK4(h) (method_of_lines.rs:36-70).
// Writes the final state; returns the per-instance status.
int oracle_heat1d_solve(double alpha, int n, double t0, double tf, double h, const double* u0, double* uf,
                        int64_t* accepted) {
    HeatPde pde(alpha);
    SemiDiscrete sd;
    sd.pde = &pde;
    sd.D = 1;
    sd.L = 1;
    sd.nodes = {n, 1};
    sd.lower = {0.0, 0.0};
    sd.dx = {1.0 / (double)(n - 1), 1.0};
    double z = 0.0;
    sd.lo_bc[0] = make_bc(0, &z, 1);
    sd.hi_bc[0] = make_bc(0, &z, 1);
    sd.build_mask();
    Settings set;
    set.h0 = h;
    set.max_steps = 10000000;
    Math math;
    State y0(u0, u0 + n);
    Result r = solve_one(DEGPU_RK4, sd, t0, tf, y0, set, math, nullptr);
    for (int i = 0; i < n; ++i) uf[i] = r.y_final[i];
    if (accepted) *accepted = r.accepted;
    return r.outcome.status;
}

static void gs_setup(SemiDiscrete& sd, GrayScottPde& pde, const degpu_gray_scott* gs) {
    pde.Du = gs->Du;
    pde.Dv = gs->Dv;
    pde.F = gs->F;
    pde.k = gs->k;
    sd.pde = &pde;
    sd.D = 2;
    sd.L = 2;
    sd.nodes = {gs->nx, gs->ny};
    sd.lower = {0.0, 0.0};
    sd.dx = {gs->dx, gs->dx};
    for (int a = 0; a < 2; ++a) {
        sd.lo_bc[a] = make_bc(2, nullptr, 2);
        sd.hi_bc[a] = make_bc(2, nullptr, 2);
    }
    sd.build_mask();
}

// Gray–Scott periodic semi-discretisation, u/v as [ny][nx] planes (node = ix + nx*iy).
int oracle_gray_scott_rhs(const degpu_gray_scott* gs, const double* u, const double* v, double* du, double* dv,
                          int threads) {
    GrayScottPde pde;
    SemiDiscrete sd;
    gs_setup(sd, pde, gs);
    size_t N = sd.len();
    State y(2 * N), d(2 * N, 0.0);
    for (size_t i = 0; i < N; ++i) {
        y[2 * i] = u[i];
        y[2 * i + 1] = v[i];
    }
    mol_diff_threaded(sd, 0.0, y, d, threads);
    for (size_t i = 0; i < N; ++i) {
        du[i] = d[2 * i];
        dv[i] = d[2 * i + 1];
    }
    return 0;
}

// `steps` calls of the crate's fixed RK4 step (fixed/ordinary.rs:58-138) after init
// (fixed/ordinary.rs:16-56) with h = dt, on the Gray–Scott system, in place.
int oracle_gray_scott_rk4(const degpu_gray_scott* gs, double t0, double dt, int64_t steps, double* u, double* v,
                          int threads) {
    GrayScottPde pde;
    SemiDiscrete sd;
    gs_setup(sd, pde, gs);
    ThreadedOde ode;
    ode.sd = &sd;
    ode.threads = threads;
    size_t N = sd.len();
    State y(2 * N);
    for (size_t i = 0; i < N; ++i) {
        y[2 * i] = u[i];
        y[2 * i + 1] = v[i];
    }
    FixedRK s;
    s.tab = tableau_rk4();
    s.set.h0 = dt;
    s.set.max_steps = steps + 1;
    Outcome o;
    int64_t fe = 0;
    if (!s.init(ode, t0, t0 + dt * (double)steps, y, fe, o)) return 1;
    for (int64_t st = 0; st < steps; ++st)
        if (!s.step(ode, fe, o)) return 2;
    for (size_t i = 0; i < N; ++i) {
        u[i] = s.y[2 * i];
        v[i] = s.y[2 * i + 1];
    }
    return 0;
}

// The general method-of-lines problem of the ABI (degpu_mol): a SemiDiscrete with the built-in PDE.
struct MolHolder {
    DiffusionPde diff;
    CoupledDiffusionPde coupled;
    GrayScottPde gs;
    SemiDiscrete sd;
};
static bool mol_setup(MolHolder& h, const degpu_mol* m) {
    const int L = m->fields;
    switch (m->pde_id) {
        case DEGPU_PDE_DIFFUSION:
            h.diff.kappa.assign(m->params, m->params + L);
            h.sd.pde = &h.diff;
            break;
        case DEGPU_PDE_COUPLED_DIFFUSION:
            if (L != 2) return false;
            h.coupled.d0 = m->params[0];
            h.coupled.d1 = m->params[1];
            h.sd.pde = &h.coupled;
            break;
        case DEGPU_PDE_GRAY_SCOTT:
            if (L != 2) return false;
            h.gs.Du = m->params[0];
            h.gs.Dv = m->params[1];
            h.gs.F = m->params[2];
            h.gs.k = m->params[3];
            h.sd.pde = &h.gs;
            break;
        default: return false;
    }
    h.sd.D = m->dims;
    h.sd.L = L;
    h.sd.nodes = {m->nodes[0], m->dims == 2 ? m->nodes[1] : 1};
    h.sd.lower = {m->lower[0], m->dims == 2 ? m->lower[1] : 0.0};
    h.sd.dx = {m->dx[0], m->dims == 2 ? m->dx[1] : 1.0};
    for (int a = 0; a < m->dims; ++a) {
        h.sd.lo_bc[a] = make_bc(m->bc_kind[a][0], m->bc_value[a][0], L);
        h.sd.hi_bc[a] = make_bc(m->bc_kind[a][1], m->bc_value[a][1], L);
    }
    h.sd.build_mask();
    return true;
}

// SemiDiscretePde::diff of a degpu_mol problem; y and dydt hold nodes * fields values.
int oracle_mol_rhs(const degpu_mol* m, double t, const double* y, double* dydt, int threads) {
    MolHolder h;
    if (!mol_setup(h, m)) return 1;
    size_t E = h.sd.len() * (size_t)m->fields;
    State yy(y, y + E), dd(E, 0.0);
    mol_diff_threaded(h.sd, t, yy, dd, threads);
    for (size_t e = 0; e < E; ++e) dydt[e] = dd[e];
    return 0;
}

// IVP::pde(..).method(rk4(h)).solve() from t0 to tf (solve_ode with the fixed RK4 step); y in place.
int oracle_mol_rk4(const degpu_mol* m, double t0, double tf, double h0, double* y, int64_t* steps, int threads) {
    MolHolder h;
    if (!mol_setup(h, m)) return 1;
    ThreadedOde ode;
    ode.sd = &h.sd;
    ode.threads = threads;
    size_t E = h.sd.len() * (size_t)m->fields;
    Settings set;
    set.h0 = h0;
    set.max_steps = 100000000;
    Math math;
    State y0(y, y + E);
    Result r = solve_one(DEGPU_RK4, ode, t0, tf, y0, set, math, nullptr);
    for (size_t e = 0; e < E; ++e) y[e] = r.y_final[e];
    if (steps) *steps = r.accepted;
    return r.outcome.status;
}
}  // extern "C"
