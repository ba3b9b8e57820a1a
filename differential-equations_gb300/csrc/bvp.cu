// bvp.cu — boundary value problems by shooting over an ensemble (degpu_solve_bvp_host).
//
// The crate's shooting methods (src/methods/bvp/shooting/single.rs, multiple.rs) run one Newton
// iteration as a sequence of IVP solves: the shot from the current unknowns and one shot per
// Jacobian column.  Here every IVP of one Newton iteration of every unfinished instance of the
// batch goes into a single ensemble solve on the device; the host then forms residuals, the
// forward-difference Jacobian and the Newton step per instance, in the crate's operation order
// (host code is compiled without multiply-add contraction), and builds the next batch.
//
// Multiple shooting re-solves every segment for every Jacobian column in the crate, although a
// column perturbs one node and so changes one segment's IVP; the others give the same bits as the
// iteration's base shots.  Only the changed segment is solved here, and the function-evaluation
// and step counters of the unchanged segments are added again, so the totals equal the crate's.
#include <cmath>
#include <vector>

#include "../../include/degpu.h"

namespace {

// One ensemble solve of a list of shots (t0, tf, y0), each owned by an instance of the batch whose
// parameters and tolerances it uses. Shots are stored flat (y0 row-major per shot) and transposed
// into the ensemble's structure-of-arrays layout when the batch runs.
struct ShotBatch {
    int dim = 0;
    std::vector<double> t0, tf, y0;
    std::vector<int64_t> owner;
    // results
    std::vector<double> y_final, t_final, dense;
    std::vector<int64_t> accepted, rejected, fevals;
    std::vector<int32_t> status;

    explicit ShotBatch(int d) : dim(d) {}
    int64_t size() const { return (int64_t)owner.size(); }
    // a shot from y; component pc (if >= 0) replaced by pv
    int64_t add(int64_t inst, double a, double b, const double* y, int pc = -1, double pv = 0.0) {
        const int64_t k = size();
        t0.push_back(a);
        tf.push_back(b);
        y0.insert(y0.end(), y, y + dim);
        if (pc >= 0) y0[(size_t)k * dim + pc] = pv;
        owner.push_back(inst);
        return k;
    }
    const double* start(int64_t k) const { return &y0[(size_t)k * dim]; }
    double end(int64_t k, int c) const { return y_final[(size_t)c * owner.size() + k]; }
    std::vector<double> yf(int64_t k) const {
        std::vector<double> v(dim);
        for (int c = 0; c < dim; ++c) v[c] = end(k, c);
        return v;
    }

    degpu_status run(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                     const std::vector<double>* t_eval) {
        const int64_t m = size();
        const int np = pb->n_params;
        if (m == 0) return DEGPU_OK;
        std::vector<double> ys((size_t)dim * m), params((size_t)(np > 0 ? np : 1) * m), rtol(m), atol(m);
        for (int64_t k = 0; k < m; ++k) {
            const int64_t i = owner[k];
            for (int c = 0; c < dim; ++c) ys[(size_t)c * m + k] = y0[(size_t)k * dim + c];
            for (int q = 0; q < np; ++q) params[(size_t)q * m + k] = in->params[(int64_t)q * in->n + i];
            rtol[k] = in->rtol[i];
            atol[k] = in->atol[i];
        }
        const int ne = t_eval ? (int)t_eval->size() : 0;
        y_final.assign((size_t)dim * m, 0.0);
        t_final.assign(m, 0.0);
        dense.assign((size_t)ne * dim * m, 0.0);
        accepted.assign(m, 0);
        rejected.assign(m, 0);
        fevals.assign(m, 0);
        status.assign(m, 0);
        degpu_batch_in bi{};
        bi.n = m;
        bi.t0 = t0.data();
        bi.tf = tf.data();
        bi.y0 = ys.data();
        bi.params = np > 0 ? params.data() : nullptr;
        bi.rtol = rtol.data();
        bi.atol = atol.data();
        bi.t_eval = ne ? t_eval->data() : nullptr;
        bi.n_eval = ne;
        degpu_batch_out bo{y_final.data(), t_final.data(), ne ? dense.data() : nullptr, accepted.data(),
                           rejected.data(),   fevals.data(),  status.data()};
        return degpu_solve_ensemble_host(pb, cfg, &bi, &bo);
    }
};

// Per-instance state of the Newton iteration.
struct Inst {
    enum Phase { ACTIVE, CONVERGED, DONE } phase = ACTIVE;
    int32_t status = DEGPU_COMPLETE;
    std::vector<double> u;                 // unknowns: y(t0), or the mesh nodes
    std::vector<double> y_err;             // state reported on failure
    double t_err = 0.0;
    int64_t fevals = 0, accepted = 0, rejected = 0, jacobian = 0;
    int32_t iterations = 0;
    int64_t base = -1;                     // first shot of this iteration
    void count(const ShotBatch& b, int64_t k) {
        fevals += b.fevals[k];
        accepted += b.accepted[k];
        rejected += b.rejected[k];
    }
    void fail(int32_t st, double t, std::vector<double> y) {
        phase = DONE;
        status = st;
        t_err = t;
        y_err = std::move(y);
    }
};

// src/traits.rs:93-99: f64::max folded from zero over |r_i|
double max_norm(const std::vector<double>& r) {
    double m = 0.0;
    for (double v : r) m = std::fmax(m, std::fabs(v));
    return m;
}

// Dense LU with partial pivoting as src/linalg/lu.rs:185-240 forms it (row-major a, negated
// multipliers, pivot row swapped column by column), then the solve of src/traits.rs:108-155.
// False when a pivot is zero.
bool lu_solve(std::vector<double>& a, int n, std::vector<double>& b) {
    std::vector<int> ip(n, 0);
    if (n == 1) {
        if (a[0] == 0.0) return false;
        b[0] = b[0] / a[0];
        return true;
    }
    for (int k = 0; k + 1 < n; ++k) {
        int m = k;
        double best = std::fabs(a[(size_t)k * n + k]);
        for (int i = k + 1; i < n; ++i)
            if (std::fabs(a[(size_t)i * n + k]) > best) {
                best = std::fabs(a[(size_t)i * n + k]);
                m = i;
            }
        ip[k] = m;
        const double pivot = a[(size_t)m * n + k];
        if (pivot == 0.0) return false;
        if (m != k) std::swap(a[(size_t)m * n + k], a[(size_t)k * n + k]);
        const double inv = 1.0 / pivot;
        for (int i = k + 1; i < n; ++i) a[(size_t)i * n + k] = -a[(size_t)i * n + k] * inv;
        for (int j = k + 1; j < n; ++j) {
            const double tj = a[(size_t)m * n + j];
            if (m != k) std::swap(a[(size_t)m * n + j], a[(size_t)k * n + j]);
            if (tj != 0.0)
                for (int i = k + 1; i < n; ++i) a[(size_t)i * n + j] = a[(size_t)i * n + j] + a[(size_t)i * n + k] * tj;
        }
    }
    if (a[(size_t)(n - 1) * n + (n - 1)] == 0.0) return false;
    for (int k = 0; k + 1 < n; ++k) {
        std::swap(b[k], b[ip[k]]);
        const double pv = b[k];
        for (int i = k + 1; i < n; ++i) b[i] = b[i] + a[(size_t)i * n + k] * pv;
    }
    for (int k = n - 1; k >= 1; --k) {
        const double xk = b[k] / a[(size_t)k * n + k];
        b[k] = xk;
        const double neg = -xk;
        for (int i = 0; i < k; ++i) b[i] = b[i] + a[(size_t)i * n + k] * neg;
    }
    b[0] = b[0] / a[0];
    return true;
}

struct Boundary {
    int dim;
    const degpu_bvp* spec;
    // Boundary::boundary(y_a, y_b, res) in the separated form r_i = y_side[comp_i] - value_i
    void eval(const double* ya, const double* yb, double* res) const {
        for (int i = 0; i < dim; ++i)
            res[i] = (spec->side[i] == 0 ? ya[spec->component[i]] : yb[spec->component[i]]) - spec->value[i];
    }
};

const double kSqrtEps = 1.4901161193847656e-08;  // sqrt(f64::EPSILON) = 2^-26

// SingleShooting::solve (single.rs:84-176) for every instance, one ensemble solve per iteration.
degpu_status single_shooting(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                             const degpu_bvp* bvp, std::vector<Inst>& st) {
    const int dim = pb->dim;
    const Boundary bd{dim, bvp};
    for (int it = 0; it < bvp->max_iterations; ++it) {
        ShotBatch b(dim);
        for (int64_t i = 0; i < in->n; ++i) {
            Inst& s = st[i];
            if (s.phase != Inst::ACTIVE) continue;
            s.base = b.add(i, in->t0[i], in->tf[i], s.u.data());
            for (int j = 0; j < dim; ++j)
                b.add(i, in->t0[i], in->tf[i], s.u.data(), j, s.u[j] + kSqrtEps * std::fmax(std::fabs(s.u[j]), 1.0));
        }
        if (b.size() == 0) break;
        degpu_status rc = b.run(pb, cfg, in, nullptr);
        if (rc != DEGPU_OK) return rc;
        for (int64_t i = 0; i < in->n; ++i) {
            Inst& s = st[i];
            if (s.phase != Inst::ACTIVE) continue;
            const int64_t k0 = s.base;
            s.count(b, k0);
            if (b.status[k0] != DEGPU_COMPLETE) {
                s.fail(b.status[k0], b.t_final[k0], b.yf(k0));
                continue;
            }
            std::vector<double> res(dim), resp(dim), jac((size_t)dim * dim);
            const std::vector<double> yb = b.yf(k0);
            bd.eval(s.u.data(), yb.data(), res.data());
            if (max_norm(res) <= bvp->tolerance) {
                s.phase = Inst::CONVERGED;
                continue;
            }
            bool ok = true;
            for (int j = 0; j < dim && ok; ++j) {
                const int64_t kj = k0 + 1 + j;
                s.count(b, kj);
                if (b.status[kj] != DEGPU_COMPLETE) {
                    s.fail(b.status[kj], b.t_final[kj], b.yf(kj));
                    ok = false;
                    break;
                }
                const double pert = kSqrtEps * std::fmax(std::fabs(s.u[j]), 1.0);
                const std::vector<double> ybp = b.yf(kj);
                bd.eval(b.start(kj), ybp.data(), resp.data());
                s.jacobian += 1;
                for (int r = 0; r < dim; ++r) jac[(size_t)r * dim + j] = (resp[r] - res[r]) / pert;
            }
            if (!ok) continue;
            std::vector<double> step(dim);
            for (int r = 0; r < dim; ++r) step[r] = -res[r];
            if (!lu_solve(jac, dim, step)) {
                s.fail(DEGPU_ERR_LINEAR_ALGEBRA, in->t0[i], s.u);
                continue;
            }
            s.iterations += 1;
            for (int r = 0; r < dim; ++r) s.u[r] = s.u[r] + step[r];
        }
    }
    return DEGPU_OK;
}

// MultipleShooting::solve (multiple.rs:190-300) for every instance (one interval for the batch).
degpu_status multiple_shooting(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                               const degpu_bvp* bvp, std::vector<Inst>& st) {
    const int dim = pb->dim, segs = bvp->segments, unknowns = (segs + 1) * dim;
    const Boundary bd{dim, bvp};
    // mesh (multiple.rs:83-107): t0 + span * i / m
    const double t0 = in->t0[0], tf = in->tf[0], span = tf - t0;
    std::vector<double> mesh(segs + 1);
    for (int i = 0; i <= segs; ++i) mesh[i] = t0 + span * (double)i / (double)segs;
    {
        // initial_nodes (multiple.rs:108-126): one shot over [t0, tf] with output at the mesh
        ShotBatch b(dim);
        for (int64_t i = 0; i < in->n; ++i) b.add(i, t0, tf, st[i].u.data());
        degpu_status rc = b.run(pb, cfg, in, &mesh);
        if (rc != DEGPU_OK) return rc;
        const int64_t m = b.size();
        for (int64_t i = 0; i < in->n; ++i) {
            Inst& s = st[i];
            s.count(b, i);
            if (b.status[i] != DEGPU_COMPLETE) {
                s.fail(b.status[i], b.t_final[i], b.yf(i));
                continue;
            }
            std::vector<double> nodes((size_t)unknowns);
            bool all = true;
            for (int k = 0; k <= segs; ++k)
                for (int c = 0; c < dim; ++c) {
                    const double v = b.dense[((size_t)k * dim + c) * m + i];
                    all = all && !std::isnan(v);
                    nodes[(size_t)k * dim + c] = v;
                }
            if (!all) {
                s.fail(DEGPU_ERR_BAD_INPUT, t0, s.u);  // not every mesh node was produced
                continue;
            }
            s.u = std::move(nodes);
        }
    }
    for (int it = 0; it < bvp->max_iterations; ++it) {
        ShotBatch b(dim);
        for (int64_t i = 0; i < in->n; ++i) {
            Inst& s = st[i];
            if (s.phase != Inst::ACTIVE) continue;
            s.base = b.size();
            for (int g = 0; g < segs; ++g) b.add(i, mesh[g], mesh[g + 1], &s.u[(size_t)g * dim]);
            // one shot per column whose node starts a segment
            for (int j = 0; j < segs * dim; ++j) {
                const int node = j / dim, c = j % dim;
                const double v = s.u[j];
                b.add(i, mesh[node], mesh[node + 1], &s.u[(size_t)node * dim], c,
                      v + kSqrtEps * std::fmax(std::fabs(v), 1.0));
            }
        }
        if (b.size() == 0) break;
        degpu_status rc = b.run(pb, cfg, in, nullptr);
        if (rc != DEGPU_OK) return rc;
        std::vector<double> res(unknowns), resp(unknowns), jac((size_t)unknowns * unknowns), yend, yendp;
        for (int64_t i = 0; i < in->n; ++i) {
            Inst& s = st[i];
            if (s.phase != Inst::ACTIVE) continue;
            const int64_t k0 = s.base;
            // residual (multiple.rs:127-170): boundary rows, then each segment's mismatch
            bd.eval(&s.u[0], &s.u[(size_t)segs * dim], res.data());
            bool ok = true;
            yend.assign((size_t)segs * dim, 0.0);
            for (int g = 0; g < segs; ++g) {
                s.count(b, k0 + g);
                if (b.status[k0 + g] != DEGPU_COMPLETE) {
                    s.fail(b.status[k0 + g], b.t_final[k0 + g], b.yf(k0 + g));
                    ok = false;
                    break;
                }
                for (int c = 0; c < dim; ++c) {
                    yend[(size_t)g * dim + c] = b.end(k0 + g, c);
                    res[(size_t)(g + 1) * dim + c] = yend[(size_t)g * dim + c] - s.u[(size_t)(g + 1) * dim + c];
                }
            }
            if (!ok) continue;
            if (max_norm(res) <= bvp->tolerance) {
                s.phase = Inst::CONVERGED;
                continue;
            }
            for (int j = 0; j < unknowns && ok; ++j) {
                const int node = j / dim, c = j % dim;
                std::vector<double> pn = s.u;
                const double yj = pn[j];
                const double pert = kSqrtEps * std::fmax(std::fabs(yj), 1.0);
                pn[j] = yj + pert;
                // the perturbed residual: segments before `node` repeat the base shots
                yendp = yend;
                for (int g = 0; g < segs; ++g) {
                    if (g == node) {
                        const int64_t kp = k0 + segs + j;
                        s.count(b, kp);
                        if (b.status[kp] != DEGPU_COMPLETE) {
                            s.fail(b.status[kp], b.t_final[kp], b.yf(kp));
                            ok = false;
                            break;
                        }
                        for (int q = 0; q < dim; ++q)
                            yendp[(size_t)g * dim + q] = b.end(kp, q);
                    } else {
                        s.count(b, k0 + g);
                    }
                }
                if (!ok) break;
                bd.eval(&pn[0], &pn[(size_t)segs * dim], resp.data());
                for (int g = 0; g < segs; ++g)
                    for (int q = 0; q < dim; ++q)
                        resp[(size_t)(g + 1) * dim + q] = yendp[(size_t)g * dim + q] - pn[(size_t)(g + 1) * dim + q];
                s.jacobian += 1;
                for (int r = 0; r < unknowns; ++r) jac[(size_t)r * unknowns + j] = (resp[r] - res[r]) / pert;
                (void)c;
            }
            if (!ok) continue;
            std::vector<double> step(unknowns);
            for (int r = 0; r < unknowns; ++r) step[r] = -res[r];
            if (!lu_solve(jac, unknowns, step)) {
                s.fail(DEGPU_ERR_LINEAR_ALGEBRA, t0, std::vector<double>(s.u.begin(), s.u.begin() + dim));
                continue;
            }
            s.iterations += 1;
            for (int r = 0; r < unknowns; ++r) s.u[r] = s.u[r] + step[r];
        }
    }
    return DEGPU_OK;
}

}  // namespace

extern "C" degpu_status degpu_solve_bvp_host(const degpu_problem* pb, const degpu_method_cfg* cfg,
                                             const degpu_batch_in* in, const degpu_bvp* bvp, degpu_batch_out* out,
                                             degpu_bvp_out* bo) {
    if (!pb || !cfg || !in || !bvp || !out || !bo) return DEGPU_BAD_INPUT;
    if (in->n < 0 || !out->y_final || !bo->y_a || !in->t0 || !in->tf || !in->y0 || !in->rtol || !in->atol)
        return DEGPU_BAD_INPUT;
    const int dim = pb->dim;
    if (dim < 1 || dim > DEGPU_HYPERPLANE_MAX_DIM || pb->rhs_id >= DEGPU_RHS_NVRTC_BASE) return DEGPU_BAD_INPUT;
    if (in->family || in->dims || (pb->n_params > 0 && !in->params)) return DEGPU_UNSUPPORTED;
    if (in->n_eval < 0 || (in->n_eval > 0 && !in->t_eval)) return DEGPU_BAD_INPUT;
    if (bvp->method != DEGPU_BVP_SINGLE && bvp->method != DEGPU_BVP_MULTIPLE) return DEGPU_BAD_INPUT;
    if (bvp->max_iterations < 0) return DEGPU_BAD_INPUT;
    for (int i = 0; i < dim; ++i)
        if (bvp->side[i] < 0 || bvp->side[i] > 1 || bvp->component[i] < 0 || bvp->component[i] >= dim)
            return DEGPU_BAD_INPUT;
    const bool multi = bvp->method == DEGPU_BVP_MULTIPLE;
    if (multi) {
        if (bvp->segments < 1 || (int64_t)(bvp->segments + 1) * dim > DEGPU_BVP_MAX_UNKNOWNS) return DEGPU_BAD_INPUT;
        for (int64_t i = 1; i < in->n; ++i)
            if (in->t0[i] != in->t0[0] || in->tf[i] != in->tf[0]) return DEGPU_UNSUPPORTED;
    }
    const int64_t n = in->n;
    if (n == 0) return DEGPU_OK;
    std::vector<Inst> st(n);
    std::vector<std::vector<double>> guess(n);
    for (int64_t i = 0; i < n; ++i) {
        st[i].u.resize(dim);
        for (int c = 0; c < dim; ++c) st[i].u[c] = in->y0[(int64_t)c * n + i];
        guess[i] = st[i].u;
    }
    // The forward-difference Jacobian perturbs by sqrt(eps) max(|u|, 1) ~ 1.5e-8 relative, below
    // FP32 resolution: a mixed solve's FP32 stages would return the unperturbed shot and a zero
    // column. Shots of a mixed BVP solve therefore run in FP64 fast arithmetic.
    degpu_method_cfg c64 = *cfg;
    if (c64.precision == DEGPU_MIXED) c64.precision = DEGPU_FP64_FAST;
    cfg = &c64;
    degpu_status rc = multi ? multiple_shooting(pb, cfg, in, bvp, st) : single_shooting(pb, cfg, in, bvp, st);
    if (rc != DEGPU_OK) return rc;
    // instances still iterating: Error::MaxSteps { t: t0, y: the guess (single) or the first node }
    for (int64_t i = 0; i < n; ++i)
        if (st[i].phase == Inst::ACTIVE)
            st[i].fail(DEGPU_ERR_MAX_STEPS, in->t0[i],
                       multi ? std::vector<double>(st[i].u.begin(), st[i].u.begin() + dim) : guess[i]);
    // the final solve from the converged initial state, into the caller's outputs
    ShotBatch fin(dim);
    std::vector<double> te;
    if (in->n_eval > 0 && out->dense) te.assign(in->t_eval, in->t_eval + in->n_eval);
    for (int64_t i = 0; i < n; ++i)
        if (st[i].phase == Inst::CONVERGED) st[i].base = fin.add(i, in->t0[i], in->tf[i], st[i].u.data());
    rc = fin.run(pb, cfg, in, te.empty() ? nullptr : &te);
    if (rc != DEGPU_OK) return rc;
    const int64_t fm = fin.size();
    const int ne = (int)te.size();
    for (int64_t i = 0; i < n; ++i) {
        Inst& s = st[i];
        const bool conv = s.phase == Inst::CONVERGED;
        int32_t status = s.status;
        double tfin = s.t_err;
        std::vector<double> yfin = s.y_err;
        if (conv) {
            const int64_t k = s.base;
            s.count(fin, k);
            status = fin.status[k];
            tfin = fin.t_final[k];
            yfin = fin.yf(k);
        }
        for (int c = 0; c < dim; ++c) {
            out->y_final[(int64_t)c * n + i] = yfin.size() == (size_t)dim ? yfin[c] : NAN;
            bo->y_a[(int64_t)c * n + i] = (conv && status == DEGPU_COMPLETE) ? s.u[c] : NAN;
        }
        if (out->t_final) out->t_final[i] = tfin;
        if (out->accepted) out->accepted[i] = s.accepted;
        if (out->rejected) out->rejected[i] = s.rejected;
        if (out->fevals) out->fevals[i] = s.fevals;
        if (out->status) out->status[i] = status;
        if (bo->iterations) bo->iterations[i] = s.iterations;
        if (bo->jacobian) bo->jacobian[i] = s.jacobian;
        if (out->dense && ne > 0)
            for (int e = 0; e < ne; ++e)
                for (int c = 0; c < dim; ++c)
                    out->dense[((int64_t)e * dim + c) * n + i] =
                        (conv && status == DEGPU_COMPLETE) ? fin.dense[((size_t)e * dim + c) * fm + s.base] : NAN;
    }
    return DEGPU_OK;
}
