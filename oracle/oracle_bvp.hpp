// oracle_bvp.hpp — CPU restatement of the crate's shooting methods for boundary value problems
// (test infrastructure only; the checker of degpu_solve_bvp_host).
//
//   SingleShooting::solve ........... src/methods/bvp/shooting/single.rs:84-176
//   MultipleShooting::{mesh, initial_nodes, residual, solve}
//                                     src/methods/bvp/shooting/multiple.rs:83-300
//   lu_decomp (dense) ............... src/linalg/lu.rs:67-240
//   State::apply_linear_solve ....... src/traits.rs:108-155
//   State::max_norm ................. src/traits.rs:93-99
//
// The boundary function is the separated form r_i = y_side[comp_i] - value_i, which is every
// boundary function of the crate's tests (tests/bvp/systems.rs) and examples. Compile with
// -ffp-contract=off like the rest of the oracle.
#pragma once

#include <cmath>
#include <vector>

#include "oracle.hpp"

namespace oracle {

struct BvpSpec {
    int method = DEGPU_BVP_SINGLE;
    int segments = 4;
    int max_iterations = 100;
    double tolerance = 1e-6;
    std::vector<int> side, comp;
    std::vector<double> value;

    // Boundary::boundary(y_a, y_b, res)
    void boundary(const State& ya, const State& yb, State& res) const {
        for (size_t i = 0; i < side.size(); ++i) res[i] = (side[i] == 0 ? ya[comp[i]] : yb[comp[i]]) - value[i];
    }
};

struct BvpResult {
    int status = DEGPU_COMPLETE;
    Result final;       // the last IVP solved: the final solve, or the one that failed
    State y_a;          // converged initial state
    int64_t iterations = 0, jacobian = 0;
    int64_t fevals = 0, accepted = 0, rejected = 0;  // totals over every IVP
};

// f64::max folded from zero over |r_i| (a NaN component is skipped)
inline double max_norm(const std::vector<double>& r) {
    double m = 0.0;
    for (double v : r) m = std::fmax(m, std::fabs(v));
    return m;
}

// src/linalg/lu.rs:67-240, dense storage (row-major a[i*n + j]): partial pivoting, negated
// multipliers below the diagonal, the pivot row swapped column by column. False when singular.
inline bool lu_decomp(std::vector<double>& a, int n, std::vector<int>& ip) {
    if (n == 1) {
        if (a[0] == 0.0) return false;
        ip[0] = 0;
        return true;
    }
    for (int k = 0; k < n - 1; ++k) {
        int m = k;
        double max_val = std::fabs(a[k * n + k]);
        for (int i = k + 1; i < n; ++i) {
            const double v = std::fabs(a[i * n + k]);
            if (v > max_val) {
                max_val = v;
                m = i;
            }
        }
        ip[k] = m;
        const double pivot = a[m * n + k];
        if (pivot == 0.0) return false;
        if (m != k) std::swap(a[m * n + k], a[k * n + k]);
        const double t = 1.0 / pivot;
        for (int i = k + 1; i < n; ++i) a[i * n + k] = -a[i * n + k] * t;
        for (int j = k + 1; j < n; ++j) {
            const double tj = a[m * n + j];
            if (m != k) std::swap(a[m * n + j], a[k * n + j]);
            if (tj != 0.0)
                for (int i = k + 1; i < n; ++i) a[i * n + j] = a[i * n + j] + a[i * n + k] * tj;
        }
    }
    return a[(n - 1) * n + (n - 1)] != 0.0;
}

// src/traits.rs:108-155
inline void lin_solve(const std::vector<double>& lu, int n, std::vector<double>& b, const std::vector<int>& ip) {
    if (n == 1) {
        b[0] = b[0] / lu[0];
        return;
    }
    for (int k = 0; k < n - 1; ++k) {
        const int m = ip[k];
        std::swap(b[k], b[m]);
        const double pv = b[k];
        for (int i = k + 1; i < n; ++i) b[i] = b[i] + lu[i * n + k] * pv;
    }
    for (int kb = 1; kb < n; ++kb) {
        const int k = n - kb;
        const double xk = b[k] / lu[k * n + k];
        b[k] = xk;
        const double neg = -xk;
        for (int i = 0; i < k; ++i) b[i] = b[i] + lu[i * n + k] * neg;
    }
    b[0] = b[0] / lu[0];
}

struct BvpSolver {
    int method;  // ERK method of the inner IVPs
    const Ode& ode;
    Settings set;
    Math math;
    bool hairer_dense = false;
    BvpResult out;

    // One IVP; false (with out.status / out.final set) when it fails, as the crate's `?` does.
    bool ivp(double a, double b, const State& y0, const std::vector<double>* t_eval, Result& r) {
        Settings s = set;
        r = solve_one(method, ode, a, b, y0, s, math, t_eval, hairer_dense);
        out.fevals += r.fevals;
        out.accepted += r.accepted;
        out.rejected += r.rejected;
        if (r.outcome.status != DEGPU_COMPLETE) {
            out.status = r.outcome.status;
            out.final = r;
            return false;
        }
        return true;
    }

    // SingleShooting::solve (single.rs:84-176)
    void single(const BvpSpec& bvp, double t0, double tf, const State& guess, const std::vector<double>* t_eval) {
        const int dim = (int)guess.size();
        State y = guess, residual(dim, 0.0);
        std::vector<double> jac(dim * dim);
        std::vector<int> ip(dim);
        const double eps = std::sqrt(std::numeric_limits<double>::epsilon());
        for (int it = 0; it < bvp.max_iterations; ++it) {
            Result r;
            if (!ivp(t0, tf, y, nullptr, r)) return;
            bvp.boundary(y, r.y_final, residual);
            if (max_norm(residual) <= bvp.tolerance) {
                out.y_a = y;
                ivp(t0, tf, y, t_eval, out.final);
                if (out.final.outcome.status == DEGPU_COMPLETE) out.status = DEGPU_COMPLETE;
                return;
            }
            for (int j = 0; j < dim; ++j) {
                State yp = y;
                const double yj = y[j];
                const double pert = eps * std::fmax(std::fabs(yj), 1.0);
                yp[j] = yj + pert;
                Result rp;
                if (!ivp(t0, tf, yp, nullptr, rp)) return;
                State resp = residual;
                bvp.boundary(yp, rp.y_final, resp);
                out.jacobian += 1;
                for (int i = 0; i < dim; ++i) jac[i * dim + j] = (resp[i] - residual[i]) / pert;
            }
            std::vector<double> step(dim);
            for (int i = 0; i < dim; ++i) step[i] = -residual[i];
            if (!lu_decomp(jac, dim, ip)) {
                out.status = DEGPU_ERR_LINEAR_ALGEBRA;
                out.final.t_final = t0;
                out.final.y_final = y;
                return;
            }
            lin_solve(jac, dim, step, ip);
            out.iterations += 1;
            for (int i = 0; i < dim; ++i) y[i] = y[i] + step[i];
        }
        out.status = DEGPU_ERR_MAX_STEPS;  // Error::MaxSteps { t: t0, y: y_guess }
        out.final.t_final = t0;
        out.final.y_final = guess;
    }

    // MultipleShooting::residual (multiple.rs:127-170)
    bool residual(const BvpSpec& bvp, const std::vector<double>& mesh, const std::vector<State>& nodes,
                  std::vector<double>& res) {
        const int dim = (int)nodes[0].size();
        res.clear();
        State br(dim, 0.0);
        bvp.boundary(nodes[0], nodes[nodes.size() - 1], br);
        for (int i = 0; i < dim; ++i) res.push_back(br[i]);
        for (int s = 0; s < bvp.segments; ++s) {
            Result r;
            if (!ivp(mesh[s], mesh[s + 1], nodes[s], nullptr, r)) return false;
            for (int i = 0; i < dim; ++i) res.push_back(r.y_final[i] - nodes[s + 1][i]);
        }
        return true;
    }

    // MultipleShooting::solve (multiple.rs:190-300)
    void multiple(const BvpSpec& bvp, double t0, double tf, const State& guess, const std::vector<double>* t_eval) {
        const int dim = (int)guess.size();
        const int segs = bvp.segments;
        if (segs < 1) {
            out.status = DEGPU_ERR_BAD_INPUT;
            return;
        }
        const int unknowns = (segs + 1) * dim;
        // mesh (multiple.rs:83-107): t0 + span * i / m
        std::vector<double> mesh;
        const double span = tf - t0;
        for (int i = 0; i <= segs; ++i) mesh.push_back(t0 + span * (double)i / (double)segs);
        const double eps = std::sqrt(std::numeric_limits<double>::epsilon());
        // initial_nodes (multiple.rs:108-126): one IVP over [t0, tf] with output at the mesh
        Result r0;
        if (!ivp(t0, tf, guess, &mesh, r0)) return;
        std::vector<State> nodes(segs + 1);
        for (int i = 0; i <= segs; ++i) {
            if (std::isnan(r0.dense[i][0])) {  // not every mesh node was produced
                out.status = DEGPU_ERR_BAD_INPUT;
                out.final.t_final = t0;
                out.final.y_final = guess;
                return;
            }
            nodes[i] = r0.dense[i];
        }
        std::vector<double> jac((size_t)unknowns * unknowns);
        std::vector<int> ip(unknowns);
        std::vector<double> res, resp;
        for (int it = 0; it < bvp.max_iterations; ++it) {
            if (!residual(bvp, mesh, nodes, res)) return;
            if (max_norm(res) <= bvp.tolerance) {
                out.y_a = nodes[0];
                ivp(t0, tf, nodes[0], t_eval, out.final);
                if (out.final.outcome.status == DEGPU_COMPLETE) out.status = DEGPU_COMPLETE;
                return;
            }
            for (int j = 0; j < unknowns; ++j) {
                const int node_idx = j / dim, ci = j % dim;
                std::vector<State> pn = nodes;
                const double yj = pn[node_idx][ci];
                const double pert = eps * std::fmax(std::fabs(yj), 1.0);
                pn[node_idx][ci] = yj + pert;
                if (!residual(bvp, mesh, pn, resp)) return;
                out.jacobian += 1;
                for (int i = 0; i < unknowns; ++i) jac[(size_t)i * unknowns + j] = (resp[i] - res[i]) / pert;
            }
            std::vector<double> step(unknowns);
            for (int i = 0; i < unknowns; ++i) step[i] = -res[i];
            if (!lu_decomp(jac, unknowns, ip)) {
                out.status = DEGPU_ERR_LINEAR_ALGEBRA;
                out.final.t_final = t0;
                out.final.y_final = nodes[0];
                return;
            }
            lin_solve(jac, unknowns, step, ip);
            out.iterations += 1;
            for (int k = 0; k <= segs; ++k)
                for (int c = 0; c < dim; ++c) nodes[k][c] = nodes[k][c] + step[k * dim + c];
        }
        out.status = DEGPU_ERR_MAX_STEPS;  // Error::MaxSteps { t: t0, y: nodes[0] }
        out.final.t_final = t0;
        out.final.y_final = nodes[0];
    }
};

}  // namespace oracle
