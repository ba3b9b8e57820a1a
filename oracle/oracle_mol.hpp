// oracle_mol.hpp — TEST INFRASTRUCTURE ONLY.  CPU restatement of the crate's method-of-lines
// finite-difference semi-discretisation:
//   StructuredGrid ............ src/pde/grid.rs:23-145 (vertex-centred, axis 0 fastest)
//   BoundaryCondition ......... src/pde/boundary.rs:11-17 (Dirichlet / Neumann)
//   SemiDiscretePde::diff ..... src/pde/semi_discrete.rs:102-287 (FiniteDifference scheme)
// plus one extension the crate does not have: a periodic face, whose neighbour wraps around the
// grid and whose spacing is given explicitly (a periodic grid of N nodes has spacing L/N).
#pragma once

#include <array>
#include <vector>

#include "oracle.hpp"

namespace oracle {

enum class BcKind { Dirichlet, Neumann, Periodic };

struct Bc {
    BcKind kind = BcKind::Neumann;
    std::vector<double> value;  // local_len values (Dirichlet value or Neumann gradient)
};

// PDE in conservative form u_t = div(flux(t,x,u,grad u)) + source(t,x,u) (src/pde/pde.rs:16-31).
struct Pde {
    virtual ~Pde() = default;
    // grad[axis] has local_len entries; only grad[axis] of the requested axis is non-zero.
    virtual void flux(double t, const double* x, const double* u, const std::vector<State>& grad,
                      std::vector<State>& flux) const = 0;
    virtual void source(double t, const double* x, const double* u, double* s, int L) const {
        for (int c = 0; c < L; ++c) s[c] = 0.0;  // default source fills zero (pde.rs:28-30)
    }
};

struct SemiDiscrete : Ode {
    const Pde* pde;
    int D;                      // 1 or 2
    int L;                      // local_len
    std::array<int, 2> nodes;   // per axis
    std::array<double, 2> lower, dx;
    std::array<Bc, 2> lo_bc, hi_bc;
    std::vector<char> dirichlet_mask;

    size_t len() const { return (size_t)nodes[0] * (D == 2 ? nodes[1] : 1); }

    // grid.rs:83-91
    std::array<int, 2> multi_index(size_t flat) const {
        std::array<int, 2> idx{0, 0};
        for (int a = 0; a < D; ++a) {
            idx[a] = (int)(flat % nodes[a]);
            flat /= nodes[a];
        }
        return idx;
    }
    size_t flat_index(std::array<int, 2> idx) const {  // grid.rs:94-106
        size_t flat = 0, stride = 1;
        for (int a = 0; a < D; ++a) {
            flat += (size_t)idx[a] * stride;
            stride *= nodes[a];
        }
        return flat;
    }
    // grid.rs:121-134, with the periodic wrap extension
    bool neighbor(size_t node, int axis, int off, size_t& out) const {
        auto idx = multi_index(node);
        bool periodic = lo_bc[axis].kind == BcKind::Periodic;
        if (off == -1) {
            if (idx[axis] > 0) idx[axis] -= 1;
            else if (periodic) idx[axis] = nodes[axis] - 1;
            else return false;
        } else {
            if (idx[axis] + 1 < nodes[axis]) idx[axis] += 1;
            else if (periodic) idx[axis] = 0;
            else return false;
        }
        out = flat_index(idx);
        return true;
    }
    int boundary_side(size_t node, int axis) const {  // grid.rs:136-145: -1 lower, +1 upper, 0 none
        auto idx = multi_index(node);
        if (idx[axis] == 0) return -1;
        if (idx[axis] + 1 == nodes[axis]) return 1;
        return 0;
    }
    void point(size_t node, double* x) const {  // grid.rs:109-114
        auto idx = multi_index(node);
        for (int a = 0; a < D; ++a) x[a] = lower[a] + dx[a] * (double)idx[a];
    }

    void build_mask() {  // semi_discrete.rs:51-62
        dirichlet_mask.assign(len(), 0);
        for (size_t node = 0; node < len(); ++node) {
            for (int a = 0; a < D; ++a) {
                int side = boundary_side(node, a);
                const Bc* bc = side < 0 ? &lo_bc[a] : side > 0 ? &hi_bc[a] : nullptr;
                if (bc && bc->kind == BcKind::Dirichlet) dirichlet_mask[node] = 1;
            }
        }
    }

    // semi_discrete.rs:150-172: one-sided gradient at the lower or upper face
    State directional_gradient(const State& y, size_t node, int axis, int side) const {
        State g(L);
        size_t nb;
        bool has = neighbor(node, axis, side, nb);
        if (has) {
            for (int c = 0; c < L; ++c) {
                double u = y[node * L + c], o = y[nb * L + c];
                g[c] = side < 0 ? (u - o) / dx[axis] : (o - u) / dx[axis];
            }
            return g;
        }
        const Bc& bc = side < 0 ? lo_bc[axis] : hi_bc[axis];
        if (bc.kind == BcKind::Neumann) return bc.value;
        for (int c = 0; c < L; ++c) {  // Dirichlet face
            double u = y[node * L + c], v = bc.value[c];
            g[c] = side < 0 ? (u - v) / dx[axis] : (v - u) / dx[axis];
        }
        return g;
    }

    // semi_discrete.rs:181-190
    State fd_flux(double t, const State& y, size_t node, int axis, int side) const {
        double x[2];
        point(node, x);
        std::vector<State> grad(D, State(L, 0.0));
        grad[axis] = directional_gradient(y, node, axis, side);
        std::vector<State> fl(D, State(L, 0.0));
        pde->flux(t, x, &y[node * L], grad, fl);
        return fl[axis];
    }

    // semi_discrete.rs:250-287
    void diff(double t, const State& y, State& dudt) const override {
        for (size_t node = 0; node < len(); ++node) {
            if (dirichlet_mask[node]) {
                for (int c = 0; c < L; ++c) dudt[node * L + c] = 0.0;
                continue;
            }
            double x[2];
            point(node, x);
            State der(L, 0.0);
            pde->source(t, x, &y[node * L], der.data(), L);
            for (int a = 0; a < D; ++a) {
                State flo = fd_flux(t, y, node, a, -1);
                State fhi = fd_flux(t, y, node, a, +1);
                for (int c = 0; c < L; ++c) der[c] = der[c] + (fhi[c] - flo[c]) / dx[a];
            }
            for (int c = 0; c < L; ++c) dudt[node * L + c] = der[c];
        }
    }
};

// tests/pde/method_of_lines.rs:3-11
struct HeatPde : Pde {
    double alpha;
    explicit HeatPde(double a) : alpha(a) {}
    void flux(double, const double*, const double*, const std::vector<State>& grad,
              std::vector<State>& fl) const override {
        fl[0][0] = alpha * grad[0][0];
    }
};

// Diffusion with one diffusivity per field (HeatEquation is the one-field case): flux_c =
// kappa_c grad_c along the axis, no source.
struct DiffusionPde : Pde {
    std::vector<double> kappa;
    void flux(double, const double*, const double*, const std::vector<State>& grad,
              std::vector<State>& fl) const override {
        for (size_t a = 0; a < grad.size(); ++a)
            for (size_t c = 0; c < kappa.size(); ++c) fl[a][c] = kappa[c] * grad[a][c];
    }
};

// tests/pde/method_of_lines.rs:13-34
struct CoupledDiffusionPde : Pde {
    double d0, d1;
    // the crate's test system is one-dimensional (flux[0] only); on more axes each axis diffuses
    // alike
    void flux(double, const double*, const double*, const std::vector<State>& grad,
              std::vector<State>& fl) const override {
        for (size_t a = 0; a < grad.size(); ++a) {
            fl[a][0] = d0 * grad[a][0];
            fl[a][1] = d1 * grad[a][1];
        }
    }
    void source(double, const double*, const double* u, double* s, int) const override {
        s[0] = u[1] - u[0];
        s[1] = u[0] - u[1];
    }
};

// 2-D Gray–Scott reaction–diffusion in the crate's PDE form: flux = (Du grad u, Dv grad v) per
// axis; source = (-u v^2 + F (1 - u), u v^2 - (F + k) v) with u v^2 evaluated as (u*v)*v.
struct GrayScottPde : Pde {
    double Du, Dv, F, k;
    void flux(double, const double*, const double*, const std::vector<State>& grad,
              std::vector<State>& fl) const override {
        for (size_t a = 0; a < grad.size(); ++a) {
            fl[a][0] = Du * grad[a][0];
            fl[a][1] = Dv * grad[a][1];
        }
    }
    void source(double, const double*, const double* u, double* s, int) const override {
        double uu = u[0], vv = u[1];
        double uvv = uu * vv * vv;
        s[0] = -uvv + F * (1.0 - uu);
        s[1] = uvv - (F + k) * vv;
    }
};

}  // namespace oracle
