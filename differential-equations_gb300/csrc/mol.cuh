// mol.cuh — the crate's method-of-lines semi-discretisation on the device, for any built-in PDE
// in conservative form  u_t = div(flux(t, x, u, grad u)) + source(t, x, u)  on a structured grid
// of one or two axes with Dirichlet, Neumann or periodic faces.
//
// Right-hand side (SemiDiscretePde::diff, src/pde/semi_discrete.rs:250-287), per node, in the
// crate's order:
//   - a node on a Dirichlet face of any axis has du/dt = 0 (the mask of :51-62);
//   - der = source(t, x, u);
//   - for axis 0, 1: flux_lo = flux(t, x, u, g_lo)[axis], flux_hi = flux(t, x, u, g_hi)[axis],
//     der_c = der_c + (flux_hi_c - flux_lo_c) / dx  (finite_difference_flux, :181-190);
//   - one-sided gradients (directional_gradient, :150-172): (u - u_lo) / dx and (u_hi - u) / dx
//     with the neighbour when there is one; at a face without one, a Neumann face gives its
//     prescribed gradient and a Dirichlet face (u - v) / dx or (v - u) / dx against its value.
//   A periodic face (an extension; the crate has Dirichlet and Neumann faces) wraps the
//   neighbour around the axis.  When dx is a power of two, "/ dx" is the exact multiplication
//   by 1/dx.
// Grid (StructuredGrid, src/pde/grid.rs:83-145): node = i0 + n0 i1 (axis 0 fastest), point
// x_a = lower_a + dx_a i_a; the state holds the L fields of a node together: y[node * L + c].
//
// Time stepping: the crate's fixed RK4 step (src/methods/erk/fixed/ordinary.rs:58-138), four
// passes per step with y_next = (((y + (b0 h) k0) + (b1 h) k1) + (b2 h) k2) + (b3 h) k3 carried in
// an accumulator:
//   pass 1: k1 = f(t + h/2, y + (h/2) k0)      acc = (y + (b0 h) k0) + (b1 h) k1
//   pass 2: k2 = f(t + h/2, y + (h/2) k1)      acc = acc + (b2 h) k2
//   pass 3: k3 = f(t + h,   y + h k2)          y_next = acc + (b3 h) k3
//   pass 0: k0 = f(t, y)                       (the derivative at the new point)
// The stage states of a node's neighbours are formed where they are read (y + (a h) k), so a
// pass reads y and k at the node and its 2 D neighbours through L1/L2 and writes its outputs once.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <map>
#include <tuple>
#include <type_traits>

#include "../../include/degpu.h"

namespace degpu {

// Geometry, faces and parameters of a solve, in the arithmetic type T.
template <class T>
struct MolGeom {
    int n[2];
    int64_t N;        // nodes
    T dx[2], inv_dx[2];
    bool pow2[2];
    double lower[2], dxd[2];  // FP64 copies for the node coordinates
    int bck[2][2];            // [axis][side] face kind
    T bcv[2][2][DEGPU_MOL_MAX_FIELDS];
    T prm[DEGPU_MOL_MAX_PARAMS];
};

// One pass of the RK4 step (or a plain right-hand-side evaluation with pass = 0, kin = NULL).
template <class T>
struct MolPass {
    int pass;
    double t;       // stage time
    const T* y;
    const T* kin;   // k_{i-1}: the stage state is y + ah kin (NULL: y itself)
    T ah;
    T* kout;        // k_i
    const T* k0;    // pass 1: k0 for the accumulation
    T bh0, bh1;     // pass 1: b0 h, b1 h; passes 2, 3: b_i h in bh0
    T* acc;
    T* ynext;       // pass 3
};

template <class T, int AX>
__device__ __forceinline__ T mol_ddx(T v, const MolGeom<T>& g) {
    return g.pow2[AX] ? v * g.inv_dx[AX] : v / g.dx[AX];
}

// Built-in PDEs (the PDE trait's flux and source, src/pde/pde.rs:16-31), each with the field
// count L.  flux(axis, u, grad, f): the crate's flux with the gradient along `axis` only (the
// other axes' gradients are zero there), f[c] = flux[axis][c].

// Diffusion with one diffusivity per field: flux_c = prm[c] grad_c, no source
// (tests/pde/method_of_lines.rs:3-11 is the one-field case, HeatEquation).
template <int NF>
struct PdeDiffusion {
    static constexpr int L = NF;
    template <class T>
    __device__ static __forceinline__ void source(double, const double*, const T*, T* s, const T*) {
#pragma unroll
        for (int c = 0; c < L; ++c) s[c] = (T)0;
    }
    template <class T>
    __device__ static __forceinline__ void flux(int, const double*, const T*, const T* gr, T* f, const T* prm) {
#pragma unroll
        for (int c = 0; c < L; ++c) f[c] = prm[c] * gr[c];
    }
};

// Two diffusing fields exchanging mass: flux_c = prm[c] grad_c, source = (u1 - u0, u0 - u1)
// (tests/pde/method_of_lines.rs:13-34, CoupledDiffusion).
struct PdeCoupledDiffusion {
    static constexpr int L = 2;
    template <class T>
    __device__ static __forceinline__ void source(double, const double*, const T* u, T* s, const T*) {
        s[0] = u[1] - u[0];
        s[1] = u[0] - u[1];
    }
    template <class T>
    __device__ static __forceinline__ void flux(int, const double*, const T*, const T* gr, T* f, const T* prm) {
        f[0] = prm[0] * gr[0];
        f[1] = prm[1] * gr[1];
    }
};

// Gray-Scott reaction-diffusion, prm = (Du, Dv, F, k): flux = (Du grad u, Dv grad v), source =
// (-u v^2 + F (1 - u), u v^2 - (F + k) v) with u v^2 as (u v) v.
struct PdeGrayScott {
    static constexpr int L = 2;
    template <class T>
    __device__ static __forceinline__ void source(double, const double*, const T* u, T* s, const T* prm) {
        const T uvv = u[0] * u[1] * u[1];
        s[0] = -uvv + prm[2] * ((T)1 - u[0]);
        s[1] = uvv - (prm[2] + prm[3]) * u[1];
    }
    template <class T>
    __device__ static __forceinline__ void flux(int, const double*, const T*, const T* gr, T* f, const T* prm) {
        f[0] = prm[0] * gr[0];
        f[1] = prm[1] * gr[1];
    }
};

// Stage state of node q: y + ah kin (or y).
template <class T, int L>
__device__ __forceinline__ void mol_state(const MolPass<T>& P, int64_t q, T* u) {
#pragma unroll
    for (int c = 0; c < L; ++c) {
        const T yv = __ldg(P.y + q * L + c);
        u[c] = P.kin ? yv + P.ah * __ldg(P.kin + q * L + c) : yv;
    }
}

// f at node (i0, i1) of a DIM-axis grid.
template <class T, class Pde, int DIM>
__device__ __forceinline__ void mol_rhs_at(int i0, int i1, const MolGeom<T>& g, const MolPass<T>& P, T* der) {
    constexpr int L = Pde::L;
    const int idx[2] = {i0, i1};
    // the Dirichlet mask: a node on a Dirichlet face of any axis
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
        const bool lo = idx[a] == 0, hi = idx[a] + 1 == g.n[a];
        const int side = lo ? 0 : (hi ? 1 : -1);  // the lower face first, as grid.rs:136-145
        if (side >= 0 && g.bck[a][side] == DEGPU_BC_DIRICHLET) {
#pragma unroll
            for (int c = 0; c < L; ++c) der[c] = (T)0;
            return;
        }
    }
    const int64_t node = (int64_t)i0 + (DIM == 2 ? (int64_t)g.n[0] * i1 : 0);
    double x[2];
#pragma unroll
    for (int a = 0; a < DIM; ++a) x[a] = g.lower[a] + g.dxd[a] * (double)idx[a];
    T u[L];
    mol_state<T, L>(P, node, u);
    Pde::source(P.t, x, u, der, g.prm);
    auto axis = [&](auto ax) {
        constexpr int a = decltype(ax)::value;
        T glo[L], ghi[L], flo[L], fhi[L];
        // lower side
        if (idx[a] > 0 || g.bck[a][0] == DEGPU_BC_PERIODIC) {
            const int j = idx[a] > 0 ? idx[a] - 1 : g.n[a] - 1;
            const int64_t q = a == 0 ? node - idx[0] + j : (int64_t)idx[0] + (int64_t)g.n[0] * j;
            T o[L];
            mol_state<T, L>(P, q, o);
#pragma unroll
            for (int c = 0; c < L; ++c) glo[c] = mol_ddx<T, a>(u[c] - o[c], g);
        } else if (g.bck[a][0] == DEGPU_BC_NEUMANN) {
#pragma unroll
            for (int c = 0; c < L; ++c) glo[c] = g.bcv[a][0][c];
        } else {
#pragma unroll
            for (int c = 0; c < L; ++c) glo[c] = mol_ddx<T, a>(u[c] - g.bcv[a][0][c], g);
        }
        // upper side
        if (idx[a] + 1 < g.n[a] || g.bck[a][1] == DEGPU_BC_PERIODIC) {
            const int j = idx[a] + 1 < g.n[a] ? idx[a] + 1 : 0;
            const int64_t q = a == 0 ? node - idx[0] + j : (int64_t)idx[0] + (int64_t)g.n[0] * j;
            T o[L];
            mol_state<T, L>(P, q, o);
#pragma unroll
            for (int c = 0; c < L; ++c) ghi[c] = mol_ddx<T, a>(o[c] - u[c], g);
        } else if (g.bck[a][1] == DEGPU_BC_NEUMANN) {
#pragma unroll
            for (int c = 0; c < L; ++c) ghi[c] = g.bcv[a][1][c];
        } else {
#pragma unroll
            for (int c = 0; c < L; ++c) ghi[c] = mol_ddx<T, a>(g.bcv[a][1][c] - u[c], g);
        }
        Pde::flux(a, x, u, glo, flo, g.prm);
        Pde::flux(a, x, u, ghi, fhi, g.prm);
#pragma unroll
        for (int c = 0; c < L; ++c) der[c] = der[c] + mol_ddx<T, a>(fhi[c] - flo[c], g);
    };
    axis(std::integral_constant<int, 0>{});
    if constexpr (DIM == 2) axis(std::integral_constant<int, 1>{});
}

// One pass over every node: k_i, and the accumulator / next state of the pass.
template <class T, class Pde, int DIM>
__global__ void __launch_bounds__(256) mol_pass_kernel(MolGeom<T> g, MolPass<T> P) {
    constexpr int L = Pde::L;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; node < g.N; node += stride) {
        const int i0 = (int)(node % g.n[0]);
        const int i1 = DIM == 2 ? (int)(node / g.n[0]) : 0;
        T k[L];
        mol_rhs_at<T, Pde, DIM>(i0, i1, g, P, k);
#pragma unroll
        for (int c = 0; c < L; ++c) {
            const int64_t e = node * L + c;
            if (P.pass != 3) P.kout[e] = k[c];
            if (P.pass == 1) {
                const T a0 = P.y[e] + P.bh0 * P.k0[e];
                P.acc[e] = a0 + P.bh1 * k[c];
            } else if (P.pass == 2) {
                P.acc[e] = P.acc[e] + P.bh0 * k[c];
            } else if (P.pass == 3) {
                P.ynext[e] = P.acc[e] + P.bh0 * k[c];
            }
        }
    }
}

// ---- host side -------------------------------------------------------------------------

// Argument checks shared by the entry points.
inline bool mol_valid(const degpu_mol* m) {
    if (!m || (m->dims != 1 && m->dims != 2)) return false;
    if (m->fields < 1 || m->fields > DEGPU_MOL_MAX_FIELDS) return false;
    for (int a = 0; a < m->dims; ++a) {
        if (m->nodes[a] < 2 || !(m->dx[a] > 0.0) || !isfinite(m->dx[a])) return false;
        for (int sd = 0; sd < 2; ++sd)
            if (m->bc_kind[a][sd] < DEGPU_BC_DIRICHLET || m->bc_kind[a][sd] > DEGPU_BC_PERIODIC) return false;
        if ((m->bc_kind[a][0] == DEGPU_BC_PERIODIC) != (m->bc_kind[a][1] == DEGPU_BC_PERIODIC)) return false;
    }
    return true;
}

template <class T>
MolGeom<T> mol_geom(const degpu_mol* m) {
    MolGeom<T> g{};
    g.n[0] = m->nodes[0];
    g.n[1] = m->dims == 2 ? m->nodes[1] : 1;
    g.N = (int64_t)g.n[0] * g.n[1];
    for (int a = 0; a < 2; ++a) {
        const double dx = a < m->dims ? m->dx[a] : 1.0;
        int e = 0;
        g.pow2[a] = frexp(dx, &e) == 0.5;
        g.dx[a] = (T)dx;
        g.inv_dx[a] = (T)(1.0 / dx);
        g.lower[a] = m->lower[a];
        g.dxd[a] = dx;
        for (int sd = 0; sd < 2; ++sd) {
            g.bck[a][sd] = a < m->dims ? m->bc_kind[a][sd] : DEGPU_BC_NEUMANN;
            for (int c = 0; c < DEGPU_MOL_MAX_FIELDS; ++c) g.bcv[a][sd][c] = (T)m->bc_value[a][sd][c];
        }
    }
    for (int q = 0; q < DEGPU_MOL_MAX_PARAMS; ++q) g.prm[q] = (T)m->params[q];
    return g;
}

// The right-hand side and the RK4 driver of one (T, PDE, axes) combination.
template <class T, class Pde, int DIM>
struct MolDriver {
    static cudaError_t launch(const MolGeom<T>& g, const MolPass<T>& P, cudaStream_t s) {
        const int64_t blocks = (g.N + 255) / 256;
        const unsigned grid = (unsigned)(blocks < 152 * 16 ? blocks : 152 * 16);
        mol_pass_kernel<T, Pde, DIM><<<grid, 256, 0, s>>>(g, P);
        return cudaGetLastError();
    }

    static degpu_status rhs(const degpu_mol* m, double t, const void* y, void* dydt, cudaStream_t s) {
        const MolGeom<T> g = mol_geom<T>(m);
        MolPass<T> P{};
        P.pass = 0;
        P.t = t;
        P.y = (const T*)y;
        P.kout = (T*)dydt;
        return launch(g, P, s) == cudaSuccess ? DEGPU_OK : DEGPU_CUDA_ERROR;
    }

    // The crate's driver loop (solve_ivp.rs:191-266) over fixed RK4 steps (fixed/ordinary.rs:16-138):
    // k0 = f(t0, y0); before a step that would pass tf, h = tf - t (done if |tf - t| < 10 eps);
    // after it, done once |tf - t| <= 10 eps.  The step times are formed on the host in the
    // crate's order (t + c_i h, t + h).
    static degpu_status rk4(const degpu_mol* m, double t0, double tf, double h, void* y, int64_t* steps,
                            cudaStream_t s) {
        const MolGeom<T> g = mol_geom<T>(m);
        const size_t E = (size_t)g.N * Pde::L;
        T* blk = nullptr;
        if (cudaMallocAsync((void**)&blk, 5 * E * sizeof(T), s) != cudaSuccess) return DEGPU_OOM;
        T* k[3] = {blk, blk + E, blk + 2 * E};
        T* acc = blk + 3 * E;
        T* ys[2] = {(T*)y, blk + 4 * E};
        int cur = 0;
        degpu_status st = DEGPU_OK;
        auto run = [&](const MolPass<T>& P) {
            if (st == DEGPU_OK && launch(g, P, s) != cudaSuccess) st = DEGPU_CUDA_ERROR;
        };
        const double eps10 = 2.220446049250313e-16 * 10.0;
        const double dir = tf > t0 ? 1.0 : -1.0;
        const double b0 = 1.0 / 6.0, b1 = 1.0 / 3.0, b2 = 1.0 / 3.0, b3 = 1.0 / 6.0;
        double t = t0;
        int64_t n = 0;
        {
            MolPass<T> P{};
            P.pass = 0;
            P.t = t;
            P.y = ys[cur];
            P.kout = k[0];
            run(P);
        }
        while (st == DEGPU_OK) {
            if ((t + h - tf) * dir > 0.0) {
                const double hn = tf - t;
                if (fabs(hn) < eps10) break;
                h = hn;
            }
            MolPass<T> P{};
            P.y = ys[cur];
            P.pass = 1;
            P.t = t + 0.5 * h;
            P.kin = k[0];
            P.ah = (T)(0.5 * h);
            P.kout = k[1];
            P.k0 = k[0];
            P.bh0 = (T)(b0 * h);
            P.bh1 = (T)(b1 * h);
            P.acc = acc;
            run(P);
            P.pass = 2;
            P.t = t + 0.5 * h;
            P.kin = k[1];
            P.kout = k[2];
            P.bh0 = (T)(b2 * h);
            run(P);
            P.pass = 3;
            P.t = t + 1.0 * h;
            P.kin = k[2];
            P.ah = (T)(1.0 * h);
            P.bh0 = (T)(b3 * h);
            P.ynext = ys[1 - cur];
            run(P);
            cur = 1 - cur;
            t = t + h;
            n += 1;
            MolPass<T> Q{};
            Q.pass = 0;
            Q.t = t;
            Q.y = ys[cur];
            Q.kout = k[0];
            run(Q);
            if (fabs(tf - t) <= eps10) break;
        }
        if (st == DEGPU_OK && cur == 1 &&
            cudaMemcpyAsync(y, ys[1], E * sizeof(T), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            st = DEGPU_CUDA_ERROR;
        cudaFreeAsync(blk, s);
        if (steps) *steps = n;
        return st;
    }
};

// Registered drivers, keyed by (pde_id, axes, fields, arithmetic class): class 0 the crate's
// order without contraction (DEGPU_FP64_PARITY), 1 FP64 with contraction, 2 FP32.
struct MolOps {
    degpu_status (*rhs)(const degpu_mol*, double, const void*, void*, cudaStream_t);
    degpu_status (*rk4)(const degpu_mol*, double, double, double, void*, int64_t*, cudaStream_t);
};
std::map<std::tuple<int, int, int, int>, MolOps>& mol_registry();

template <class T, class Pde, int DIM>
void register_mol(int pde_id, int cls) {
    mol_registry()[{pde_id, DIM, Pde::L, cls}] = MolOps{&MolDriver<T, Pde, DIM>::rhs, &MolDriver<T, Pde, DIM>::rk4};
}

template <class T>
void register_mol_all(int cls) {
    register_mol<T, PdeDiffusion<1>, 1>(DEGPU_PDE_DIFFUSION, cls);
    register_mol<T, PdeDiffusion<2>, 1>(DEGPU_PDE_DIFFUSION, cls);
    register_mol<T, PdeDiffusion<1>, 2>(DEGPU_PDE_DIFFUSION, cls);
    register_mol<T, PdeDiffusion<2>, 2>(DEGPU_PDE_DIFFUSION, cls);
    register_mol<T, PdeCoupledDiffusion, 1>(DEGPU_PDE_COUPLED_DIFFUSION, cls);
    register_mol<T, PdeCoupledDiffusion, 2>(DEGPU_PDE_COUPLED_DIFFUSION, cls);
    register_mol<T, PdeGrayScott, 1>(DEGPU_PDE_GRAY_SCOTT, cls);
    register_mol<T, PdeGrayScott, 2>(DEGPU_PDE_GRAY_SCOTT, cls);
}

void register_mol_parity();
void register_mol_fast();

}  // namespace degpu
