// bvp.cu — boundary value problems by shooting over an ensemble (degpu_solve_bvp_host).
//
// The crate's shooting methods (src/methods/bvp/shooting/single.rs, multiple.rs) run one Newton
// iteration as a sequence of IVP solves: the shot from the current unknowns and one shot per
// Jacobian column. Here the whole Newton loop of the batch stays on the device:
//   * a build kernel writes every shot of one pass (every unfinished instance, every column) into
//     one ensemble batch, gathering each instance's parameters and tolerances;
//   * the ensemble solve runs the pass (degpu_solve_ensemble on device pointers);
//   * a Newton kernel (one thread per instance) forms the residual, the convergence test, the
//     forward-difference Jacobian, the crate's dense LU and the update, in the crate's operation
//     order (this translation unit is compiled without multiply-add contraction);
//   * a compaction kernel lists the instances still iterating for the next pass.
// The host only launches and reads one count per pass.
//
// Multiple shooting re-solves every segment for every Jacobian column in the crate, although a
// column perturbs one node and so changes one segment's IVP; the others give the same bits as the
// pass's base shots. Only the changed segment is solved here, and the function-evaluation and step
// counters of the unchanged segments are added again, so the totals equal the crate's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/degpu.h"

namespace {

constexpr double kSqrtEps = 1.4901161193847656e-08;  // sqrt(f64::EPSILON) = 2^-26
constexpr int kUMax = DEGPU_BVP_MAX_UNKNOWNS;
enum : int32_t { ACTIVE = 0, CONVERGED = 1, DONE = 2 };

// Per-instance Newton state and the batch's settings (device arrays, structure of arrays).
struct Dev {
    int64_t n;
    int dim, U, segs, np;
    double tol;
    const double *t0, *tf, *params, *rtol, *atol;  // the caller's inputs
    double* u;      // [U][n] unknowns: y(t0), or the mesh nodes
    double* guess;  // [dim][n]
    int32_t *phase, *status, *iters;
    double *t_err, *y_err;  // state reported on failure, y_err [dim][n]
    int64_t *fev, *acc, *rej, *jac;
    double* jm;  // [n][U*U] Jacobian scratch
    int32_t side[DEGPU_HYPERPLANE_MAX_DIM], comp[DEGPU_HYPERPLANE_MAX_DIM];
    double value[DEGPU_HYPERPLANE_MAX_DIM];
    double mesh[kUMax + 1];
};

// One pass of shots: inputs and outputs of an ensemble solve.
struct Shots {
    int64_t m;
    double *t0, *tf, *y0, *params, *rtol, *atol;  // y0 [dim][m], params [np][m]
    double *y_final, *t_final, *dense;            // y_final [dim][m]
    int64_t *acc, *rej, *fev;
    int32_t* status;
};

__device__ __forceinline__ double bnd(const Dev& d, int i, const double* ya, const double* yb) {
    // Boundary::boundary in the separated form r_i = y_side[comp_i] - value_i
    return (d.side[i] == 0 ? ya[d.comp[i]] : yb[d.comp[i]]) - d.value[i];
}

__device__ __forceinline__ void count(const Dev& d, const Shots& s, int64_t i, int64_t k) {
    d.fev[i] += s.fev[k];
    d.acc[i] += s.acc[k];
    d.rej[i] += s.rej[k];
}

__device__ __forceinline__ void fail(const Dev& d, int64_t i, int32_t st, double t, const double* y, int64_t ystride) {
    d.phase[i] = DONE;
    d.status[i] = st;
    d.t_err[i] = t;
    for (int c = 0; c < d.dim; ++c) d.y_err[(int64_t)c * d.n + i] = y[(int64_t)c * ystride];
}

// Dense LU with partial pivoting as src/linalg/lu.rs:185-240 forms it (row-major a, negated
// multipliers, pivot row swapped column by column), then the solve of src/traits.rs:108-155.
// False when a pivot is zero.
__device__ bool lu_solve(double* a, int n, double* b) {
    int ip[kUMax];
    if (n == 1) {
        if (a[0] == 0.0) return false;
        b[0] = b[0] / a[0];
        return true;
    }
    for (int k = 0; k + 1 < n; ++k) {
        int m = k;
        double best = fabs(a[k * n + k]);
        for (int i = k + 1; i < n; ++i)
            if (fabs(a[i * n + k]) > best) {
                best = fabs(a[i * n + k]);
                m = i;
            }
        ip[k] = m;
        const double pivot = a[m * n + k];
        if (pivot == 0.0) return false;
        if (m != k) {
            const double x = a[m * n + k];
            a[m * n + k] = a[k * n + k];
            a[k * n + k] = x;
        }
        const double inv = 1.0 / pivot;
        for (int i = k + 1; i < n; ++i) a[i * n + k] = -a[i * n + k] * inv;
        for (int j = k + 1; j < n; ++j) {
            const double tj = a[m * n + j];
            if (m != k) {
                const double x = a[m * n + j];
                a[m * n + j] = a[k * n + j];
                a[k * n + j] = x;
            }
            if (tj != 0.0)
                for (int i = k + 1; i < n; ++i) a[i * n + j] = a[i * n + j] + a[i * n + k] * tj;
        }
    }
    if (a[(n - 1) * n + (n - 1)] == 0.0) return false;
    for (int k = 0; k + 1 < n; ++k) {
        const double x = b[k];
        b[k] = b[ip[k]];
        b[ip[k]] = x;
        const double pv = b[k];
        for (int i = k + 1; i < n; ++i) b[i] = b[i] + a[i * n + k] * pv;
    }
    for (int k = n - 1; k >= 1; --k) {
        const double xk = b[k] / a[k * n + k];
        b[k] = xk;
        const double neg = -xk;
        for (int i = 0; i < k; ++i) b[i] = b[i] + a[i * n + k] * neg;
    }
    b[0] = b[0] / a[0];
    return true;
}

// src/traits.rs:93-99: f64::max folded from zero over |r_i|
__device__ __forceinline__ double max_norm(const double* r, int n) {
    double m = 0.0;
    for (int i = 0; i < n; ++i) m = fmax(m, fabs(r[i]));
    return m;
}

__global__ void k_init(Dev d, const double* y0) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    for (int c = 0; c < d.dim; ++c) {
        const double v = y0[(int64_t)c * d.n + i];
        d.guess[(int64_t)c * d.n + i] = v;
        d.u[(int64_t)c * d.n + i] = v;
    }
    d.phase[i] = ACTIVE;
    d.status[i] = DEGPU_COMPLETE;
    d.iters[i] = 0;
    d.fev[i] = d.acc[i] = d.rej[i] = d.jac[i] = 0;
}

// The instances whose phase is `want`, in any order (their work is independent).
__global__ void k_compact(const int32_t* phase, int64_t n, int32_t want, int64_t* list, unsigned long long* cnt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || phase[i] != want) return;
    list[atomicAdd(cnt, 1ull)] = i;
}

// Gathers one shot: the instance's parameters and tolerances, the start state and interval.
__device__ __forceinline__ void put_shot(const Dev& d, const Shots& s, int64_t k, int64_t i, double a, double b) {
    s.t0[k] = a;
    s.tf[k] = b;
    for (int q = 0; q < d.np; ++q) s.params[(int64_t)q * s.m + k] = d.params[(int64_t)q * d.n + i];
    s.rtol[k] = d.rtol[i];
    s.atol[k] = d.atol[i];
}

// single shooting: per instance the shot from u and one per column (u_j + sqrt(eps) max(|u_j|, 1))
__global__ void k_build_single(Dev d, const int64_t* act, int64_t nact, Shots s) {
    const int per = d.dim + 1;
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= nact * per) return;
    const int64_t i = act[k / per];
    const int j = (int)(k % per) - 1;
    put_shot(d, s, k, i, d.t0[i], d.tf[i]);
    for (int c = 0; c < d.dim; ++c) {
        double v = d.u[(int64_t)c * d.n + i];
        if (c == j) v = v + kSqrtEps * fmax(fabs(v), 1.0);
        s.y0[(int64_t)c * s.m + k] = v;
    }
}

// multiple shooting: per instance the segments from the nodes, then one shot per column whose
// node starts a segment (that segment from the perturbed node)
__global__ void k_build_multi(Dev d, const int64_t* act, int64_t nact, Shots s) {
    const int per = d.segs * (1 + d.dim);
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= nact * per) return;
    const int64_t i = act[k / per];
    const int r = (int)(k % per);
    int node, pc = -1;
    if (r < d.segs) {
        node = r;
    } else {
        node = (r - d.segs) / d.dim;
        pc = (r - d.segs) % d.dim;
    }
    put_shot(d, s, k, i, d.mesh[node], d.mesh[node + 1]);
    for (int c = 0; c < d.dim; ++c) {
        double v = d.u[(int64_t)(node * d.dim + c) * d.n + i];
        if (c == pc) v = v + kSqrtEps * fmax(fabs(v), 1.0);
        s.y0[(int64_t)c * s.m + k] = v;
    }
}

// the initial-nodes shot of multiple shooting: one per instance, from the guess over [t0, tf]
__global__ void k_build_nodes_shot(Dev d, Shots s) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    put_shot(d, s, i, i, d.t0[i], d.tf[i]);
    for (int c = 0; c < d.dim; ++c) s.y0[(int64_t)c * s.m + i] = d.guess[(int64_t)c * d.n + i];
}

// initial_nodes (multiple.rs:108-126): the nodes are the shot's output at the mesh points
__global__ void k_take_nodes(Dev d, Shots s) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    count(d, s, i, i);
    if (s.status[i] != DEGPU_COMPLETE) {
        fail(d, i, s.status[i], s.t_final[i], s.y_final + i, s.m);
        return;
    }
    bool all = true;
    for (int k = 0; k <= d.segs; ++k)
        for (int c = 0; c < d.dim; ++c) {
            const double v = s.dense[((int64_t)k * d.dim + c) * s.m + i];
            all = all && !isnan(v);
            d.u[(int64_t)(k * d.dim + c) * d.n + i] = v;
        }
    if (!all) fail(d, i, DEGPU_ERR_BAD_INPUT, d.t0[i], d.guess + i, d.n);  // a mesh node was not produced
}

// SingleShooting::solve (single.rs:84-176), one pass for instance act[a]
__global__ void k_newton_single(Dev d, const int64_t* act, int64_t nact, Shots s) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= nact) return;
    const int64_t i = act[a];
    const int dim = d.dim, per = dim + 1;
    const int64_t k0 = a * per;
    count(d, s, i, k0);
    if (s.status[k0] != DEGPU_COMPLETE) {
        fail(d, i, s.status[k0], s.t_final[k0], s.y_final + k0, s.m);
        return;
    }
    double u[DEGPU_HYPERPLANE_MAX_DIM], yb[DEGPU_HYPERPLANE_MAX_DIM], res[DEGPU_HYPERPLANE_MAX_DIM];
    double up[DEGPU_HYPERPLANE_MAX_DIM], resp[DEGPU_HYPERPLANE_MAX_DIM];
    for (int c = 0; c < dim; ++c) {
        u[c] = d.u[(int64_t)c * d.n + i];
        yb[c] = s.y_final[(int64_t)c * s.m + k0];
    }
    for (int r = 0; r < dim; ++r) res[r] = bnd(d, r, u, yb);
    if (max_norm(res, dim) <= d.tol) {
        d.phase[i] = CONVERGED;
        return;
    }
    double* J = d.jm + i * (int64_t)d.U * d.U;
    for (int j = 0; j < dim; ++j) {
        const int64_t kj = k0 + 1 + j;
        count(d, s, i, kj);
        if (s.status[kj] != DEGPU_COMPLETE) {
            fail(d, i, s.status[kj], s.t_final[kj], s.y_final + kj, s.m);
            return;
        }
        const double pert = kSqrtEps * fmax(fabs(u[j]), 1.0);
        for (int c = 0; c < dim; ++c) {
            up[c] = c == j ? u[c] + pert : u[c];
            yb[c] = s.y_final[(int64_t)c * s.m + kj];
        }
        for (int r = 0; r < dim; ++r) resp[r] = bnd(d, r, up, yb);
        d.jac[i] += 1;
        for (int r = 0; r < dim; ++r) J[r * dim + j] = (resp[r] - res[r]) / pert;
    }
    double step[DEGPU_HYPERPLANE_MAX_DIM];
    for (int r = 0; r < dim; ++r) step[r] = -res[r];
    if (!lu_solve(J, dim, step)) {
        fail(d, i, DEGPU_ERR_LINEAR_ALGEBRA, d.t0[i], d.u + i, d.n);
        return;
    }
    d.iters[i] += 1;
    for (int r = 0; r < dim; ++r) d.u[(int64_t)r * d.n + i] = u[r] + step[r];
}

// MultipleShooting::solve (multiple.rs:190-300), one pass for instance act[a]
__global__ void k_newton_multi(Dev d, const int64_t* act, int64_t nact, Shots s) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= nact) return;
    const int64_t i = act[a];
    const int dim = d.dim, segs = d.segs, U = d.U, per = segs * (1 + dim);
    const int64_t k0 = a * per;
    double u[kUMax], res[kUMax], resp[kUMax], yend[kUMax], yendp[kUMax];
    for (int r = 0; r < U; ++r) u[r] = d.u[(int64_t)r * d.n + i];
    // residual (multiple.rs:127-170): boundary rows, then each segment's mismatch
    for (int r = 0; r < dim; ++r) res[r] = bnd(d, r, u, u + segs * dim);
    for (int g = 0; g < segs; ++g) {
        count(d, s, i, k0 + g);
        if (s.status[k0 + g] != DEGPU_COMPLETE) {
            fail(d, i, s.status[k0 + g], s.t_final[k0 + g], s.y_final + k0 + g, s.m);
            return;
        }
        for (int c = 0; c < dim; ++c) {
            yend[g * dim + c] = s.y_final[(int64_t)c * s.m + k0 + g];
            res[(g + 1) * dim + c] = yend[g * dim + c] - u[(g + 1) * dim + c];
        }
    }
    if (max_norm(res, U) <= d.tol) {
        d.phase[i] = CONVERGED;
        return;
    }
    double* J = d.jm + i * (int64_t)U * U;
    for (int j = 0; j < U; ++j) {
        const int node = j / dim;
        const double yj = u[j];
        const double pert = kSqrtEps * fmax(fabs(yj), 1.0);
        u[j] = yj + pert;  // the perturbed nodes (restored below)
        // the perturbed residual: segments other than `node` repeat the pass's base shots
        for (int g = 0; g < segs; ++g) {
            if (g == node) {
                const int64_t kp = k0 + segs + j;
                count(d, s, i, kp);
                if (s.status[kp] != DEGPU_COMPLETE) {
                    fail(d, i, s.status[kp], s.t_final[kp], s.y_final + kp, s.m);
                    return;
                }
                for (int q = 0; q < dim; ++q) yendp[g * dim + q] = s.y_final[(int64_t)q * s.m + kp];
            } else {
                count(d, s, i, k0 + g);
                for (int q = 0; q < dim; ++q) yendp[g * dim + q] = yend[g * dim + q];
            }
        }
        for (int r = 0; r < dim; ++r) resp[r] = bnd(d, r, u, u + segs * dim);
        for (int g = 0; g < segs; ++g)
            for (int q = 0; q < dim; ++q) resp[(g + 1) * dim + q] = yendp[g * dim + q] - u[(g + 1) * dim + q];
        u[j] = yj;
        d.jac[i] += 1;
        for (int r = 0; r < U; ++r) J[r * U + j] = (resp[r] - res[r]) / pert;
    }
    for (int r = 0; r < U; ++r) res[r] = -res[r];
    if (!lu_solve(J, U, res)) {
        fail(d, i, DEGPU_ERR_LINEAR_ALGEBRA, d.t0[i], d.u + i, d.n);
        return;
    }
    d.iters[i] += 1;
    for (int r = 0; r < U; ++r) d.u[(int64_t)r * d.n + i] = u[r] + res[r];
}

// Error::MaxSteps { t: t0, y: the guess (single) or the first node (multiple) } for the
// instances still iterating after max_iterations passes
__global__ void k_fail_remaining(Dev d, int multi) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= d.n || d.phase[i] != ACTIVE) return;
    fail(d, i, DEGPU_ERR_MAX_STEPS, d.t0[i], (multi ? d.u : d.guess) + i, d.n);
}

__global__ void k_build_final(Dev d, const int64_t* conv, int64_t nconv, Shots s, int64_t* fidx) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= nconv) return;
    const int64_t i = conv[k];
    fidx[i] = k;
    put_shot(d, s, k, i, d.t0[i], d.tf[i]);
    for (int c = 0; c < d.dim; ++c) s.y0[(int64_t)c * s.m + k] = d.u[(int64_t)c * d.n + i];
}

// the final solve from the converged initial state, into the caller's output layout
__global__ void k_finish(Dev d, const int64_t* fidx, Shots s, int ne, double* y_final, double* t_final,
                         double* dense, int32_t* status, double* y_a) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const int64_t k = d.phase[i] == CONVERGED ? fidx[i] : -1;
    int32_t st = d.status[i];
    if (k >= 0) {
        count(d, s, i, k);
        st = s.status[k];
        t_final[i] = s.t_final[k];
        for (int c = 0; c < d.dim; ++c) y_final[(int64_t)c * d.n + i] = s.y_final[(int64_t)c * s.m + k];
    } else {
        t_final[i] = d.t_err[i];
        for (int c = 0; c < d.dim; ++c) y_final[(int64_t)c * d.n + i] = d.y_err[(int64_t)c * d.n + i];
    }
    status[i] = st;
    const bool ok = k >= 0 && st == DEGPU_COMPLETE;
    for (int c = 0; c < d.dim; ++c) y_a[(int64_t)c * d.n + i] = ok ? d.u[(int64_t)c * d.n + i] : NAN;
    for (int e = 0; e < ne; ++e)
        for (int c = 0; c < d.dim; ++c)
            dense[((int64_t)e * d.dim + c) * d.n + i] = ok ? s.dense[((int64_t)e * d.dim + c) * s.m + k] : NAN;
}

// Stream-ordered device allocations released at the end of the call.
struct Arena {
    cudaStream_t s;
    std::vector<void*> ptrs;
    bool ok = true;
    template <class T>
    T* get(size_t count) {
        void* p = nullptr;
        if (cudaMallocAsync(&p, (count ? count : 1) * sizeof(T), s) != cudaSuccess) {
            ok = false;
            return nullptr;
        }
        ptrs.push_back(p);
        return (T*)p;
    }
    ~Arena() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
    }
};

unsigned blocks(int64_t n) { return (unsigned)((n + 127) / 128); }

}  // namespace

extern "C" degpu_status degpu_solve_bvp_host(const degpu_problem* pb, const degpu_method_cfg* cfg,
                                             const degpu_batch_in* in, const degpu_bvp* bvp, degpu_batch_out* out,
                                             degpu_bvp_out* bo) {
    if (!pb || !cfg || !in || !bvp || !out || !bo) return DEGPU_BAD_INPUT;
    if (in->n < 0 || !out->y_final || !bo->y_a || !in->t0 || !in->tf || !in->y0 || !in->rtol || !in->atol)
        return DEGPU_BAD_INPUT;
    // the shots of a Newton pass are assembled with one scalar tolerance per instance
    if (in->rtol_vec || in->atol_vec) return DEGPU_UNSUPPORTED;
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
    // The forward-difference Jacobian perturbs by sqrt(eps) max(|u|, 1) ~ 1.5e-8 relative, below
    // FP32 resolution: a mixed solve's FP32 stages would return the unperturbed shot and a zero
    // column. Shots of a mixed BVP solve therefore run in FP64 fast arithmetic.
    degpu_method_cfg c64 = *cfg;
    if (c64.precision == DEGPU_MIXED) c64.precision = DEGPU_FP64_FAST;
    const int np = pb->n_params, segs = multi ? bvp->segments : 0;
    const int U = multi ? (segs + 1) * dim : dim;
    const int per = multi ? segs * (1 + dim) : dim + 1;
    const int ne = (in->n_eval > 0 && out->dense) ? in->n_eval : 0;

    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return DEGPU_CUDA_ERROR;
    degpu_status st = DEGPU_OK;
    {
        Arena ar{s};
        Dev d{};
        d.n = n;
        d.dim = dim;
        d.U = U;
        d.segs = segs;
        d.np = np;
        d.tol = bvp->tolerance;
        for (int i = 0; i < DEGPU_HYPERPLANE_MAX_DIM; ++i) {
            d.side[i] = bvp->side[i];
            d.comp[i] = bvp->component[i];
            d.value[i] = bvp->value[i];
        }
        // mesh (multiple.rs:83-107): t0 + span * i / m
        std::vector<double> mesh;
        if (multi) {
            const double span = in->tf[0] - in->t0[0];
            for (int i = 0; i <= segs; ++i) mesh.push_back(in->t0[0] + span * (double)i / (double)segs);
            for (int i = 0; i <= segs; ++i) d.mesh[i] = mesh[i];
        }
        auto up = [&](const double* src, size_t count) -> double* {
            double* p = ar.get<double>(count);
            if (p) cudaMemcpyAsync(p, src, count * sizeof(double), cudaMemcpyHostToDevice, s);
            return p;
        };
        d.t0 = up(in->t0, n);
        d.tf = up(in->tf, n);
        d.params = np > 0 ? up(in->params, (size_t)np * n) : nullptr;
        d.rtol = up(in->rtol, n);
        d.atol = up(in->atol, n);
        double* y0 = up(in->y0, (size_t)dim * n);
        double* te = ne ? up(in->t_eval, ne) : nullptr;
        double* mesh_d = multi ? up(mesh.data(), mesh.size()) : nullptr;
        d.u = ar.get<double>((size_t)U * n);
        d.guess = ar.get<double>((size_t)dim * n);
        d.phase = ar.get<int32_t>(n);
        d.status = ar.get<int32_t>(n);
        d.iters = ar.get<int32_t>(n);
        d.t_err = ar.get<double>(n);
        d.y_err = ar.get<double>((size_t)dim * n);
        d.fev = ar.get<int64_t>(n);
        d.acc = ar.get<int64_t>(n);
        d.rej = ar.get<int64_t>(n);
        d.jac = ar.get<int64_t>(n);
        d.jm = ar.get<double>((size_t)n * U * U);
        int64_t* list = ar.get<int64_t>(n);
        int64_t* fidx = ar.get<int64_t>(n);
        unsigned long long* cnt = ar.get<unsigned long long>(1);
        // shot buffers, sized for the largest pass
        const int64_t mmax = n * (int64_t)(per > 1 ? per : 1);
        const int nd = std::max(ne, multi ? segs + 1 : 0);
        Shots sh{};
        sh.t0 = ar.get<double>(mmax);
        sh.tf = ar.get<double>(mmax);
        sh.y0 = ar.get<double>((size_t)dim * mmax);
        sh.params = ar.get<double>((size_t)(np > 0 ? np : 1) * mmax);
        sh.rtol = ar.get<double>(mmax);
        sh.atol = ar.get<double>(mmax);
        sh.y_final = ar.get<double>((size_t)dim * mmax);
        sh.t_final = ar.get<double>(mmax);
        sh.dense = nd ? ar.get<double>((size_t)nd * dim * n) : nullptr;
        sh.acc = ar.get<int64_t>(mmax);
        sh.rej = ar.get<int64_t>(mmax);
        sh.fev = ar.get<int64_t>(mmax);
        sh.status = ar.get<int32_t>(mmax);
        // the caller's outputs, on the device until the end
        double* o_y = ar.get<double>((size_t)dim * n);
        double* o_t = ar.get<double>(n);
        double* o_dense = ne ? ar.get<double>((size_t)ne * dim * n) : nullptr;
        int32_t* o_st = ar.get<int32_t>(n);
        double* o_ya = ar.get<double>((size_t)dim * n);
        if (!ar.ok) {
            st = DEGPU_OOM;
        } else {
            const degpu_problem prob{pb->rhs_id, dim, np, 0};
            // one ensemble solve of the first m shots (laid out for that m by the build kernels);
            // t_eval (device) gives dense output
            auto solve = [&](int64_t m, const double* t_eval, int n_eval) -> degpu_status {
                sh.m = m;
                degpu_batch_in bi{};
                bi.n = m;
                bi.t0 = sh.t0;
                bi.tf = sh.tf;
                bi.y0 = sh.y0;
                bi.params = np > 0 ? sh.params : nullptr;
                bi.rtol = sh.rtol;
                bi.atol = sh.atol;
                bi.t_eval = t_eval;
                bi.n_eval = n_eval;
                degpu_batch_out bo_{sh.y_final, sh.t_final, n_eval ? sh.dense : nullptr, sh.acc, sh.rej, sh.fev,
                                    sh.status};
                return degpu_solve_ensemble(&prob, &c64, &bi, &bo_, (void*)s);
            };
            // the instances in phase `want` into `list`; their count to the host
            auto select = [&](int32_t want, int64_t& count_out) -> degpu_status {
                unsigned long long h = 0;
                if (cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s) != cudaSuccess) return DEGPU_CUDA_ERROR;
                k_compact<<<blocks(n), 128, 0, s>>>(d.phase, n, want, list, cnt);
                if (cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                    cudaStreamSynchronize(s) != cudaSuccess)
                    return DEGPU_CUDA_ERROR;
                count_out = (int64_t)h;
                return DEGPU_OK;
            };
            k_init<<<blocks(n), 128, 0, s>>>(d, y0);
            if (multi) {
                sh.m = n;
                k_build_nodes_shot<<<blocks(n), 128, 0, s>>>(d, sh);
                st = solve(n, mesh_d, segs + 1);
                if (st == DEGPU_OK) k_take_nodes<<<blocks(n), 128, 0, s>>>(d, sh);
            }
            for (int it = 0; st == DEGPU_OK && it < bvp->max_iterations; ++it) {
                int64_t nact = 0;
                st = select(ACTIVE, nact);
                if (st != DEGPU_OK || nact == 0) break;
                sh.m = nact * per;
                if (multi)
                    k_build_multi<<<blocks(sh.m), 128, 0, s>>>(d, list, nact, sh);
                else
                    k_build_single<<<blocks(sh.m), 128, 0, s>>>(d, list, nact, sh);
                st = solve(sh.m, nullptr, 0);
                if (st != DEGPU_OK) break;
                if (multi)
                    k_newton_multi<<<blocks(nact), 128, 0, s>>>(d, list, nact, sh);
                else
                    k_newton_single<<<blocks(nact), 128, 0, s>>>(d, list, nact, sh);
            }
            if (st == DEGPU_OK) {
                k_fail_remaining<<<blocks(n), 128, 0, s>>>(d, multi ? 1 : 0);
                int64_t nconv = 0;
                st = select(CONVERGED, nconv);
                if (st == DEGPU_OK && nconv > 0) {
                    sh.m = nconv;
                    k_build_final<<<blocks(nconv), 128, 0, s>>>(d, list, nconv, sh, fidx);
                    st = solve(nconv, te, ne);
                }
                if (st == DEGPU_OK) {
                    k_finish<<<blocks(n), 128, 0, s>>>(d, fidx, sh, ne, o_y, o_t, o_dense, o_st, o_ya);
                    auto down = [&](void* dst, const void* src, size_t bytes) {
                        if (dst && src && bytes) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
                    };
                    down(out->y_final, o_y, (size_t)dim * n * 8);
                    down(out->t_final, o_t, n * 8);
                    down(out->dense, o_dense, (size_t)ne * dim * n * 8);
                    down(out->accepted, d.acc, n * 8);
                    down(out->rejected, d.rej, n * 8);
                    down(out->fevals, d.fev, n * 8);
                    down(out->status, o_st, n * 4);
                    down(bo->y_a, o_ya, (size_t)dim * n * 8);
                    down(bo->iterations, d.iters, n * 4);
                    down(bo->jacobian, d.jac, n * 8);
                    if (cudaGetLastError() != cudaSuccess) st = DEGPU_CUDA_ERROR;
                }
            }
        }
        if (cudaStreamSynchronize(s) != cudaSuccess && st == DEGPU_OK) st = DEGPU_CUDA_ERROR;
    }
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return st;
}
