// stencil.cuh — method-of-lines RK4 for 2-D Gray–Scott on a periodic grid.
//
// Right-hand side: the crate's flux-form finite-difference semi-discretisation
// (src/pde/semi_discrete.rs:250-287 with finite_difference_flux :181-190 and
// directional_gradient :150-172) of
//     u_t = div(Du grad u) - u v^2 + F (1 - u),   v_t = div(Dv grad v) + u v^2 - (F + k) v
// with periodic neighbours (an extension; the crate has Dirichlet / Neumann faces only).  Per
// node and field, in the crate's order: der = source; for axis x then y:
//     F_lo = D * ((c - c_lo) / dx),  F_hi = D * ((c_hi - c) / dx),  der = der + (F_hi - F_lo) / dx.
// When dx is a power of two, "/ dx" is replaced by the exact multiplication by 1/dx.
//
// Time stepping: the crate's fixed RK4 step (src/methods/erk/fixed/ordinary.rs:58-138) with
// y_next = (((y + (b0 h) k0) + (b1 h) k1) + (b2 h) k2) + (b3 h) k3 accumulated across passes:
//   pass 1: k1 = f(y + (h/2) k0)          acc = (y + (b0 h) k0) + (b1 h) k1
//   pass 2: k2 = f(y + (h/2) k1)          acc = acc + (b2 h) k2
//   pass 3: k3 = f(y + h k2)              y_next = acc + (b3 h) k3
//   pass 4: k0 = f(y_next)                (the crate's non-FSAL derivative at the new point)
// Each pass reads its stage inputs at the node and its four neighbours through L1/L2 (a 5-point
// stencil: horizontal neighbours share the cache line, vertical ones hit L1/L2), so DRAM sees
// each array once per pass.  Algorithmic bytes per node per step: 4 + 5 + 4 + 2 arrays read/written
// of 2 fields -> (8 + 10 + 8 + 4) * sizeof(T) = 240 B (FP64), 120 B (FP32).
// FP32 runs the same four stages in one launch per step where the grid divides into 64 x 32
// tiles (gs_step_fused_kernel, below): 32 B per node and step, the same values bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace degpu {

template <class T>
struct GsParams {
    int nx, ny;
    T Du, Dv, F, k, dx, inv_dx;
    T cu, cv;   // FP32 form: Du / dx^2, Dv / dx^2
    T ah;       // stage coefficient a_{i,i-1} * h
    T bh0, bh1; // accumulation coefficients b_i * h of the pass
};

// Explicit rounding of every operation, so that the passes and the fused step (different kernels,
// different surrounding code) compute the same values whatever the compiler would contract: gs_m
// and gs_a are a single rounded multiply and add, gs_f a fused multiply-add, except in the parity
// build (-fmad=false, DEGPU_NO_FMAD), where gs_f is a multiply then an add as the crate computes.
__device__ __forceinline__ float gs_m(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double gs_m(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float gs_a(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double gs_a(double a, double b) { return __dadd_rn(a, b); }
#if defined(DEGPU_NO_FMAD)
template <class T>
__device__ __forceinline__ T gs_f(T a, T b, T c) { return gs_a(gs_m(a, b), c); }
#else
__device__ __forceinline__ float gs_f(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double gs_f(double a, double b, double c) { return __fma_rn(a, b, c); }
#endif

template <class T, bool POW2>
__device__ __forceinline__ T gs_ddx(T a, const GsParams<T>& p) {
    if constexpr (POW2)
        return gs_m(a, p.inv_dx);
    else
        return a / p.dx;
}

// one node's f from its stage state and its four neighbours (l, r: x -+ 1; d, u: y -+ 1), in the
// crate's order: der = source; for axis x then y: der = der + (F_hi - F_lo) / dx with
// F_lo = D ((c - c_lo) / dx), F_hi = D ((c_hi - c) / dx)
template <class T, bool POW2>
__device__ __forceinline__ void gs_node(const GsParams<T>& p, T u, T v, T ul, T vl, T ur, T vr, T ud, T vd, T uu,
                                        T vu, T& du, T& dv) {
    if constexpr (sizeof(T) == 4) {
        // FP32 (this build's own form, not the crate's order): the 5-point Laplacian as a sum of
        // the four neighbour differences (each exact where neighbours lie within a factor of two)
        // times D / dx^2, fused into the source term
        const T uvv = gs_m(gs_m(u, v), v);
        const T lu = gs_a(gs_a(gs_a(ur, -u), gs_a(ul, -u)), gs_a(gs_a(uu, -u), gs_a(ud, -u)));
        const T lv = gs_a(gs_a(gs_a(vr, -v), gs_a(vl, -v)), gs_a(gs_a(vu, -v), gs_a(vd, -v)));
        du = gs_f(p.cu, lu, gs_f(p.F, gs_a((T)1, -u), -uvv));
        dv = gs_f(p.cv, lv, gs_f(-gs_a(p.F, p.k), v, uvv));
        return;
    }
    const T uvv = gs_m(gs_m(u, v), v);
    T a_u = gs_f(p.F, gs_a((T)1, -u), -uvv);     // -u v^2 + F (1 - u)
    T a_v = gs_f(-gs_a(p.F, p.k), v, uvv);       //  u v^2 - (F + k) v
    auto flux = [&](T a, T c, T lo, T hi, T D) {  // a + (F_hi - F_lo) / dx
        const T flo = gs_m(D, gs_ddx<T, POW2>(gs_a(c, -lo), p));
        const T fhi = gs_m(D, gs_ddx<T, POW2>(gs_a(hi, -c), p));
        if constexpr (POW2)
            return gs_f(gs_a(fhi, -flo), p.inv_dx, a);
        else
            return gs_a(a, gs_a(fhi, -flo) / p.dx);
    };
    a_u = flux(a_u, u, ul, ur, p.Du);
    a_v = flux(a_v, v, vl, vr, p.Dv);
    a_u = flux(a_u, u, ud, uu, p.Du);
    a_v = flux(a_v, v, vd, vu, p.Dv);
    du = a_u;
    dv = a_v;
}

// f at node (i, j); `get(i, j, u, v)` returns the stage state at a node.
template <class T, bool POW2, class Get>
__device__ __forceinline__ void gs_rhs_at(int i, int j, const GsParams<T>& p, Get get, T& du, T& dv) {
    const int im = i == 0 ? p.nx - 1 : i - 1, ip = i == p.nx - 1 ? 0 : i + 1;
    const int jm = j == 0 ? p.ny - 1 : j - 1, jp = j == p.ny - 1 ? 0 : j + 1;
    T u, v, ul, vl, ur, vr, ud, vd, uu, vu;
    get(i, j, u, v);
    get(im, j, ul, vl);
    get(ip, j, ur, vr);
    get(i, jm, ud, vd);
    get(i, jp, uu, vu);
    gs_node<T, POW2>(p, u, v, ul, vl, ur, vr, ud, vd, uu, vu, du, dv);
}

struct GsPlanes {
    const void* yu;
    const void* yv;
    const void* ku;   // stage input k_{i-1}
    const void* kv;
    const void* k0u;  // pass 1: k0 (for the accumulation)
    const void* k0v;
    void* ou;         // stage output k_i (passes 1, 2, 4)
    void* ov;
    void* accu;       // accumulator (in/out)
    void* accv;
    void* ynu;        // pass 3 output y_next
    void* ynv;
};

// PASS: 1, 2, 3 (stages) or 4 (k0 = f(y)).
template <class T, bool POW2, int PASS>
__global__ void __launch_bounds__(256) gs_pass_kernel(GsPlanes P, GsParams<T> p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= p.nx || j >= p.ny) return;
    const int64_t nx = p.nx;
    const T* yu = (const T*)P.yu;
    const T* yv = (const T*)P.yv;
    const T* ku = (const T*)P.ku;
    const T* kv = (const T*)P.kv;
    const int64_t c = (int64_t)j * nx + i;
    T du, dv;
    if constexpr (PASS == 4) {
        auto get = [&](int ii, int jj, T& u, T& v) {
            int64_t q = (int64_t)jj * nx + ii;
            u = __ldg(yu + q);
            v = __ldg(yv + q);
        };
        gs_rhs_at<T, POW2>(i, j, p, get, du, dv);
        ((T*)P.ou)[c] = du;
        ((T*)P.ov)[c] = dv;
    } else {
        const T ah = p.ah;
        auto get = [&](int ii, int jj, T& u, T& v) {
            int64_t q = (int64_t)jj * nx + ii;
            u = gs_f(ah, __ldg(ku + q), __ldg(yu + q));
            v = gs_f(ah, __ldg(kv + q), __ldg(yv + q));
        };
        gs_rhs_at<T, POW2>(i, j, p, get, du, dv);
        if constexpr (PASS == 1) {
            const T* k0u = (const T*)P.k0u;
            const T* k0v = (const T*)P.k0v;
            T au = gs_f(p.bh0, k0u[c], yu[c]);
            T av = gs_f(p.bh0, k0v[c], yv[c]);
            ((T*)P.accu)[c] = gs_f(p.bh1, du, au);
            ((T*)P.accv)[c] = gs_f(p.bh1, dv, av);
            ((T*)P.ou)[c] = du;
            ((T*)P.ov)[c] = dv;
        } else if constexpr (PASS == 2) {
            T* accu = (T*)P.accu;
            T* accv = (T*)P.accv;
            accu[c] = gs_f(p.bh0, du, accu[c]);
            accv[c] = gs_f(p.bh0, dv, accv[c]);
            ((T*)P.ou)[c] = du;
            ((T*)P.ov)[c] = dv;
        } else {
            const T* accu = (const T*)P.accu;
            const T* accv = (const T*)P.accv;
            ((T*)P.ynu)[c] = gs_f(p.bh0, du, accu[c]);
            ((T*)P.ynv)[c] = gs_f(p.bh0, dv, accv[c]);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Register-blocked form: each thread owns a 4 x 4 block of nodes (4 along x in one 16-byte
// vector for FP32, two for FP64; 4 rows).  A warp covers 128 consecutive x; its lanes hand the
// stage state of their edge columns to their neighbours by shuffles, and only lanes 0 and 31
// load the columns beyond the warp (with the periodic wrap).  Rows j0-1 .. j0+4 are loaded once
// and shared by the four output rows.  Per node the arithmetic is gs_rhs_at's, in the same order.
// Requires nx % 128 == 0 and ny % 16 == 0 (the block is 32 x 4 threads = 128 x 16 nodes).
// ---------------------------------------------------------------------------------------------
template <class T>
struct Vec4 {
    T v[4];
};

template <class T>
__device__ __forceinline__ Vec4<T> ld4(const T* p) {
    Vec4<T> r;
    if constexpr (sizeof(T) == 4) {
        float4 q = __ldg((const float4*)p);
        r.v[0] = q.x; r.v[1] = q.y; r.v[2] = q.z; r.v[3] = q.w;
    } else {
        double2 a = __ldg((const double2*)p), b = __ldg((const double2*)p + 1);
        r.v[0] = a.x; r.v[1] = a.y; r.v[2] = b.x; r.v[3] = b.y;
    }
    return r;
}
template <class T>
__device__ __forceinline__ void st4(T* p, const Vec4<T>& r) {
    if constexpr (sizeof(T) == 4) {
        *(float4*)p = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
    } else {
        ((double2*)p)[0] = make_double2(r.v[0], r.v[1]);
        ((double2*)p)[1] = make_double2(r.v[2], r.v[3]);
    }
}

template <class T, bool POW2, int PASS>
__global__ void __launch_bounds__(128) gs_pass_vec_kernel(GsPlanes P, GsParams<T> p) {
    constexpr int R = 4;  // rows per thread
    const int lane = threadIdx.x & 31;
    const int wy = threadIdx.x >> 5;  // warp within block: 4 warps stacked in y
    const int xb = blockIdx.x * 128;
    const int x0 = xb + lane * 4;
    const int j0 = (blockIdx.y * 4 + wy) * R;
    const int64_t nx = p.nx;
    const int ny = p.ny;
    const T* yu = (const T*)P.yu;
    const T* yv = (const T*)P.yv;
    const T* ku = (const T*)P.ku;
    const T* kv = (const T*)P.kv;
    const bool has_k = PASS != 4;
    const T ah = p.ah;
    // stage state of rows j0-1 .. j0+R (R+2 rows) at this lane's 4 columns
    T su[R + 2][4], sv[R + 2][4];
#pragma unroll
    for (int r = 0; r < R + 2; ++r) {
        int j = j0 - 1 + r;
        j = j < 0 ? j + ny : (j >= ny ? j - ny : j);
        const int64_t o = (int64_t)j * nx + x0;
        Vec4<T> a = ld4(yu + o), b = ld4(yv + o);
        if (has_k) {
            Vec4<T> c = ld4(ku + o), d = ld4(kv + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                su[r][q] = gs_f(ah, c.v[q], a.v[q]);
                sv[r][q] = gs_f(ah, d.v[q], b.v[q]);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                su[r][q] = a.v[q];
                sv[r][q] = b.v[q];
            }
        }
    }
    // columns x0-1 and x0+4 of the output rows: from the neighbouring lanes, or loaded at the warp
    // edges (periodic wrap)
    const int xl = xb == 0 ? (int)nx - 1 : xb - 1;
    const int xr = xb + 128 == (int)nx ? 0 : xb + 128;
    T lu[R], lv[R], ru[R], rv[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        lu[r] = __shfl_up_sync(0xffffffffu, su[r + 1][3], 1);
        lv[r] = __shfl_up_sync(0xffffffffu, sv[r + 1][3], 1);
        ru[r] = __shfl_down_sync(0xffffffffu, su[r + 1][0], 1);
        rv[r] = __shfl_down_sync(0xffffffffu, sv[r + 1][0], 1);
    }
    if (lane == 0 || lane == 31) {
        const int xe = lane == 0 ? xl : xr;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int64_t o = (int64_t)(j0 + r) * nx + xe;
            T eu = __ldg(yu + o), ev = __ldg(yv + o);
            if (has_k) {
                eu = gs_f(ah, __ldg(ku + o), eu);
                ev = gs_f(ah, __ldg(kv + o), ev);
            }
            if (lane == 0) {
                lu[r] = eu;
                lv[r] = ev;
            } else {
                ru[r] = eu;
                rv[r] = ev;
            }
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = j0 + r;
        const int64_t o = (int64_t)j * nx + x0;
        Vec4<T> du, dv;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            T ul = q == 0 ? lu[r] : su[r + 1][q - 1];
            T vl = q == 0 ? lv[r] : sv[r + 1][q - 1];
            T ur = q == 3 ? ru[r] : su[r + 1][q + 1];
            T vr = q == 3 ? rv[r] : sv[r + 1][q + 1];
            gs_node<T, POW2>(p, su[r + 1][q], sv[r + 1][q], ul, vl, ur, vr, su[r][q], sv[r][q], su[r + 2][q],
                             sv[r + 2][q], du.v[q], dv.v[q]);
        }
        if constexpr (PASS == 4) {
            st4((T*)P.ou + o, du);
            st4((T*)P.ov + o, dv);
        } else if constexpr (PASS == 1) {
            Vec4<T> y_u = ld4(yu + o), y_v = ld4(yv + o), k_u = ld4((const T*)P.k0u + o), k_v = ld4((const T*)P.k0v + o);
            Vec4<T> au, av;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                au.v[q] = gs_f(p.bh1, du.v[q], gs_f(p.bh0, k_u.v[q], y_u.v[q]));
                av.v[q] = gs_f(p.bh1, dv.v[q], gs_f(p.bh0, k_v.v[q], y_v.v[q]));
            }
            st4((T*)P.accu + o, au);
            st4((T*)P.accv + o, av);
            st4((T*)P.ou + o, du);
            st4((T*)P.ov + o, dv);
        } else if constexpr (PASS == 2) {
            Vec4<T> au = ld4((const T*)P.accu + o), av = ld4((const T*)P.accv + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                au.v[q] = gs_f(p.bh0, du.v[q], au.v[q]);
                av.v[q] = gs_f(p.bh0, dv.v[q], av.v[q]);
            }
            st4((T*)P.accu + o, au);
            st4((T*)P.accv + o, av);
            st4((T*)P.ou + o, du);
            st4((T*)P.ov + o, dv);
        } else {
            Vec4<T> au = ld4((const T*)P.accu + o), av = ld4((const T*)P.accv + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                au.v[q] = gs_f(p.bh0, du.v[q], au.v[q]);
                av.v[q] = gs_f(p.bh0, dv.v[q], av.v[q]);
            }
            st4((T*)P.ynu + o, au);
            st4((T*)P.ynv + o, av);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Fused FP32 RK4 step (temporal blocking): one launch per step instead of four passes.  A block
// owns a TX x TY tile of nodes and stages the tile plus a 4-node halo of y and k0 in shared memory
// (both fields of a node side by side, one 8-byte word); the four stages then run on shrinking
// regions (tile + 3, + 2, + 1 and the tile itself), so no stage result goes through HBM.  Per step
// HBM sees y and k0 in and y_next and k0 out: 32 B per node against the passes' 120 B.  The cost
// is the halo: f is evaluated on (TX+6)(TY+6) + (TX+4)(TY+4) + (TX+2)(TY+2) + TX TY nodes per
// tile (1.15 x the tile's four evaluations at 64 x 32).  The stage state is double-buffered in
// shared memory, so each stage's derivative goes straight into the accumulator and the next
// stage state, and one barrier separates the stages.  The halo comes in with 16-byte loads (four
// nodes along x), and each thread evaluates two vertically adjacent nodes, which share two of
// their shared-memory loads.
// Per node the arithmetic is the passes', in the same order (stage states y + (a h) k, gs_node,
// the accumulation ((y + (b0 h) k0) + (b1 h) k1) + (b2 h) k2 + (b3 h) k3), so the results equal
// the four-pass kernels' bit for bit.  Requires nx % TX == 0 and ny % TY == 0.
// ---------------------------------------------------------------------------------------------
struct GsFusedPlanes {
    const float* yu;
    const float* yv;
    const float* ku;  // k0 = f(y) of this step's start
    const float* kv;
    float* nu;        // y_next
    float* nv;
    float* knu;       // k0 of the next step, f(y_next)
    float* knv;
};
struct GsFusedCoef {
    float ah1, ah2, ah3;       // stage coefficients a_{i,i-1} h
    float bh0, bh1, bh2, bh3;  // weights b_i h
};

#ifndef DEGPU_GS_THREADS
#define DEGPU_GS_THREADS 512
#endif
constexpr int GS_FUSED_THREADS = DEGPU_GS_THREADS;

template <int TX, int TY>
constexpr size_t gs_fused_smem() {
    return 4 * (size_t)(TX + 8) * (TY + 8) * sizeof(float2);
}

template <bool POW2, int TX, int TY>
__global__ void __launch_bounds__(GS_FUSED_THREADS) gs_step_fused_kernel(GsFusedPlanes P, GsParams<float> p,
                                                                         GsFusedCoef cf) {
    constexpr int HALO = 4, W = TX + 2 * HALO, HH = TY + 2 * HALO, N = W * HH;
    static_assert(TX % 4 == 0 && TY % 2 == 0, "16-byte row chunks and row pairs");
    extern __shared__ float2 gs_sm[];
    float2* Ys = gs_sm;          // y on the tile + 4
    float2* S0 = gs_sm + N;      // stage states, alternating
    float2* S1 = gs_sm + 2 * N;
    float2* As = gs_sm + 3 * N;  // accumulator (rows of the tile + 1; other columns unused)
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int nx = p.nx, ny = p.ny;
    // y and k0 on the tile + 4 (periodic wrap) in 16-byte chunks of 4 nodes along x (x0 - 4 and nx
    // are multiples of 4, so a chunk never straddles the wrap); s1 = y + (a10 h) k0 there, the
    // accumulator's first term y + (b0 h) k0 on the rows of the tile + 1
    constexpr int CH = W / 4;
    for (int i = threadIdx.x; i < CH * HH; i += GS_FUSED_THREADS) {
        const int r = i / CH, c = (i - r * CH) * 4;
        int gx = x0 - HALO + c;
        gx += gx < 0 ? nx : (gx >= nx ? -nx : 0);
        int gy = y0 - HALO + r;
        gy += gy < 0 ? ny : (gy >= ny ? -ny : 0);
        const int64_t g = (int64_t)gy * nx + gx;
        const float4 yu = __ldg(reinterpret_cast<const float4*>(P.yu + g));
        const float4 yv = __ldg(reinterpret_cast<const float4*>(P.yv + g));
        const float4 ku = __ldg(reinterpret_cast<const float4*>(P.ku + g));
        const float4 kv = __ldg(reinterpret_cast<const float4*>(P.kv + g));
        const int q = r * W + c;  // even: 16-byte aligned pairs of nodes
        float4* y4 = reinterpret_cast<float4*>(Ys + q);
        y4[0] = make_float4(yu.x, yv.x, yu.y, yv.y);
        y4[1] = make_float4(yu.z, yv.z, yu.w, yv.w);
        float4* s4 = reinterpret_cast<float4*>(S0 + q);
        s4[0] = make_float4(gs_f(cf.ah1, ku.x, yu.x), gs_f(cf.ah1, kv.x, yv.x), gs_f(cf.ah1, ku.y, yu.y),
                            gs_f(cf.ah1, kv.y, yv.y));
        s4[1] = make_float4(gs_f(cf.ah1, ku.z, yu.z), gs_f(cf.ah1, kv.z, yv.z), gs_f(cf.ah1, ku.w, yu.w),
                            gs_f(cf.ah1, kv.w, yv.w));
        if (r >= HALO - 1 && r < HH - HALO + 1) {
            float4* a4 = reinterpret_cast<float4*>(As + q);
            a4[0] = make_float4(gs_f(cf.bh0, ku.x, yu.x), gs_f(cf.bh0, kv.x, yv.x), gs_f(cf.bh0, ku.y, yu.y),
                                gs_f(cf.bh0, kv.y, yv.y));
            a4[1] = make_float4(gs_f(cf.bh0, ku.z, yu.z), gs_f(cf.bh0, kv.z, yv.z), gs_f(cf.bh0, ku.w, yu.w),
                                gs_f(cf.bh0, kv.w, yv.w));
        }
    }
    __syncthreads();
    // stage K: k = f(Sc) on the tile + K, two vertically adjacent nodes per thread (rows r and r + 1
    // share their middle loads); the accumulator on the tile + 1 takes (b h) k and the next stage
    // state y + (a h) k goes to Sn (after the last stage: y_next = acc + (b3 h) k3)
    auto stage = [&](auto kk, const float2* Sc, float2* Sn, float bh, float ah) {
        constexpr int K = decltype(kk)::value, w = TX + 2 * K, h2 = (TY + 2 * K) / 2, off = HALO - K;
        auto node = [&](int r, int c, int q, float2 sc, float2 sl, float2 sr, float2 sd, float2 su) {
            float du, dv;
            gs_node<float, POW2>(p, sc.x, sc.y, sl.x, sl.y, sr.x, sr.y, sd.x, sd.y, su.x, su.y, du, dv);
            if constexpr (K > 1) {
                if (r >= HALO - 1 && r < HH - HALO + 1 && c >= HALO - 1 && c < W - HALO + 1) {
                    const float2 a = As[q];
                    As[q] = make_float2(gs_f(bh, du, a.x), gs_f(bh, dv, a.y));
                }
                const float2 y = Ys[q];
                Sn[q] = make_float2(gs_f(ah, du, y.x), gs_f(ah, dv, y.y));
            } else {
                const float2 a = As[q];
                Sn[q] = make_float2(gs_f(bh, du, a.x), gs_f(bh, dv, a.y));
            }
        };
        for (int i = threadIdx.x; i < w * h2; i += GS_FUSED_THREADS) {
            const int rp = i / w;
            const int r = 2 * rp + off, c = i - rp * w + off;
            const int q = r * W + c;
            const float2 sd = Sc[q - W], s0 = Sc[q], s1 = Sc[q + W], su = Sc[q + 2 * W];
            node(r, c, q, s0, Sc[q - 1], Sc[q + 1], sd, s1);
            node(r + 1, c, q + W, s1, Sc[q + W - 1], Sc[q + W + 1], s0, su);
        }
    };
    stage(std::integral_constant<int, 3>{}, S0, S1, cf.bh1, cf.ah2);  // k1 on the tile + 3
    __syncthreads();
    stage(std::integral_constant<int, 2>{}, S1, S0, cf.bh2, cf.ah3);  // k2 on the tile + 2
    __syncthreads();
    stage(std::integral_constant<int, 1>{}, S0, S1, cf.bh3, 0.0f);    // k3 and y_next on the tile + 1
    __syncthreads();
    // k0 of the next step = f(y_next) on the tile, two rows per thread; y_next and k0 out
    for (int i = threadIdx.x; i < TX * (TY / 2); i += GS_FUSED_THREADS) {
        const int rp = i / TX;
        const int r = 2 * rp + HALO, c = i - rp * TX + HALO;
        const int q = r * W + c;
        const float2 sd = S1[q - W], s0 = S1[q], s1 = S1[q + W], su = S1[q + 2 * W];
        float du0, dv0, du1, dv1;
        const float2 l0 = S1[q - 1], r0 = S1[q + 1], l1 = S1[q + W - 1], r1 = S1[q + W + 1];
        gs_node<float, POW2>(p, s0.x, s0.y, l0.x, l0.y, r0.x, r0.y, sd.x, sd.y, s1.x, s1.y, du0, dv0);
        gs_node<float, POW2>(p, s1.x, s1.y, l1.x, l1.y, r1.x, r1.y, s0.x, s0.y, su.x, su.y, du1, dv1);
        const int64_t g = (int64_t)(y0 + r - HALO) * nx + (x0 + c - HALO);
        P.nu[g] = s0.x;
        P.nv[g] = s0.y;
        P.knu[g] = du0;
        P.knv[g] = dv0;
        P.nu[g + nx] = s1.x;
        P.nv[g + nx] = s1.y;
        P.knu[g + nx] = du1;
        P.knv[g + nx] = dv1;
    }
}

// Launchers for one precision (instantiated in stencil.cu and, for the parity build, in
// inst_parity_stencil.cu with -fmad=false).
// the vector kernels load and store 16 bytes at a time: every plane must start on a 16-byte boundary
inline bool gs_planes_aligned16(const GsPlanes& P) {
    const void* ptrs[] = {P.yu, P.yv, P.ku, P.kv, P.k0u, P.k0v, P.ou, P.ov, P.accu, P.accv, P.ynu, P.ynv};
    for (const void* q : ptrs)
        if (((uintptr_t)q & 15u) != 0) return false;
    return true;
}

template <class T, bool POW2>
cudaError_t gs_launch_pass(int pass, const GsPlanes& P, const GsParams<T>& p, cudaStream_t s) {
    if (p.nx % 128 == 0 && p.ny % 16 == 0 && gs_planes_aligned16(P)) {
        dim3 blk(128);
        dim3 grd(p.nx / 128, p.ny / 16);
        switch (pass) {
            case 1: gs_pass_vec_kernel<T, POW2, 1><<<grd, blk, 0, s>>>(P, p); break;
            case 2: gs_pass_vec_kernel<T, POW2, 2><<<grd, blk, 0, s>>>(P, p); break;
            case 3: gs_pass_vec_kernel<T, POW2, 3><<<grd, blk, 0, s>>>(P, p); break;
            default: gs_pass_vec_kernel<T, POW2, 4><<<grd, blk, 0, s>>>(P, p); break;
        }
        return cudaGetLastError();
    }
    dim3 blk(64, 4);
    dim3 grd((p.nx + blk.x - 1) / blk.x, (p.ny + blk.y - 1) / blk.y);
    switch (pass) {
        case 1: gs_pass_kernel<T, POW2, 1><<<grd, blk, 0, s>>>(P, p); break;
        case 2: gs_pass_kernel<T, POW2, 2><<<grd, blk, 0, s>>>(P, p); break;
        case 3: gs_pass_kernel<T, POW2, 3><<<grd, blk, 0, s>>>(P, p); break;
        default: gs_pass_kernel<T, POW2, 4><<<grd, blk, 0, s>>>(P, p); break;
    }
    return cudaGetLastError();
}

using GsPassFn64 = cudaError_t (*)(int, const GsPlanes&, const GsParams<double>&, cudaStream_t);
using GsPassFn32 = cudaError_t (*)(int, const GsPlanes&, const GsParams<float>&, cudaStream_t);

// parity (no contraction) FP64 passes, from inst_parity_stencil.cu
GsPassFn64 gs_parity_pass(bool pow2);

}  // namespace degpu
