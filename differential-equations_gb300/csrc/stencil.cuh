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
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace degpu {

template <class T>
struct GsParams {
    int nx, ny;
    T Du, Dv, F, k, dx, inv_dx;
    T ah;       // stage coefficient a_{i,i-1} * h
    T bh0, bh1; // accumulation coefficients b_i * h of the pass
};

template <class T, bool POW2>
__device__ __forceinline__ T gs_ddx(T a, const GsParams<T>& p) {
    if constexpr (POW2)
        return a * p.inv_dx;
    else
        return a / p.dx;
}

// f at node (i, j); `get(i, j, u, v)` returns the stage state at a node.
template <class T, bool POW2, class Get>
__device__ __forceinline__ void gs_rhs_at(int i, int j, const GsParams<T>& p, Get get, T& du, T& dv) {
    const int im = i == 0 ? p.nx - 1 : i - 1, ip = i == p.nx - 1 ? 0 : i + 1;
    const int jm = j == 0 ? p.ny - 1 : j - 1, jp = j == p.ny - 1 ? 0 : j + 1;
    T u, v;
    get(i, j, u, v);
    T uvv = u * v * v;
    T a_u = -uvv + p.F * ((T)1 - u);
    T a_v = uvv - (p.F + p.k) * v;
    T ul, vl, ur, vr;
    get(im, j, ul, vl);
    get(ip, j, ur, vr);
    {
        T flo_u = p.Du * gs_ddx<T, POW2>(u - ul, p);
        T fhi_u = p.Du * gs_ddx<T, POW2>(ur - u, p);
        a_u = a_u + gs_ddx<T, POW2>(fhi_u - flo_u, p);
        T flo_v = p.Dv * gs_ddx<T, POW2>(v - vl, p);
        T fhi_v = p.Dv * gs_ddx<T, POW2>(vr - v, p);
        a_v = a_v + gs_ddx<T, POW2>(fhi_v - flo_v, p);
    }
    T ud, vd, uu, vu;
    get(i, jm, ud, vd);
    get(i, jp, uu, vu);
    {
        T flo_u = p.Du * gs_ddx<T, POW2>(u - ud, p);
        T fhi_u = p.Du * gs_ddx<T, POW2>(uu - u, p);
        a_u = a_u + gs_ddx<T, POW2>(fhi_u - flo_u, p);
        T flo_v = p.Dv * gs_ddx<T, POW2>(v - vd, p);
        T fhi_v = p.Dv * gs_ddx<T, POW2>(vu - v, p);
        a_v = a_v + gs_ddx<T, POW2>(fhi_v - flo_v, p);
    }
    du = a_u;
    dv = a_v;
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
            u = __ldg(yu + q) + ah * __ldg(ku + q);
            v = __ldg(yv + q) + ah * __ldg(kv + q);
        };
        gs_rhs_at<T, POW2>(i, j, p, get, du, dv);
        if constexpr (PASS == 1) {
            const T* k0u = (const T*)P.k0u;
            const T* k0v = (const T*)P.k0v;
            T au = yu[c] + p.bh0 * k0u[c];
            T av = yv[c] + p.bh0 * k0v[c];
            ((T*)P.accu)[c] = au + p.bh1 * du;
            ((T*)P.accv)[c] = av + p.bh1 * dv;
            ((T*)P.ou)[c] = du;
            ((T*)P.ov)[c] = dv;
        } else if constexpr (PASS == 2) {
            T* accu = (T*)P.accu;
            T* accv = (T*)P.accv;
            accu[c] = accu[c] + p.bh0 * du;
            accv[c] = accv[c] + p.bh0 * dv;
            ((T*)P.ou)[c] = du;
            ((T*)P.ov)[c] = dv;
        } else {
            const T* accu = (const T*)P.accu;
            const T* accv = (const T*)P.accv;
            ((T*)P.ynu)[c] = accu[c] + p.bh0 * du;
            ((T*)P.ynv)[c] = accv[c] + p.bh0 * dv;
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

// one node's f from its stage state and its four neighbours (gs_rhs_at's operation order)
template <class T, bool POW2>
__device__ __forceinline__ void gs_node(const GsParams<T>& p, T u, T v, T ul, T vl, T ur, T vr, T ud, T vd, T uu,
                                        T vu, T& du, T& dv) {
    T uvv = u * v * v;
    T a_u = -uvv + p.F * ((T)1 - u);
    T a_v = uvv - (p.F + p.k) * v;
    {
        T flo_u = p.Du * gs_ddx<T, POW2>(u - ul, p);
        T fhi_u = p.Du * gs_ddx<T, POW2>(ur - u, p);
        a_u = a_u + gs_ddx<T, POW2>(fhi_u - flo_u, p);
        T flo_v = p.Dv * gs_ddx<T, POW2>(v - vl, p);
        T fhi_v = p.Dv * gs_ddx<T, POW2>(vr - v, p);
        a_v = a_v + gs_ddx<T, POW2>(fhi_v - flo_v, p);
    }
    {
        T flo_u = p.Du * gs_ddx<T, POW2>(u - ud, p);
        T fhi_u = p.Du * gs_ddx<T, POW2>(uu - u, p);
        a_u = a_u + gs_ddx<T, POW2>(fhi_u - flo_u, p);
        T flo_v = p.Dv * gs_ddx<T, POW2>(v - vd, p);
        T fhi_v = p.Dv * gs_ddx<T, POW2>(vu - v, p);
        a_v = a_v + gs_ddx<T, POW2>(fhi_v - flo_v, p);
    }
    du = a_u;
    dv = a_v;
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
                su[r][q] = a.v[q] + ah * c.v[q];
                sv[r][q] = b.v[q] + ah * d.v[q];
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
                eu = eu + ah * __ldg(ku + o);
                ev = ev + ah * __ldg(kv + o);
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
                au.v[q] = (y_u.v[q] + p.bh0 * k_u.v[q]) + p.bh1 * du.v[q];
                av.v[q] = (y_v.v[q] + p.bh0 * k_v.v[q]) + p.bh1 * dv.v[q];
            }
            st4((T*)P.accu + o, au);
            st4((T*)P.accv + o, av);
            st4((T*)P.ou + o, du);
            st4((T*)P.ov + o, dv);
        } else if constexpr (PASS == 2) {
            Vec4<T> au = ld4((const T*)P.accu + o), av = ld4((const T*)P.accv + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                au.v[q] = au.v[q] + p.bh0 * du.v[q];
                av.v[q] = av.v[q] + p.bh0 * dv.v[q];
            }
            st4((T*)P.accu + o, au);
            st4((T*)P.accv + o, av);
            st4((T*)P.ou + o, du);
            st4((T*)P.ov + o, dv);
        } else {
            Vec4<T> au = ld4((const T*)P.accu + o), av = ld4((const T*)P.accv + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                au.v[q] = au.v[q] + p.bh0 * du.v[q];
                av.v[q] = av.v[q] + p.bh0 * dv.v[q];
            }
            st4((T*)P.ynu + o, au);
            st4((T*)P.ynv + o, av);
        }
    }
}

// Launchers for one precision (instantiated in stencil.cu and, for the parity build, in
// inst_parity_stencil.cu with -fmad=false).
template <class T, bool POW2>
cudaError_t gs_launch_pass(int pass, const GsPlanes& P, const GsParams<T>& p, cudaStream_t s) {
    if (p.nx % 128 == 0 && p.ny % 16 == 0) {
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
