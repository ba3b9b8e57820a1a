// stencil.cu — host side of the Gray–Scott method-of-lines path (degpu_gray_scott_rk4 /
// degpu_gray_scott_rhs).  The RK4 step loop is captured once into a CUDA graph (two steps per
// graph, because the state is double-buffered) and replayed, so a 1000-step run costs ~500 graph
// launches instead of 4000 kernel launches.
#include <math.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/degpu.h"
#include "stencil.cuh"

namespace degpu {

static bool is_pow2(double x) {
    if (!(x > 0.0) || !isfinite(x)) return false;
    int e;
    double m = frexp(x, &e);
    return m == 0.5;
}

// The fused FP32 step (one launch per RK4 step, gs_step_fused_kernel) replaces the four passes
// where the grid divides into its tiles (nx % 64 == 0, ny % 32 == 0); degpu_internal_gs_fused_step(0) turns it off (the tests
// compare the two).
// tiles of 64 x 32 nodes, 512 threads, two blocks (2 x 92 KB of shared memory) per SM: measured
// on 4096^2 with one node per thread and scalar halo loads, 0.239 ms per step against 0.246 ms for
// 32 x 32 tiles with 256 threads, 0.251 ms for 32 x 32 with 512 and 0.300 ms for 64 x 32 with 256
// (the four passes: 0.317 ms); with two rows per thread and 16-byte halo loads, 0.202 ms
#ifndef DEGPU_GS_TX
#define DEGPU_GS_TX 64
#define DEGPU_GS_TY 32
#endif
constexpr int GS_TX = DEGPU_GS_TX, GS_TY = DEGPU_GS_TY;
static std::atomic<int> g_gs_fused{1};

// the kernel's shared-memory opt-in (92 KB), set on each device before the first launch there
// (and so outside any stream capture)
template <bool POW2>
static cudaError_t gs_fused_prepare() {
    static std::mutex mu;
    static std::vector<int> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, 0);
    if (done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(gs_step_fused_kernel<POW2, GS_TX, GS_TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gs_fused_smem<GS_TX, GS_TY>());
    if (e == cudaSuccess) done[dev] = 1;
    return e;
}

template <bool POW2>
static cudaError_t gs_fused_launch(const GsFusedPlanes& P, const GsParams<float>& p, const GsFusedCoef& cf,
                                   cudaStream_t s) {
    constexpr size_t smem = gs_fused_smem<GS_TX, GS_TY>();
    dim3 grd(p.nx / GS_TX, p.ny / GS_TY);
    gs_step_fused_kernel<POW2, GS_TX, GS_TY><<<grd, GS_FUSED_THREADS, smem, s>>>(P, p, cf);
    return cudaGetLastError();
}

template <class T>
struct GsRun {
    using Fn = cudaError_t (*)(int, const GsPlanes&, const GsParams<T>&, cudaStream_t);
    Fn fn;
    GsParams<T> p;
    double h;
    bool fused = false;  // FP32 only: one fused launch per step, k0 alternating between buf[0..1] and buf[2..3]
    bool pow2 = true;
    T* buf[10];  // k0u k0v k1u k1v k2u k2v accu accv ybu ybv

    cudaError_t pass4(const void* yu, const void* yv, cudaStream_t s) {
        GsPlanes P{};
        P.yu = yu;
        P.yv = yv;
        P.ou = buf[0];
        P.ov = buf[1];
        return fn(4, P, p, s);
    }
    // one RK4 step from (yu, yv) into (nu, nv); k0 in buf[0..1] on entry and exit (the fused
    // form: in buf[2 kin .. 2 kin + 1] on entry, in the other pair on exit)
    cudaError_t step(const void* yu, const void* yv, void* nu, void* nv, cudaStream_t s, int kin = 0) {
        const double b0 = 1.0 / 6.0, b1 = 1.0 / 3.0, b2 = 1.0 / 3.0, b3 = 1.0 / 6.0;
        if constexpr (sizeof(T) == 4) {
            if (fused) {
                GsFusedPlanes F{};
                F.yu = (const float*)yu;
                F.yv = (const float*)yv;
                F.ku = (const float*)buf[2 * kin];
                F.kv = (const float*)buf[2 * kin + 1];
                F.nu = (float*)nu;
                F.nv = (float*)nv;
                F.knu = (float*)buf[2 - 2 * kin];
                F.knv = (float*)buf[3 - 2 * kin];
                // the passes' coefficients, rounded the same way
                GsFusedCoef cf{(T)(0.5 * h), (T)(0.5 * h), (T)(1.0 * h), (T)(b0 * h), (T)(b1 * h), (T)(b2 * h),
                               (T)(b3 * h)};
                return pow2 ? gs_fused_launch<true>(F, p, cf, s) : gs_fused_launch<false>(F, p, cf, s);
            }
        }
        GsPlanes P{};
        P.yu = yu;
        P.yv = yv;
        cudaError_t e;
        // pass 1: k1 = f(y + (0.5 h) k0); acc = (y + (b0 h) k0) + (b1 h) k1
        GsParams<T> q = p;
        q.ah = (T)(0.5 * h);
        q.bh0 = (T)(b0 * h);
        q.bh1 = (T)(b1 * h);
        P.ku = buf[0]; P.kv = buf[1]; P.k0u = buf[0]; P.k0v = buf[1];
        P.ou = buf[2]; P.ov = buf[3]; P.accu = buf[6]; P.accv = buf[7];
        if ((e = fn(1, P, q, s)) != cudaSuccess) return e;
        // pass 2: k2 = f(y + (0.5 h) k1); acc += (b2 h) k2
        q.ah = (T)(0.5 * h);
        q.bh0 = (T)(b2 * h);
        P.ku = buf[2]; P.kv = buf[3]; P.ou = buf[4]; P.ov = buf[5];
        if ((e = fn(2, P, q, s)) != cudaSuccess) return e;
        // pass 3: k3 = f(y + (1.0 h) k2); y_next = acc + (b3 h) k3
        q.ah = (T)(1.0 * h);
        q.bh0 = (T)(b3 * h);
        P.ku = buf[4]; P.kv = buf[5]; P.ynu = nu; P.ynv = nv;
        if ((e = fn(3, P, q, s)) != cudaSuccess) return e;
        // pass 4: k0 = f(y_next)
        return pass4(nu, nv, s);
    }
};

template <class T>
static degpu_status gs_run(const degpu_gray_scott* gs, typename GsRun<T>::Fn fn, double dt, int64_t steps, T* u, T* v,
                           cudaStream_t s, bool pow2 = true) {
    const size_t N = (size_t)gs->nx * gs->ny;
    GsRun<T> R;
    R.fn = fn;
    R.h = dt;
    R.pow2 = pow2;
    // the fused step loads y in 16-byte chunks: the caller's planes must start on 16-byte boundaries
    R.fused = sizeof(T) == 4 && g_gs_fused && gs->nx % GS_TX == 0 && gs->ny % GS_TY == 0 &&
              ((uintptr_t)u & 15u) == 0 && ((uintptr_t)v & 15u) == 0;
    if (R.fused && (pow2 ? gs_fused_prepare<true>() : gs_fused_prepare<false>()) != cudaSuccess)
        return DEGPU_CUDA_ERROR;
    R.p.nx = gs->nx;
    R.p.ny = gs->ny;
    R.p.Du = (T)gs->Du;
    R.p.Dv = (T)gs->Dv;
    R.p.F = (T)gs->F;
    R.p.k = (T)gs->k;
    R.p.dx = (T)gs->dx;
    R.p.inv_dx = (T)(1.0 / gs->dx);
    R.p.cu = (T)(gs->Du / (gs->dx * gs->dx));
    R.p.cv = (T)(gs->Dv / (gs->dx * gs->dx));
    void* block = nullptr;
    if (cudaMallocAsync(&block, 10 * N * sizeof(T), s) != cudaSuccess) return DEGPU_OOM;
    for (int q = 0; q < 10; ++q) R.buf[q] = (T*)block + q * N;
    degpu_status st = DEGPU_OK;
    T* ya[2] = {u, R.buf[8]};
    T* yb[2] = {v, R.buf[9]};
    int cur = 0;
    // init: k0 = f(t0, y0)  (fixed/ordinary.rs:44)
    if (R.pass4(u, v, s) != cudaSuccess) st = DEGPU_CUDA_ERROR;
    int64_t done = 0;
    if (st == DEGPU_OK && steps >= 2) {
        // capture two steps (y -> B -> y) into a graph on a private stream
        cudaStream_t cs;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) st = DEGPU_CUDA_ERROR;
        if (st == DEGPU_OK) {
            cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
            cudaError_t e1 = R.step(ya[0], yb[0], ya[1], yb[1], cs, 0);
            cudaError_t e2 = R.step(ya[1], yb[1], ya[0], yb[0], cs, 1);
            cudaError_t ec = cudaStreamEndCapture(cs, &g);
            if (e1 != cudaSuccess || e2 != cudaSuccess || ec != cudaSuccess ||
                cudaGraphInstantiate(&ge, g, 0) != cudaSuccess)
                st = DEGPU_CUDA_ERROR;
            cudaStreamDestroy(cs);
        }
        for (; st == DEGPU_OK && done + 2 <= steps; done += 2)
            if (cudaGraphLaunch(ge, s) != cudaSuccess) st = DEGPU_CUDA_ERROR;
        if (ge) cudaGraphExecDestroy(ge);
        if (g) cudaGraphDestroy(g);
    }
    if (st == DEGPU_OK && done < steps) {
        if (R.step(ya[0], yb[0], ya[1], yb[1], s, 0) != cudaSuccess) st = DEGPU_CUDA_ERROR;
        cur = 1;
        done += 1;
    }
    if (st == DEGPU_OK && cur == 1) {
        if (cudaMemcpyAsync(u, ya[1], N * sizeof(T), cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(v, yb[1], N * sizeof(T), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            st = DEGPU_CUDA_ERROR;
    }
    cudaFreeAsync(block, s);
    return st;
}

}  // namespace degpu

using namespace degpu;

extern "C" {

degpu_status degpu_gray_scott_rk4(const degpu_gray_scott* gs, int32_t precision, double t0, double dt, int64_t steps,
                                  void* u, void* v, void* stream) {
    (void)t0;  // the Gray–Scott right-hand side is autonomous
    if (!gs || !u || !v || gs->nx < 3 || gs->ny < 3 || steps < 0 || !(dt > 0.0) || !(gs->dx > 0.0))
        return DEGPU_BAD_INPUT;
    if (steps == 0) return DEGPU_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const bool p2 = is_pow2(gs->dx);
    switch (precision) {
        case DEGPU_FP64_PARITY:
            return gs_run<double>(gs, gs_parity_pass(p2), dt, steps, (double*)u, (double*)v, s);
        case DEGPU_FP64_FAST:
            return gs_run<double>(gs, p2 ? &gs_launch_pass<double, true> : &gs_launch_pass<double, false>, dt, steps,
                                  (double*)u, (double*)v, s);
        case DEGPU_MIXED:
            return gs_run<float>(gs, &gs_launch_pass<float, true>, dt, steps, (float*)u, (float*)v, s, true);
        default:
            return DEGPU_BAD_INPUT;
    }
}

// Internal: the fused FP32 step on (1) or off (0); returns the previous setting.
int degpu_internal_gs_fused_step(int on) {
    return g_gs_fused.exchange(on ? 1 : 0);
}

degpu_status degpu_gray_scott_rhs(const degpu_gray_scott* gs, const double* u, const double* v, double* du, double* dv,
                                  void* stream) {
    if (!gs || !u || !v || !du || !dv || gs->nx < 3 || gs->ny < 3 || !(gs->dx > 0.0)) return DEGPU_BAD_INPUT;
    GsParams<double> p{};
    p.nx = gs->nx;
    p.ny = gs->ny;
    p.Du = gs->Du;
    p.Dv = gs->Dv;
    p.F = gs->F;
    p.k = gs->k;
    p.dx = gs->dx;
    p.inv_dx = 1.0 / gs->dx;
    GsPlanes P{};
    P.yu = u;
    P.yv = v;
    P.ou = du;
    P.ov = dv;
    return gs_parity_pass(is_pow2(gs->dx))(4, P, p, (cudaStream_t)stream) == cudaSuccess ? DEGPU_OK
                                                                                          : DEGPU_CUDA_ERROR;
}

}  // extern "C"
