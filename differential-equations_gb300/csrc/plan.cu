// plan.cu — longest-first work lists for the multi-family persistent kernel.
//
// Three small kernels, no host round trip:
//   count   : each instance gets a precision class (1 when a mixed solve sends it to FP64
//             because its rtol is below the mixed-precision bound, else 0), a cost key
//             (plan_log2_cost: log2 scale, 128 buckets, descending) and a position inside its
//             (class, family, bucket) cell by atomic increment;
//   scan    : exclusive scan over the 2 x 3 x 128 cells -> list offsets, list starts and lengths;
//   scatter : items[offset(cell) + position] = instance.
// Then one persistent launch per class: FP64 first (its instances are the most expensive ones),
// the mixed kernel after it; or, for the run-to-completion layout, one launch per list.
// Ordering inside a bucket follows the atomics and is not deterministic; every instance's result
// is independent of the order in which instances are taken, so solutions are deterministic.
#include <mutex>
#include <cuda_runtime.h>
#include <math.h>

#include "registry.cuh"

namespace degpu {

std::map<std::tuple<int, int, int>, MultiLaunchFn>& multi_registry() {
    static std::map<std::tuple<int, int, int>, MultiLaunchFn> m;
    return m;
}

static constexpr int NB = 128;

__device__ __forceinline__ int fam_slot(int id) {
    return id == DEGPU_RHS_VAN_DER_POL ? 0 : id == DEGPU_RHS_PENDULUM ? 1 : id == DEGPU_RHS_LORENZ ? 2 : -1;
}

static constexpr int NLISTS = 6;  // (class, family)

__global__ void plan_count_kernel(int64_t n, const double* t0, const double* tf, const double* rtol,
                                  const double* params, int n_params, const int32_t* family, int fam_const,
                                  double inv_order, double h0, double split, int* cells, int* pos, int* key,
                                  int* bad) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int f = fam_slot(family ? family[i] : fam_const);
    if (f < 0) {
        atomicExch(bad, 1);
        f = 0;
    }
    double span = fabs(tf[i] - t0[i]);
    double c = plan_log2_cost(f, span, rtol[i], inv_order, h0, params, n, i, n_params);
    if (!isfinite(c)) c = 0.0;
    int b = (int)floor((c + 24.0) * 1.5);
    b = b < 0 ? 0 : (b > NB - 1 ? NB - 1 : b);
    const int cls = rtol[i] < split ? 1 : 0;  // split = 0: every instance in class 0
    int k = (cls * 3 + f) * NB + (NB - 1 - b);  // descending cost
    pos[i] = atomicAdd(&cells[k], 1);
    key[i] = k;
}

__global__ void plan_scan_kernel(int* cells, int64_t* start, int64_t* count) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int64_t run = 0;
    for (int f = 0; f < NLISTS; ++f) {
        start[f] = run;
        for (int b = 0; b < NB; ++b) {
            int c = cells[f * NB + b];
            cells[f * NB + b] = (int)run;
            run += c;
        }
        count[f] = run - start[f];
    }
}

__global__ void plan_scatter_kernel(int64_t n, const int* pos, const int* key, const int* cells, int64_t* items) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    items[cells[key[i]] + pos[i]] = i;
}

// Scratch of one plan: cells, start, count, head, bad, items, pos, key.
struct Plan {
    char* blk = nullptr;
    int64_t* items = nullptr;
    int64_t* start = nullptr;  // [NLISTS]
    int64_t* count = nullptr;  // [NLISTS]
    unsigned long long* head = nullptr;
};

// Runs count/scan/scatter into a fresh stream-ordered scratch block (freed by the caller).
static degpu_status run_plan(const degpu_method_cfg* cfg, const EnsArgs& a, const int32_t* family_dev,
                             int fam_const, double split, Plan& pl, cudaStream_t s) {
    const int64_t n = a.n;
    const size_t cells_bytes = ((size_t)NB * NLISTS * 4 + 7) / 8 * 8;
    const size_t head_bytes = cells_bytes + NLISTS * 8 * 3 + 8;
    size_t bytes = head_bytes + n * 8 + n * 4 + n * 4 + 64;
    if (cudaMallocAsync((void**)&pl.blk, bytes, s) != cudaSuccess) return DEGPU_OOM;
    int* cells = (int*)pl.blk;
    pl.start = (int64_t*)(pl.blk + cells_bytes);
    pl.count = pl.start + NLISTS;
    pl.head = (unsigned long long*)(pl.count + NLISTS);
    int* bad = (int*)(pl.head + NLISTS);
    pl.items = (int64_t*)(pl.blk + head_bytes);
    int* pos = (int*)(pl.items + n);
    int* key = pos + n;
    if (cudaMemsetAsync(pl.blk, 0, head_bytes, s) != cudaSuccess) return DEGPU_CUDA_ERROR;
    const double inv_order = method_inv_order(cfg->method);
    unsigned blocks = (unsigned)((n + 255) / 256);
    plan_count_kernel<<<blocks, 256, 0, s>>>(n, a.t0, a.tf, a.rtol, a.params, a.n_params, family_dev, fam_const,
                                              inv_order, cfg->h0 != 0.0 ? cfg->h0 : 1.0, split, cells, pos, key,
                                              bad);
    plan_scan_kernel<<<1, 32, 0, s>>>(cells, pl.start, pl.count);
    plan_scatter_kernel<<<blocks, 256, 0, s>>>(n, pos, key, cells, pl.items);
    return cudaGetLastError() == cudaSuccess ? DEGPU_OK : DEGPU_CUDA_ERROR;
}

// One non-blocking helper stream per device (created on first use) for the second class of a
// split solve.
static cudaStream_t helper_stream() {
    static std::mutex mu;
    static cudaStream_t per_dev[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> g(mu);
    if (!per_dev[dev] && cudaStreamCreateWithFlags(&per_dev[dev], cudaStreamNonBlocking) != cudaSuccess)
        per_dev[dev] = nullptr;
    return per_dev[dev];
}

// Plans and launches one multi-family persistent solve (two launches when a mixed solve splits
// by rtol).  Returns DEGPU_UNSUPPORTED when no kernel is registered for the combination.
degpu_status multi_solve(const degpu_method_cfg* cfg, const EnsArgs& a, const int32_t* family_dev, int fam_const,
                         bool dense, cudaStream_t s, bool crossing) {
    const int d = crossing ? 2 : (dense ? 1 : 0);
    auto it = multi_registry().find({cfg->method, cfg->precision, d});
    if (it == multi_registry().end()) return DEGPU_UNSUPPORTED;
    const double split = mixed_split(cfg);
    MultiLaunchFn fp64_launch = nullptr;
    if (split > 0.0) {
        // the tight class: FP32-pair stages where built, else FP64
        auto it64 = multi_registry().find({cfg->method, mixed_low_precision(cfg), d});
        if (it64 == multi_registry().end()) it64 = multi_registry().find({cfg->method, DEGPU_FP64_FAST, d});
        if (it64 == multi_registry().end()) return DEGPU_UNSUPPORTED;
        fp64_launch = it64->second;
    }
    const int64_t n = a.n;
    Plan pl;
    degpu_status st = run_plan(cfg, a, family_dev, fam_const, split, pl, s);
    // class 1 (tight) lists: start/count/head [3..6); class 0: [0..3)
    if (st == DEGPU_OK && fp64_launch) {
        // The two classes run concurrently: the second launch goes to a helper stream that waits
        // for the plan, so its blocks take the SMs the first launch frees at its tail; the
        // caller's stream then waits for both.
        cudaStream_t s2 = helper_stream();
        cudaEvent_t planned = nullptr, second = nullptr;
        if (!s2 || cudaEventCreateWithFlags(&planned, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&second, cudaEventDisableTiming) != cudaSuccess) {
            s2 = s;  // no helper: one after the other on the caller's stream
        } else if (cudaEventRecord(planned, s) != cudaSuccess || cudaStreamWaitEvent(s2, planned, 0) != cudaSuccess) {
            st = DEGPU_CUDA_ERROR;
        }
        if (st == DEGPU_OK) {
            MultiQueue q{pl.items, pl.start + 3, pl.count + 3, pl.head + 3};
            if (fp64_launch(a, q, n, s) != cudaSuccess) st = DEGPU_CUDA_ERROR;
        }
        if (st == DEGPU_OK) {
            MultiQueue q{pl.items, pl.start, pl.count, pl.head};
            if (it->second(a, q, n, s2) != cudaSuccess) st = DEGPU_CUDA_ERROR;
        }
        if (s2 != s && second) {
            if (cudaEventRecord(second, s2) != cudaSuccess || cudaStreamWaitEvent(s, second, 0) != cudaSuccess)
                st = DEGPU_CUDA_ERROR;
        }
        if (planned) cudaEventDestroy(planned);
        if (second) cudaEventDestroy(second);
    } else if (st == DEGPU_OK) {
        MultiQueue q{pl.items, pl.start, pl.count, pl.head};
        if (it->second(a, q, n, s) != cudaSuccess) st = DEGPU_CUDA_ERROR;
    }
    if (pl.blk) cudaFreeAsync(pl.blk, s);
    return st;
}

// One run-to-completion launch per (precision class, family) of the production families, each
// over its longest-first work list: the lanes of a warp get instances of similar cost, so a warp
// is not held by one long instance while its other lanes sit finished.
degpu_status sorted_thread_solve(const degpu_method_cfg* cfg, const EnsArgs& a, const int32_t* family_dev,
                                 int fam_const, bool dense, cudaStream_t s, bool crossing) {
    auto& reg = crossing ? cross_registry() : ens_registry();
    const double split = mixed_split(cfg);
    static const int ids[3] = {DEGPU_RHS_VAN_DER_POL, DEGPU_RHS_PENDULUM, DEGPU_RHS_LORENZ};
    Plan pl;
    degpu_status st = run_plan(cfg, a, family_dev, fam_const, split, pl, s);
    int64_t hs[NLISTS] = {}, hc[NLISTS] = {};
    if (st == DEGPU_OK &&
        (cudaMemcpyAsync(hs, pl.start, sizeof(hs), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
         cudaMemcpyAsync(hc, pl.count, sizeof(hc), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
         cudaStreamSynchronize(s) != cudaSuccess))
        st = DEGPU_CUDA_ERROR;
    for (int l = NLISTS - 1; l >= 0 && st == DEGPU_OK; --l) {  // FP64 class first
        if (hc[l] == 0) continue;
        int prec = l >= 3 ? mixed_low_precision(cfg) : cfg->precision;
        auto it = reg.find(VariantKey{cfg->method, ids[l % 3], prec, dense ? 1 : 0});
        if (l >= 3 && it == reg.end()) {
            prec = DEGPU_FP64_FAST;
            it = reg.find(VariantKey{cfg->method, ids[l % 3], prec, dense ? 1 : 0});
        }
        if (it == reg.end()) {
            st = DEGPU_UNSUPPORTED;
            break;
        }
        EnsArgs ga = a;
        ga.index = pl.items + hs[l];
        ga.count = hc[l];
        if (it->second(ga, DEGPU_KERNEL_THREAD, s) != cudaSuccess) st = DEGPU_CUDA_ERROR;
    }
    if (pl.blk) cudaFreeAsync(pl.blk, s);
    return st;
}

}  // namespace degpu
