// noalloc.cu — degpu_solve_ensemble_noalloc: the persistent multi-family ensemble solve whose
// work lists live in a fixed device array of this library instead of memory allocated per call.
//
// Who needs it: callers that must not allocate device memory while they run.  Examples are an
// application that reserves the whole device memory pool for itself at start-up and forbids any
// later cudaMalloc (to keep its footprint fixed and avoid fragmentation), and a latency-critical
// loop that cannot afford an allocator call in its step (cudaMalloc/cudaFree may synchronise the
// device).  Such a caller still provides the inputs and outputs; the few megabytes of work-list
// space the solve needs come from `noalloc_scratch` below.
//
// The array is part of the library's device code.  CUDA loads a library's device code lazily
// by default (CUDA_MODULE_LOADING=LAZY), so on each device the array and the solve's kernels are
// loaded by the first call that needs them: that loading is the one device allocation this entry
// point causes.  A caller that reserves the device's memory for itself makes one call (any small
// batch) on each device first, before it reserves the pool and before any stream capture; from
// then on the array stays resident until the process exits and no call allocates.  All calls
// share it and it keeps the previous call's contents, so each call first clears the part that
// must start at zero; two calls whose work overlaps on the GPU (different streams, or different
// host threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include "registry.cuh"

namespace degpu {

namespace {

constexpr int NA_NB = 128;    // cost buckets per family
constexpr int NA_LISTS = 6;   // (precision class, family): class 1 = FP64 part of a mixed solve
constexpr int64_t NA_MAX = DEGPU_NOALLOC_MAX_INSTANCES;

// layout of the scratch array (bytes)
constexpr size_t NA_CELLS = 0;                                   // int[NA_LISTS * NA_NB]
constexpr size_t NA_START = NA_CELLS + NA_LISTS * NA_NB * 4;     // int64[NA_LISTS]
constexpr size_t NA_COUNT = NA_START + NA_LISTS * 8;             // int64[NA_LISTS]
constexpr size_t NA_HEAD = NA_COUNT + NA_LISTS * 8;              // u64[NA_LISTS]
constexpr size_t NA_ZERO_END = NA_HEAD + NA_LISTS * 8;           // cleared by every call
constexpr size_t NA_ITEMS = (NA_ZERO_END + 255) / 256 * 256;     // int64[NA_MAX]
constexpr size_t NA_POS = NA_ITEMS + (size_t)NA_MAX * 8;         // int[NA_MAX]
constexpr size_t NA_KEY = NA_POS + (size_t)NA_MAX * 4;           // int[NA_MAX]
constexpr size_t NA_BYTES = NA_KEY + (size_t)NA_MAX * 4;

static __device__ __align__(256) unsigned char noalloc_scratch[NA_BYTES];

// The array's device address on the current device, looked up on every call: a cached address
// would outlive a cudaDeviceReset or a new primary context, and once the module is loaded the
// lookup is a host-side table query.
degpu_status scratch_address(void** out) {
    void* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, noalloc_scratch) != cudaSuccess || !p) return DEGPU_CUDA_ERROR;
    *out = p;
    return DEGPU_OK;
}

__device__ __forceinline__ int na_slot(int id) {
    return id == DEGPU_RHS_VAN_DER_POL ? 0 : id == DEGPU_RHS_PENDULUM ? 1 : id == DEGPU_RHS_LORENZ ? 2 : -1;
}

// Precision class (1: rtol below the mixed-precision bound `split`), cost key and (class,
// family, bucket) position; an instance of another family is reported as BadInput and left out
// of the lists.
__global__ void na_count_kernel(int64_t n, const double* t0, const double* tf, const double* rtol,
                                const double* params, int n_params, const int32_t* family, int fam_const,
                                double inv_order, double h0, double split, unsigned char* scratch,
                                int32_t* status, double* y_final, double* t_final, int dmax) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int* cells = (int*)(scratch + NA_CELLS);
    int* pos = (int*)(scratch + NA_POS);
    int* key = (int*)(scratch + NA_KEY);
    int f = na_slot(family ? family[i] : fam_const);
    if (f < 0) {
        // not one of the three families of the fixed lists: BadInput, and NaN where a result
        // would go (status is required whenever a family map is given)
        status[i] = DEGPU_ERR_BAD_INPUT;
        for (int c = 0; c < dmax; ++c) y_final[(int64_t)c * n + i] = __longlong_as_double(0x7ff8000000000000ll);
        if (t_final) t_final[i] = __longlong_as_double(0x7ff8000000000000ll);
        key[i] = -1;
        return;
    }
    double span = fabs(tf[i] - t0[i]);
    double c = plan_log2_cost(f, span, rtol[i], inv_order, h0, params, n, i, n_params);
    if (!isfinite(c)) c = 0.0;
    int b = (int)floor((c + 24.0) * 1.5);
    b = b < 0 ? 0 : (b > NA_NB - 1 ? NA_NB - 1 : b);
    const int cls = rtol[i] < split ? 1 : 0;
    int k = (cls * 3 + f) * NA_NB + (NA_NB - 1 - b);
    pos[i] = atomicAdd(&cells[k], 1);
    key[i] = k;
}

__global__ void na_scan_kernel(unsigned char* scratch) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int* cells = (int*)(scratch + NA_CELLS);
    int64_t* start = (int64_t*)(scratch + NA_START);
    int64_t* count = (int64_t*)(scratch + NA_COUNT);
    int64_t run = 0;
    for (int f = 0; f < NA_LISTS; ++f) {
        start[f] = run;
        for (int b = 0; b < NA_NB; ++b) {
            int c = cells[f * NA_NB + b];
            cells[f * NA_NB + b] = (int)run;
            run += c;
        }
        count[f] = run - start[f];
    }
}

__global__ void na_scatter_kernel(int64_t n, unsigned char* scratch) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int* key = (const int*)(scratch + NA_KEY);
    int k = key[i];
    if (k < 0) return;
    const int* cells = (const int*)(scratch + NA_CELLS);
    const int* pos = (const int*)(scratch + NA_POS);
    int64_t* items = (int64_t*)(scratch + NA_ITEMS);
    items[cells[k] + pos[i]] = i;
}

}  // namespace
}  // namespace degpu

using namespace degpu;

extern "C" degpu_status degpu_solve_ensemble_noalloc(const degpu_problem* pb, const degpu_method_cfg* cfg,
                                                     const degpu_batch_in* in, degpu_batch_out* out, void* stream) {
    // the checks degpu_solve_ensemble makes, then the limits of this entry point
    degpu_status v = validate_solve_args(pb, cfg, in, out);
    if (v != DEGPU_OK) return v;
    if (in->n > NA_MAX) return DEGPU_BAD_INPUT;  // beyond DEGPU_NOALLOC_MAX_INSTANCES
    if (in->n == 0) return DEGPU_OK;
    if (cfg->method > DEGPU_CASH_KARP) return DEGPU_UNSUPPORTED;  // Verner's pairs: not in the fixed lists
    if (in->n_eval > 0 || in->dims) return DEGPU_UNSUPPORTED;
    if (in->family) {
        // the family map is on the device: the rows must have room for every family, and the
        // per-instance status is where an instance of an unsupported family is reported
        if (pb->dim < 3 || pb->n_params < 3 || !in->params || !out->status) return DEGPU_BAD_INPUT;
    } else {
        const int id = pb->rhs_id;
        if (id != DEGPU_RHS_LORENZ && id != DEGPU_RHS_VAN_DER_POL && id != DEGPU_RHS_PENDULUM) return DEGPU_UNSUPPORTED;
    }
    ensure_registered();
    auto it = multi_registry().find({cfg->method, cfg->precision, 0});
    if (it == multi_registry().end()) return DEGPU_UNSUPPORTED;
    const double split = mixed_split(cfg);
    MultiLaunchFn fp64_launch = nullptr;
    if (split > 0.0) {
        auto it64 = multi_registry().find({cfg->method, mixed_low_precision(cfg), 0});
        if (it64 == multi_registry().end()) it64 = multi_registry().find({cfg->method, DEGPU_FP64_FAST, 0});
        if (it64 == multi_registry().end()) return DEGPU_UNSUPPORTED;
        fp64_launch = it64->second;
    }
    void* base = nullptr;
    degpu_status st = scratch_address(&base);
    if (st != DEGPU_OK) return st;
    unsigned char* scratch = (unsigned char*)base;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n = in->n;

    // the lists, counts and heads from the previous call are still in the array: clear them
    if (cudaMemsetAsync(scratch, 0, NA_ZERO_END, s) != cudaSuccess) return DEGPU_CUDA_ERROR;
    const double inv_order = method_inv_order(cfg->method);
    const unsigned blocks = (unsigned)((n + 255) / 256);
    na_count_kernel<<<blocks, 256, 0, s>>>(n, in->t0, in->tf, in->rtol, in->params, pb->n_params, in->family,
                                           pb->rhs_id, inv_order, cfg->h0 != 0.0 ? cfg->h0 : 1.0, split, scratch,
                                           out->status, out->y_final, out->t_final, pb->dim);
    na_scan_kernel<<<1, 32, 0, s>>>(scratch);
    na_scatter_kernel<<<blocks, 256, 0, s>>>(n, scratch);
    if (cudaGetLastError() != cudaSuccess) return DEGPU_CUDA_ERROR;

    EnsArgs a{};
    a.n = n;
    a.count = n;
    a.t0 = in->t0;
    a.tf = in->tf;
    a.y0 = in->y0;
    a.params = in->params;
    a.rtol = in->rtol;
    a.atol = in->atol;
    a.rtol_vec = in->rtol_vec;
    a.atol_vec = in->atol_vec;
    a.dmax = pb->dim;
    a.y_final = out->y_final;
    a.t_final = out->t_final;
    a.accepted = out->accepted;
    a.rejected = out->rejected;
    a.fevals = out->fevals;
    a.status = out->status;
    a.h0 = cfg->h0;
    a.h_min = cfg->h_min;
    a.h_max = cfg->h_max;
    a.max_steps = cfg->max_steps;
    a.safety = cfg->safety_factor;
    a.min_scale = cfg->min_scale;
    a.max_scale = cfg->max_scale;
    a.safety_f = (float)a.safety;
    a.min_scale_f = (float)a.min_scale;
    a.max_scale_f = (float)a.max_scale;
    a.dense_mode = cfg->dense_mode;
    a.n_params = pb->n_params;
    const int64_t* items = (const int64_t*)(scratch + NA_ITEMS);
    const int64_t* start = (const int64_t*)(scratch + NA_START);
    const int64_t* count = (const int64_t*)(scratch + NA_COUNT);
    unsigned long long* head = (unsigned long long*)(scratch + NA_HEAD);
    // the FP64 lists of a mixed solve first (class 1: lists 3..5), then class 0
    if (fp64_launch) {
        MultiQueue q64{items, start + 3, count + 3, head + 3};
        if (fp64_launch(a, q64, n, s) != cudaSuccess) return DEGPU_CUDA_ERROR;
    }
    MultiQueue q{items, start, count, head};
    return it->second(a, q, n, s) == cudaSuccess ? DEGPU_OK : DEGPU_CUDA_ERROR;
}
