// registry.cuh — table of compiled (method, family, precision, dense) kernel variants.
//
// Each instantiation translation unit registers launchers for the variants it compiles; the ABI
// looks a variant up by key.  The parity variants live in translation units compiled with
// -fmad=false, so that no multiply-add is contracted into an FMA anywhere on that path.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <tuple>

#include "erk_core.cuh"

namespace degpu {

using EnsLaunchFn = cudaError_t (*)(const EnsArgs& a, int kernel, cudaStream_t s);

struct VariantKey {
    int method, rhs, prec, dense;
    bool operator<(const VariantKey& o) const {
        return std::tie(method, rhs, prec, dense) < std::tie(o.method, o.rhs, o.prec, o.dense);
    }
};

std::map<VariantKey, EnsLaunchFn>& ens_registry();

template <class Tab>
constexpr int method_id() {
    return Tab::METHOD;
}

// 1 / order of the method's error estimate (0 for fixed steps): the rtol exponent of the cost
// model that orders the work lists.
inline double method_inv_order(int method) {
    switch (method) {
        case DEGPU_RK4: return 0.0;
        case DEGPU_DOP853: return 1.0 / 8.0;
        case DEGPU_RKV655E: case DEGPU_RKV656E: return 1.0 / 6.0;
        case DEGPU_RKV766E: case DEGPU_RKV767E: return 1.0 / 7.0;
        case DEGPU_RKV877E: case DEGPU_RKV878E: return 1.0 / 8.0;
        case DEGPU_RKV988E: case DEGPU_RKV989E: return 1.0 / 9.0;
        default: return 1.0 / 5.0;
    }
}

int device_sm_count();

template <class Tab, class Rhs, class P, bool DENSE>
cudaError_t launch_ens(const EnsArgs& a, int kernel, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    if (kernel == DEGPU_KERNEL_PERSISTENT) {
        static int blocks_per_sm = -1;
        if (blocks_per_sm < 0) {
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &blocks_per_sm, erk_persistent_kernel<Tab, Rhs, P, DENSE>, 128, 0);
            if (e != cudaSuccess) return e;
            if (blocks_per_sm < 1) blocks_per_sm = 1;
        }
        long long grid = (long long)blocks_per_sm * device_sm_count();
        long long need = (a.count + 127) / 128;
        if (grid > need) grid = need;
        erk_persistent_kernel<Tab, Rhs, P, DENSE><<<(unsigned)grid, 128, 0, s>>>(a);
    } else {
        long long blocks = (a.count + 127) / 128;
        erk_thread_kernel<Tab, Rhs, P, DENSE><<<(unsigned)blocks, 128, 0, s>>>(a);
    }
    return cudaGetLastError();
}

// Run-to-completion kernels only (a persistent request runs them too).
template <class Tab, class Rhs, class P, bool DENSE>
cudaError_t launch_thread_only(const EnsArgs& a, int, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    erk_thread_kernel<Tab, Rhs, P, DENSE><<<(unsigned)((a.count + 127) / 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

template <class Tab, class Rhs, class P>
void register_thread_variant() {
    ens_registry()[VariantKey{method_id<Tab>(), Rhs::ID, P::ID, 0}] = &launch_thread_only<Tab, Rhs, P, false>;
    ens_registry()[VariantKey{method_id<Tab>(), Rhs::ID, P::ID, 1}] = &launch_thread_only<Tab, Rhs, P, true>;
}

template <class Tab, class Rhs, class P>
void register_variant() {
    ens_registry()[VariantKey{method_id<Tab>(), Rhs::ID, P::ID, 0}] = &launch_ens<Tab, Rhs, P, false>;
    ens_registry()[VariantKey{method_id<Tab>(), Rhs::ID, P::ID, 1}] = &launch_ens<Tab, Rhs, P, true>;
}

// Crossing-detection kernels (degpu_solve_ensemble_crossing), keyed like ens_registry with dense = 1.
std::map<VariantKey, EnsLaunchFn>& cross_registry();

template <class Tab, class Rhs, class P>
cudaError_t launch_cross(const EnsArgs& a, int, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    erk_cross_kernel<Tab, Rhs, P><<<(unsigned)((a.count + 127) / 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

template <class Rhs, class P>
void register_cross_all_methods() {
    cross_registry()[VariantKey{DEGPU_RK4, Rhs::ID, P::ID, 1}] = &launch_cross<TabRK4, Rhs, P>;
    cross_registry()[VariantKey{DEGPU_DOPRI5, Rhs::ID, P::ID, 1}] = &launch_cross<TabDopri5, Rhs, P>;
    cross_registry()[VariantKey{DEGPU_DOP853, Rhs::ID, P::ID, 1}] = &launch_cross<TabDop853, Rhs, P>;
}
// The adaptive (embedded-pair) methods, in their own translation units.
template <class Rhs, class P>
void register_cross_embedded_methods() {
    cross_registry()[VariantKey{DEGPU_RKF45, Rhs::ID, P::ID, 1}] = &launch_cross<TabRKF45, Rhs, P>;
    cross_registry()[VariantKey{DEGPU_CASH_KARP, Rhs::ID, P::ID, 1}] = &launch_cross<TabCashKarp, Rhs, P>;
}

// Resumable round kernels of the serving path, keyed with dense = 1 for the kernels that also
// write output times.
struct RoundOps {
    size_t park_bytes;  // resident state per instance
    cudaError_t (*launch)(const EnsArgs& a, void* park, int budget, unsigned long long* done, int max_blocks,
                          cudaStream_t s);
};
std::map<VariantKey, RoundOps>& round_registry();

template <class Tab, class Rhs, class P, bool DENSE = false>
cudaError_t launch_round(const EnsArgs& a, void* park, int budget, unsigned long long* done, int max_blocks,
                         cudaStream_t s) {
    using L = Lane<Tab, Rhs, P, DENSE>;
    if (a.count <= 0) return cudaSuccess;
    static int blocks_per_sm = -1;
    if (blocks_per_sm < 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm,
                                                                      erk_round_kernel<Tab, Rhs, P, DENSE>, 128, 0);
        if (e != cudaSuccess) return e;
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    long long grid = (long long)blocks_per_sm * device_sm_count();
    long long need = (a.count + 127) / 128;
    if (grid > need) grid = need;
    if (max_blocks > 0 && grid > max_blocks) grid = max_blocks;
    erk_round_kernel<Tab, Rhs, P, DENSE><<<(unsigned)grid, 128, 0, s>>>(a, (Parked<L>*)park, budget, done);
    return cudaGetLastError();
}

template <class Tab, class Rhs, class P, bool DENSE = false>
void register_round() {
    round_registry()[VariantKey{method_id<Tab>(), Rhs::ID, P::ID, DENSE ? 1 : 0}] =
        RoundOps{sizeof(Parked<Lane<Tab, Rhs, P, DENSE>>), &launch_round<Tab, Rhs, P, DENSE>};
}

template <class Rhs, class P, bool DENSE = false>
void register_round_all_methods() {
    register_round<TabRK4, Rhs, P, DENSE>();
    register_round<TabDopri5, Rhs, P, DENSE>();
    register_round<TabDop853, Rhs, P, DENSE>();
}

// Multi-family persistent kernels: families Van der Pol (slot 0), pendulum (1), Lorenz (2).
using MultiLaunchFn = cudaError_t (*)(const EnsArgs& a, const MultiQueue& q, int64_t total, cudaStream_t s);
std::map<std::tuple<int, int, int>, MultiLaunchFn>& multi_registry();

template <class Tab, class P, bool DENSE, bool CROSS = false>
cudaError_t launch_multi(const EnsArgs& a, const MultiQueue& q, int64_t total, cudaStream_t s) {
    auto kern = erk_multi_kernel<Tab, P, DENSE, RhsVanDerPol, RhsPendulum, RhsLorenz, CROSS>;
    static int blocks_per_sm = -1;
    if (blocks_per_sm < 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, 128, 0);
        if (e != cudaSuccess) return e;
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    long long grid = (long long)blocks_per_sm * device_sm_count();
    long long need = (total + 127) / 128;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, 128, 0, s>>>(a, q);
    return cudaGetLastError();
}

// Keys (method, precision, kind): kind 0 final states, 1 output times, 2 crossing / event detection.
template <class Tab, class P>
void register_multi() {
    multi_registry()[{method_id<Tab>(), P::ID, 0}] = &launch_multi<Tab, P, false>;
    multi_registry()[{method_id<Tab>(), P::ID, 1}] = &launch_multi<Tab, P, true>;
}
template <class Tab, class P>
void register_multi_cross() {
    multi_registry()[{method_id<Tab>(), P::ID, 2}] = &launch_multi<Tab, P, true, true>;
}

// Per-translation-unit registration hooks (called once by the ABI).
void register_parity_main();
void register_parity_tests();
void register_fast();
void register_mixed();
void register_parity_multi();
void register_multi_fast_mixed();
void register_multi_cross();
void register_multi_embedded();
void register_cross_parity();
void register_cross_fast_mixed();
void register_cross_embedded_parity();
void register_cross_embedded_fast_mixed();
void register_embedded_parity();
void register_embedded_fast_mixed();
void register_verner65_parity();
void register_verner76_parity();
void register_verner87_parity();
void register_verner98_parity();
void register_verner65_fast();
void register_verner76_fast();
void register_verner87_fast();
void register_verner98_fast();
void register_verner_cross65_parity();
void register_verner_cross76_parity();
void register_verner_cross87_parity();
void register_verner_cross98_parity();
void register_verner_cross6576_fast();
void register_verner_cross8798_fast();
void register_plain();
void register_mixed_f64ctrl();
void register_mixed_pair();
void register_round_dense_parity();
void register_round_dense_fast_mixed();
void register_groups();
void register_mixed_pair853();
void ensure_registered();

// Estimated log2 cost of one instance, the sort key of the longest-first work lists.  Fitted to
// the step counts of 30,000 instances of the uneven Van der Pol / pendulum / Lorenz ensemble
// solved by the CPU restatement (DOPRI5): log2 steps ~ log2 |tf - t0| - 0.875 log2(rtol) / order
// plus a family term in the parameters (Van der Pol: stiffer for larger mu; Lorenz: chaotic for
// rho above 24.74); the residual spread is 0.13-0.33 in log2 against 0.18-0.78 without the family
// terms.  It only orders work: results do not depend on it.  Fixed-step methods use |tf - t0| / h0.
__device__ __forceinline__ double plan_log2_cost(int slot, double span, double rtol, double inv_order, double h0,
                                                 const double* params, int64_t n, int64_t i, int n_params) {
    if (!(inv_order > 0.0)) return log2(span / fabs(h0));
    double c = log2(span) - 0.875 * inv_order * log2(rtol);
    if (params) {
        if (slot == 0 && n_params >= 1) {  // Van der Pol, p = [mu]
            const double lm = log2(params[i]);
            c += 0.37 * lm + 0.024 * lm * lm;
        } else if (slot == 1 && n_params >= 3) {  // pendulum, p = [gamma, A, Omega]
            c += 0.4 * params[2 * n + i];
        } else if (slot == 2 && n_params >= 2) {  // Lorenz, p = [sigma, rho, beta]
            const double rho = params[n + i];
            c += 0.047 * rho + (rho > 24.74 ? 0.38 : 0.0);
        }
    }
    return c;
}

// Longest-first planning + one multi-family persistent launch per precision class (plan.cu).
degpu_status multi_solve(const degpu_method_cfg* cfg, const EnsArgs& a, const int32_t* family_dev, int fam_const,
                         bool dense, cudaStream_t s, bool crossing = false);

// One run-to-completion launch per (precision class, family) over the same longest-first lists;
// `crossing` launches the crossing-detection kernels (dense = 1) instead.
degpu_status sorted_thread_solve(const degpu_method_cfg* cfg, const EnsArgs& a, const int32_t* family_dev,
                                 int fam_const, bool dense, cudaStream_t s, bool crossing = false);

// Mixed-precision split of a solve (degpu_set_mixed_min_rtol): the rtol bound below which an
// instance of a DEGPU_MIXED solve runs the DEGPU_FP64_FAST variant; 0 when cfg asks for another
// precision or for RK4.
double mixed_split(const degpu_method_cfg* cfg);

// The arithmetic of the instances below the split of a mixed solve: FP32-pair stages
// (PrecMixedPair) where they are built (DOPRI5), else DEGPU_FP64_FAST.  Callers fall back to
// DEGPU_FP64_FAST when the layout they launch has no pair kernel.
int mixed_low_precision(const degpu_method_cfg* cfg);

// Argument checks shared by the ensemble entry points (degpu_abi.cu): null pointers, sizes, enum
// ranges and the problem's dimension and parameter count -> DEGPU_BAD_INPUT.
degpu_status validate_solve_args(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                                 const degpu_batch_out* out);

// Right-hand-side evaluation kernels (degpu_eval_rhs)
using RhsLaunchFn = cudaError_t (*)(int64_t n, const double* t, const double* y, const double* p, double* dydt,
                                    cudaStream_t s);
std::map<std::pair<int, int>, RhsLaunchFn>& rhs_registry();

template <class Rhs, class P>
__global__ void eval_rhs_kernel(int64_t n, const double* t, const double* y, const double* p, double* dydt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    using S = typename P::S;
    S yy[Rhs::D], dd[Rhs::D];
    double pp[Rhs::NP > 0 ? Rhs::NP : 1];
    for (int q = 0; q < Rhs::NP; ++q) pp[q] = p[(int64_t)q * n + i];
    for (int c = 0; c < Rhs::D; ++c) yy[c] = (S)y[(int64_t)c * n + i];
    Rhs::template diff<P>(t[i], yy, dd, pp);
    for (int c = 0; c < Rhs::D; ++c) dydt[(int64_t)c * n + i] = (double)dd[c];
}

template <class Rhs, class P>
cudaError_t launch_rhs(int64_t n, const double* t, const double* y, const double* p, double* dydt, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    eval_rhs_kernel<Rhs, P><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, t, y, p, dydt);
    return cudaGetLastError();
}

template <class Rhs, class P>
void register_rhs() {
    rhs_registry()[{Rhs::ID, P::ID}] = &launch_rhs<Rhs, P>;
}

}  // namespace degpu
