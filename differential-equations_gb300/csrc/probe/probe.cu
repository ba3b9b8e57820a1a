// probe.cu — libdegpu_probe.so: measurement and device self-checks, kept out of the integrator
// library.  Not part of the public ABI.
//  - degpu_internal_fma_peak: FP64 / FP32 FMA throughput, the roofline denominator of the
//    ALU-bound ensemble kernels.  Each thread runs 8 independent FMA chains; the grid covers every
//    SM several times over.
//  - degpu_internal_conv_check: the mixed form's integer-op conversions on the device.
//  - degpu_internal_pow_ctrl_neg_check: the plain FP64 form's controller power on the device,
//    compiled as the plain form is (FMA contraction on, CUDA's FP32 log2f/exp2f in its start).
#include <cuda_runtime.h>
#include <stdint.h>

#include "erk_core.cuh"

template <class T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = (T)(threadIdx.x + j);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
    }
    T s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    if (s == (T)12345.678) out[0] = s;  // keeps the chains alive
}

extern "C" int degpu_internal_fma_peak(int fp64, double* tflops) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* out = nullptr;
    if (cudaMalloc(&out, 16) != cudaSuccess) return 1;
    const int threads = 256, blocks = sms * 8;
    const int iters = fp64 ? 4096 : 65536;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (fp64)
            fma_probe_kernel<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7);
        else
            fma_probe_kernel<float><<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// wide[i] = widen_f32(f[i]), narrow[i] = narrow_rz(d[i]) (erk_core.cuh).  Device pointers.
__global__ void conv_check_kernel(int64_t n, const float* f, double* wide, const double* d, float* narrow) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    wide[i] = degpu::widen_f32(f[i]);
    narrow[i] = degpu::narrow_rz(d[i]);
}

extern "C" int degpu_internal_conv_check(int64_t n, const float* f, double* wide, const double* d, float* narrow) {
    if (n <= 0) return 0;
    conv_check_kernel<<<(unsigned)((n + 255) / 256), 256>>>(n, f, wide, d, narrow);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

// out[i] = x[i]^y through the plain form's controller power (PrecPlain::pow).  Device pointers.
__global__ void pow_check_kernel(int64_t n, const double* x, double y, double* out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = degpu::PrecPlain::pow(x[i], y);
}

extern "C" int degpu_internal_pow_ctrl_neg_check(int64_t n, const double* x, double y, double* out) {
    if (n <= 0) return 0;
    pow_check_kernel<<<(unsigned)((n + 255) / 256), 256>>>(n, x, y, out);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}
