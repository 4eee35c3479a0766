// mdt_peak.cu -- FP64 / FP32 fused-multiply-add throughput microbenchmark, and a read-out of
// the thermostats' deviate streams for statistical checks.
//
// The EMT force kernels are bound by CUDA-core arithmetic, not by HBM or tensor cores,
// so their roofline denominator is the GPU's measured FMA rate: every thread keeps 8
// independent FMA chains in registers for `iters` iterations, the grid covers every SM
// several times over, and CUDA events time the launch.
#include <cuda_runtime.h>

#include "../../include/mdt_gpu.h"
#include "mdt_common.cuh"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_chains(T *out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == (T)-12345.0) out[blockIdx.x] = s;  // keeps the chains alive
}

template <typename T> double run(int iters) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = sms * 8, block = 256;
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * grid) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T><<<grid, block>>>(out, iters / 8 + 1, (T)0.999999, (T)1e-7);  // warm-up
    cudaEventRecord(e0);
    fma_chains<T><<<grid, block>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return -1.0;
    const double flops = 2.0 * 8 * 16 * (double)iters * grid * block;
    return flops / (ms * 1e-3);
}

// out[i] = the deviate the propagators draw at (seed, traj, step, slot i, stream)
__global__ void deviates_kernel(double *out, int64_t n, int32_t kind, uint64_t seed, uint32_t traj,
                                uint32_t step, uint32_t stream) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = kind == 0 ? mdt::normal_deviate(seed, traj, step, (uint32_t)i, stream)
                           : mdt::uniform_deviate(seed, traj, step, (uint32_t)i, stream);
}

}  // namespace

extern "C" int32_t mdt_rng_deviates(int32_t kind, uint64_t seed, int32_t traj, int32_t step, int32_t stream,
                                    int64_t n, double *out) {
    if (!out || n < 0 || n > ((int64_t)1 << 32) || (kind != 0 && kind != 1) || traj < 0 || step < 0 ||
        stream < 1 || stream > 5)
        return MDT_ERR_ARG;
    if (n == 0) return MDT_OK;
    double *d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * n) != cudaSuccess) return MDT_ERR_NOMEM;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n + 255) / 256;
    const int grid = (int)(want < (int64_t)sms * 16 ? want : (int64_t)sms * 16);
    deviates_kernel<<<grid, 256>>>(d, n, kind, seed, (uint32_t)traj, (uint32_t)step, (uint32_t)stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, d, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? MDT_OK : MDT_ERR_CUDA;
}

extern "C" int32_t mdt_peak_fma(int32_t precision, int32_t iters, double *flops_per_s) {
    if (!flops_per_s || iters < 1) return MDT_ERR_ARG;
    const double v = precision == MDT_PREC_FP32 ? run<float>(iters) : run<double>(iters);
    if (v <= 0) return MDT_ERR_CUDA;
    *flops_per_s = v;
    return MDT_OK;
}
