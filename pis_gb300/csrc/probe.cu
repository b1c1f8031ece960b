// probe.cu - measurement hook: the arithmetic peak of this GPU's FP32 and FP64 pipes.
//
// The roofline of the force kernels needs the FP32 (mixed path) and FP64 (plain path) pipe rates,
// which the copy / GEMM peaks measured elsewhere do not give. Every thread runs eight independent
// fused multiply-add chains (enough in flight to cover the pipe latency at full occupancy); the
// grid fills every SM with 2048 threads. No counterpart in the reference.
#include <cuda_runtime.h>

#include <algorithm>

#include "pis_gpu.h"

namespace {

constexpr int CHAINS = 8;

template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(T* out, int iters, T a, T b) {
    T x[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = (T)(threadIdx.x + c);
    for (int k = 0; k < iters; ++k)
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) x[c] = fma(x[c], a, b);
    T s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += x[c];
    if (s == (T)-1.0) out[blockIdx.x] = s;  // never true: keeps the chains from being removed
}

template <typename T>
cudaError_t time_probe(int iters, double* tflops) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = sms * 8, threads = 256;
    T* out = nullptr;
    if ((e = cudaMalloc(&out, sizeof(T) * blocks)) != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {  // the first launch is a warm-up
        cudaEventRecord(a);
        k_fma_probe<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-6);
        cudaEventRecord(b);
        e = cudaEventSynchronize(b);
        if (e != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0) best = std::min(best, ms);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return e;
    const double flops = 2.0 * CHAINS * (double)iters * blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return cudaSuccess;
}

}  // namespace

extern "C" pis_status pis_gpu_probe_peaks(double* fp32_tflops, double* fp64_tflops) {
    if (!fp32_tflops || !fp64_tflops) return PIS_ERR_INVALID_ARGUMENT;
    if (time_probe<float>(1 << 14, fp32_tflops) != cudaSuccess) return PIS_ERR_CUDA;
    if (time_probe<double>(1 << 10, fp64_tflops) != cudaSuccess) return PIS_ERR_CUDA;
    return PIS_OK;
}
