// mavi_peak.cu — FMA-throughput microbenchmark: the measured FP32 / FP64
// pipe peaks that the pair-force roofline is quoted against.
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mavi_cuda.h"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 2048;

// kChains independent FMA chains per thread so the pipe, not latency, limits.
template <typename T>
__global__ void fma_loop(T* out, T a, T b) {
    T x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = (T)(threadIdx.x + c);
    for (int i = 0; i < kIters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = x[c] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    if (s == (T)12345.678) out[0] = s;   // keeps the loop alive
}

template <typename T>
int run(int device, double* flops) {
    if (cudaSetDevice(device) != cudaSuccess) return MAVI_ERR_NO_DEVICE;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return MAVI_ERR_CUDA;
    const int threads = 512, blocks = sms * 8;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    fma_loop<T><<<blocks, threads>>>(out, (T)0.999999, (T)1e-7);   // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5; r++) {
        cudaEventRecord(a);
        fma_loop<T><<<blocks, threads>>>(out, (T)0.999999, (T)1e-7);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return MAVI_ERR_CUDA;
    double fl = 2.0 * kChains * (double)kIters * threads * (double)blocks;
    *flops = fl / (best * 1e-3);
    return MAVI_OK;
}

}  // namespace

extern "C" int mavi_fma_peak(int32_t precision, int32_t device, double* flops_per_s) {
    if (!flops_per_s) return MAVI_ERR_INVALID_ARG;
    return precision == MAVI_PREC_FP64 ? run<double>(device, flops_per_s) : run<float>(device, flops_per_s);
}
