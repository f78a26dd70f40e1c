// probe.cu — throughput probes of the FP64 pipe, the roofline denominator of this path.
// The measured peaks cover HBM copy bandwidth and bf16 tensor throughput only; the
// kernels here are bound by FP64 arithmetic, so its peak is measured the same way, live.
#include <cuda_runtime.h>

#include <string>

#include "internal.h"

namespace {

// 8 independent FMA chains per thread; values stay bounded (|b| < 1).
__global__ void k_dfma(double* out, int iters, double b, double c) {
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = 1e-3 * (threadIdx.x + k);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 1234.5678) out[0] = s;  // keeps the chains alive
}

// 4 independent chains of IEEE divides (the compiler's correctly rounded division).
__global__ void k_ddiv(double* out, int iters, double b, double c) {
    double a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = 1.5 + 1e-3 * (threadIdx.x + k);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 4; ++k) a[k] = b / a[k] + c;
    }
    double s = a[0] + a[1] + a[2] + a[3];
    if (s == 1234.5678) out[0] = s;
}

}  // namespace

extern "C" int dense_measure_fp64(int kind, double* result) {
    if (!result) return DENSE_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return DENSE_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DENSE_ERR_CUDA;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return DENSE_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = sms * 8;
    const int iters = kind == 0 ? 4096 : 512;
    auto launch = [&](int n) {
        if (kind == 0) k_dfma<<<blocks, threads>>>(out, n, 0.9999999, 1e-7);
        else k_ddiv<<<blocks, threads>>>(out, n, 0.75, 0.5);
    };
    launch(iters / 8);  // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(e0);
        launch(iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return DENSE_ERR_CUDA;
    const double nthreads = (double)threads * blocks;
    if (kind == 0) *result = 2.0 * 8.0 * iters * nthreads / (best * 1e-3);  // FLOP/s
    else *result = 4.0 * iters * nthreads / (best * 1e-3);                   // divides/s
    return DENSE_OK;
}
