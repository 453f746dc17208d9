// Measured FP64 fused multiply-add throughput of the current device.
//
// The FP64 form of the step is bound by the FP64 pipe on GB300, so its ALU
// roofline needs the pipe's rate on this part as the denominator, measured the
// same way as any other peak: a kernel of independent FMA chains (no memory
// traffic beyond one store per thread), timed with CUDA events, best of a few
// launches.  No reference counterpart: a measurement aid.
#include <cuda_runtime.h>

#include "../../include/gpe_gb300.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_dfma_chains(double* out, int iters, double a, double b) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = 1e-3 * (double)(threadIdx.x + c);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" int gpe_gb_fp64_fma_rate(double* tflops) {
    if (!tflops) return GPE_ERR_ARGUMENT;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int)e;
    const int blocks = sms * 8, iters = 2048;
    double* out = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t st = nullptr;
    e = cudaMalloc(&out, (size_t)blocks * kThreads * sizeof(double));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    float best = 0.0f;
    for (int rep = 0; rep < 6 && e == cudaSuccess; rep++) {
        cudaEventRecord(a, st);
        k_dfma_chains<<<blocks, kThreads, 0, st>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(b, st);
        e = cudaEventSynchronize(b);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (e == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms;  // first launch: warm-up
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (st) cudaStreamDestroy(st);
    if (out) cudaFree(out);
    if (e != cudaSuccess) return (int)e;
    const double flops = 2.0 * kChains * (double)iters * (double)blocks * kThreads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return 0;
}
