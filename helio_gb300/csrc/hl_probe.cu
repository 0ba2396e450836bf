// hl_probe.cu — FP32 FMA-throughput probe: the measured denominator of the FP32
// roofline. Every thread runs 8 independent FFMA chains; one FFMA is 2 FLOPs.
#include "hl_common.cuh"
#include "hl_internal.h"

namespace hl {
namespace {

constexpr int kProbeChains = 8;

__global__ void __launch_bounds__(256) fp32_probe_kernel(float seed, int iters, float* __restrict__ sink) {
    float a[kProbeChains];
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) a[c] = seed + float(threadIdx.x + c);
    const float m = 0.999999f, b = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kProbeChains; ++c) a[c] = __fmaf_rn(a[c], m, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) s += a[c];
    if (s == 1234.5678f) sink[threadIdx.x] = s;  // never true; keeps the chains live
}

}  // namespace

cudaError_t run_fp32_probe(int device, double* tflops) {
    int sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    float* sink = nullptr;
    if ((e = cudaMalloc(&sink, 256 * sizeof(float))) != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    fp32_probe_kernel<<<blocks, threads>>>(1.0f, 256, sink);  // warm-up
    double best = 0.0;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(a);
        fp32_probe_kernel<<<blocks, threads>>>(1.0f, iters, sink);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        const double flops = 2.0 * kProbeChains * double(iters) * blocks * threads;
        if (ms > 0.0f) best = fmax(best, flops / (double(ms) * 1e-3) / 1e12);
    }
    e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    *tflops = best;
    return e;
}

}  // namespace hl
