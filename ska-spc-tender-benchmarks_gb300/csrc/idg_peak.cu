// idg_peak.cu -- FP32 FMA throughput of the current device, measured.
//
// The gridder and degridder are FP32-pipe bound; their roofline denominator is
// the device's achievable FFMA rate, which this measures with 8 independent
// dependent chains per thread on every SM (2 flop per FMA).
#include <cuda_runtime.h>

#include "idg_internal.h"

namespace idg {

namespace {
__global__ void ffma_peak_kernel(float *out, int iters, float a, float b) {
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            x0 = fmaf(x0, a, b);
            x1 = fmaf(x1, a, b);
            x2 = fmaf(x2, a, b);
            x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b);
            x5 = fmaf(x5, a, b);
            x6 = fmaf(x6, a, b);
            x7 = fmaf(x7, a, b);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
} // namespace

cudaError_t measure_fp32_peak(double *flops) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int threads = 256, blocks = sms * 8, iters = 4000;
    float *out = nullptr;
    e = cudaMalloc(&out, sizeof(float) * threads * blocks);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    ffma_peak_kernel<<<blocks, threads>>>(out, 50, 1.0001f, 0.5f); // warm-up, clocks up
    double best = 0;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(a);
        ffma_peak_kernel<<<blocks, threads>>>(out, iters, 1.0001f, 0.5f);
        cudaEventRecord(b);
        e = cudaEventSynchronize(b);
        if (e != cudaSuccess) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        const double f = 2.0 * threads * (double)blocks * iters * 16 * 8 / (ms * 1e-3);
        if (f > best) best = f;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e == cudaSuccess) e = cudaGetLastError();
    *flops = best;
    return e;
}

} // namespace idg
