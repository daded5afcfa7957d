// FP32 FMA throughput probes, scalar fma.rn.f32 and packed fma.rn.f32x2: the denominator
// of the sampler's roofline is the larger of the two (the sampler is bound by the FP32
// pipe; the measured peaks at hand cover HBM copy bandwidth and BF16 tensor throughput
// only).
#include <cuda_runtime.h>

#include "device_math.cuh"
#include "host.h"

namespace rbmg {
namespace {

__global__ void fma_probe_kernel(float* out, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
    float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 123.456f) out[threadIdx.x] = s;   // keeps the chains alive, never true in practice
}

// the same chains on packed pairs: fma.rn.f32x2, two FMAs per instruction
__global__ void fma2_probe_kernel(float* out, int iters, float a, float b) {
    const float x0 = threadIdx.x * 1e-7f;
    pair_t x[8];
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = pk2(x0 + c, x0 + c + 0.5f);
    const pair_t aa = splat2(a), bb = splat2(b);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
#pragma unroll
            for (int c = 0; c < 8; c++) x[c] = fma2(x[c], aa, bb);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        float lo, hi;
        up2(x[c], lo, hi);
        s += lo + hi;
    }
    if (s == 123.456f) out[threadIdx.x] = s;
}

template <bool PAIRS>
int probe(int iters, double* tflops) {
    if (!tflops || iters <= 0) return fail(RBMG_EINVAL, "probe: bad arguments");
    int dev = 0, sms = 0;
    RBMG_CK(cudaGetDevice(&dev));
    RBMG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    float* out = nullptr;
    RBMG_CK(cudaMalloc(&out, 1024 * sizeof(float)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    auto run = [&](int n) {
        if (PAIRS) fma2_probe_kernel<<<blocks, threads, 0, stream()>>>(out, n, 0.9999f, 1e-4f);
        else fma_probe_kernel<<<blocks, threads, 0, stream()>>>(out, n, 0.9999f, 1e-4f);
    };
    run(iters / 4);   // warm-up
    cudaEventRecord(e0, stream());
    run(iters);
    cudaEventRecord(e1, stream());
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return cuda_fail(err, "probe");
    const double flops = (PAIRS ? 4.0 : 2.0) * 8 * 16 * static_cast<double>(iters) * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return RBMG_OK;
}

}  // namespace
}  // namespace rbmg

using namespace rbmg;

extern "C" int rbmg_probe_fp32_tflops(int iters, double* tflops) { return probe<false>(iters, tflops); }

extern "C" int rbmg_probe_fp32x2_tflops(int iters, double* tflops) { return probe<true>(iters, tflops); }
