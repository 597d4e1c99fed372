// bhk_diag.cu -- measured FP32 FMA peak of the device, the roofline denominator of the tracer.
//
// Every thread runs 8 independent FMA chains (enough to cover the FMA latency at full occupancy);
// the result is stored so the chains are not optimised away. FLOPs = threads x iterations x 8 x 2.
#include <cuda_runtime.h>

#include "../../include/bhk.h"

namespace {

constexpr int kChains = 8;

__global__ void fma_peak_kernel(float* sink, int iters, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-3f + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 1234.5678f) sink[blockIdx.x] = s;  // practically never taken; keeps the chains live
}

}  // namespace

extern "C" bhk_status bhk_fp32_fma_peak(int device, double* tflops) {
    if (!tflops) return BHK_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return BHK_ECUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int block = 256, per_sm = 8, iters = 1 << 16;
    const int grid = sms * per_sm;
    float* sink = nullptr;
    if (cudaMalloc(&sink, sizeof(float) * grid) != cudaSuccess) return BHK_ENOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        fma_peak_kernel<<<grid, block>>>(sink, iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess) return BHK_ECUDA;
    const double flops = 2.0 * kChains * double(iters) * double(grid) * block;
    *tflops = flops / (best * 1e-3) / 1e12;
    return BHK_OK;
}
