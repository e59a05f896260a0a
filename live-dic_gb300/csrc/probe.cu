// FP32 pipe throughput probe: the denominator of the IC-GN roofline.
//
// Every thread runs eight independent fused multiply-add chains, so the
// measurement is bound by the FP32 pipes rather than by dependency latency;
// the grid fills every SM with eight 256-thread CTAs.  The chains' sum is
// stored so that nothing is optimised away.
#include <cuda_runtime.h>

#include "../../include/gbdic.h"

namespace {

__global__ void __launch_bounds__(256) fma_probe_kernel(float seed, int rounds, float *out) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.0f, a2 = a0 + 2.0f, a3 = a0 + 3.0f;
    float a4 = a0 + 4.0f, a5 = a0 + 5.0f, a6 = a0 + 6.0f, a7 = a0 + 7.0f;
    const float m = 0.9999999f, c = 1e-7f;
#pragma unroll 1
    for (int r = 0; r < rounds; ++r) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
}

}  // namespace

extern "C" int gbdic_fp32_peak_probe(int32_t device, double *tflops) {
    if (!tflops) return GBDIC_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return GBDIC_ECUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return GBDIC_ECUDA;
    const int blocks = sms * 8, threads = 256, rounds = 4096;
    float *out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)) != cudaSuccess) return GBDIC_ECUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_probe_kernel<<<blocks, threads>>>(1.0f, rounds / 8, out);  // warm-up
    double best = 0.0;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0);
        fma_probe_kernel<<<blocks, threads>>>(1.0f, rounds, out);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 8.0 * 16.0 * rounds * (double)blocks * threads;
        if (ms > 0.0f) best = flops / (ms * 1e-3) / 1e12 > best ? flops / (ms * 1e-3) / 1e12 : best;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return GBDIC_ECUDA;
    *tflops = best;
    return GBDIC_OK;
}
