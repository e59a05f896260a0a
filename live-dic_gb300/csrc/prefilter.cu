// Target B-spline prefilter (reference: shaders/icgn.wgsl:145-214 and the
// taps of wgpu_backend.py:_fir_weights, 527-541).
//
// The reference runs two passes through a global scratch plane (x, then y).
// Here one CTA produces a 64 x 32 output tile: it stages the mirrored
// (32+24) x (64+24) byte footprint in shared memory, runs the 25-tap x pass
// for all 56 footprint rows into a second shared tile, then the 25-tap y
// pass, and writes the float32 coefficient plane once.  Every output is the
// same sequence of fmaf(tap, sample, acc) over taps -12..12 as the two-pass
// form, so the result is bit-identical to it; HBM sees 1 B read + 4 B
// written per pixel instead of 1 + 4 + 4 + 4 + 4.
#include "gbdic_common.cuh"
#include "gbdic_kernels.h"

namespace gbdic {

namespace {
constexpr int kTileW = 64;
constexpr int kTileH = 32;
constexpr int kRadius = 12;
constexpr int kInW = kTileW + 2 * kRadius;   // 88
constexpr int kInH = kTileH + 2 * kRadius;   // 56
constexpr int kThreads = 256;

__constant__ float c_fir[25];

__global__ void __launch_bounds__(kThreads) fir_prefilter_kernel(const uint8_t *__restrict__ img,
                                                                 int W, int H, int pitch,
                                                                 float *__restrict__ coef) {
    __shared__ float s_in[kInH * kInW];
    __shared__ float s_x[kInH * kTileW];
    const int x0 = blockIdx.x * kTileW, y0 = blockIdx.y * kTileH;
    const int tid = threadIdx.x;
    for (int i = tid; i < kInH * kInW; i += kThreads) {
        const int r = i / kInW, c = i - r * kInW;
        const int sy = mirror_clamp(y0 + r - kRadius, H);
        const int sx = mirror_clamp(x0 + c - kRadius, W);
        s_in[i] = (float)__ldg(img + (size_t)sy * pitch + sx);
    }
    __syncthreads();
    for (int i = tid; i < kInH * kTileW; i += kThreads) {
        const int r = i / kTileW, c = i - r * kTileW;
        const float *src = s_in + r * kInW + c;
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 25; ++k) acc = fmaf(c_fir[k], src[k], acc);
        s_x[i] = acc;
    }
    __syncthreads();
    for (int i = tid; i < kTileH * kTileW; i += kThreads) {
        const int r = i / kTileW, c = i - r * kTileW;
        const int x = x0 + c, y = y0 + r;
        if (x >= W || y >= H) continue;
        const float *src = s_x + r * kTileW + c;
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 25; ++k) acc = fmaf(c_fir[k], src[k * kTileW], acc);
        coef[(size_t)y * W + x] = acc;
    }
}
}  // namespace

cudaError_t set_fir_taps(const float *taps25) {
    return cudaMemcpyToSymbol(c_fir, taps25, 25 * sizeof(float));
}

cudaError_t launch_fir_prefilter(const uint8_t *img, int W, int H, int pitch, float *coef,
                                 cudaStream_t stream) {
    dim3 grid((W + kTileW - 1) / kTileW, (H + kTileH - 1) / kTileH);
    fir_prefilter_kernel<<<grid, kThreads, 0, stream>>>(img, W, H, pitch, coef);
    return cudaGetLastError();
}

}  // namespace gbdic
