// Target B-spline prefilter (reference: shaders/icgn.wgsl:145-214 and the
// taps of wgpu_backend.py:_fir_weights, 527-541).
//
// The reference runs two passes through a global scratch plane (x, then y).
// Here one CTA produces a 64 x 32 output tile: it stages the mirrored
// (32+24) x (64+24) byte footprint in shared memory (4-byte loads for
// interior tiles), runs the 25-tap x pass for all 56 footprint rows into a
// second shared tile, then the 25-tap y pass, and writes the float32
// coefficient plane once.  Every output is the
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
constexpr int kRun = 8;                      // outputs per thread along the filtered axis
constexpr int kWin = kRun + 2 * kRadius;     // 32 samples feed a run

__constant__ float c_fir[25];

// Register blocking: a thread filters a run of 8 consecutive outputs from a
// 32-sample window held in registers (8 shared-memory vector loads in x,
// 32 scalar loads down a column in y) instead of 25 shared loads per output.
__global__ void __launch_bounds__(kThreads) fir_prefilter_kernel(const uint8_t *__restrict__ img,
                                                                 int W, int H, int pitch,
                                                                 float *__restrict__ coef) {
    __shared__ __align__(16) float s_in[kInH * kInW];
    __shared__ __align__(16) float s_x[kInH * kTileW];
    const int x0 = blockIdx.x * kTileW, y0 = blockIdx.y * kTileH;
    const int tid = threadIdx.x;
    const bool interior = x0 >= kRadius && y0 >= kRadius && x0 + kTileW + kRadius <= W &&
                          y0 + kTileH + kRadius <= H && (pitch & 3) == 0 &&
                          (reinterpret_cast<uintptr_t>(img) & 3) == 0;
    if (interior) {
        // Footprint rows start at x0 - 12, a multiple of 4: 22 aligned 4-byte words per row.
        constexpr int kWords = kInW / 4;
        for (int i = tid; i < kInH * kWords; i += kThreads) {
            const int r = i / kWords, w = i - r * kWords;
            const uint32_t v = __ldg(reinterpret_cast<const uint32_t *>(img + (size_t)(y0 + r - kRadius) * pitch +
                                                                        (x0 - kRadius)) + w);
            float4 f = make_float4((float)(v & 0xffu), (float)((v >> 8) & 0xffu), (float)((v >> 16) & 0xffu),
                                   (float)(v >> 24));
            *reinterpret_cast<float4 *>(s_in + r * kInW + 4 * w) = f;
        }
    } else {
        for (int i = tid; i < kInH * kInW; i += kThreads) {
            const int r = i / kInW, c = i - r * kInW;
            const int sy = mirror_clamp(y0 + r - kRadius, H);
            const int sx = mirror_clamp(x0 + c - kRadius, W);
            s_in[i] = (float)__ldg(img + (size_t)sy * pitch + sx);
        }
    }
    __syncthreads();
    // x pass: every footprint row, 8 runs of 8 outputs.
    for (int item = tid; item < kInH * (kTileW / kRun); item += kThreads) {
        const int r = item / (kTileW / kRun), run = item - r * (kTileW / kRun);
        const float4 *src = reinterpret_cast<const float4 *>(s_in + r * kInW + run * kRun);
        float v[kWin];
#pragma unroll
        for (int q = 0; q < kWin / 4; ++q) {
            const float4 f = src[q];
            v[4 * q] = f.x; v[4 * q + 1] = f.y; v[4 * q + 2] = f.z; v[4 * q + 3] = f.w;
        }
        float acc[kRun];
#pragma unroll
        for (int j = 0; j < kRun; ++j) acc[j] = 0.0f;
#pragma unroll
        for (int k = 0; k < 25; ++k) {
            const float t = c_fir[k];
#pragma unroll
            for (int j = 0; j < kRun; ++j) acc[j] = fmaf(t, v[j + k], acc[j]);
        }
        float4 *dst = reinterpret_cast<float4 *>(s_x + r * kTileW + run * kRun);
        dst[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        dst[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
    }
    __syncthreads();
    // y pass: one column run of 8 outputs per thread (64 columns x 4 runs).
    {
        const int c = tid % kTileW, run = tid / kTileW;
        const int x = x0 + c;
        const float *src = s_x + run * kRun * kTileW + c;
        float v[kWin];
#pragma unroll
        for (int q = 0; q < kWin; ++q) v[q] = src[q * kTileW];
        float acc[kRun];
#pragma unroll
        for (int j = 0; j < kRun; ++j) acc[j] = 0.0f;
#pragma unroll
        for (int k = 0; k < 25; ++k) {
            const float t = c_fir[k];
#pragma unroll
            for (int j = 0; j < kRun; ++j) acc[j] = fmaf(t, v[j + k], acc[j]);
        }
        if (x < W) {
#pragma unroll
            for (int j = 0; j < kRun; ++j) {
                const int y = y0 + run * kRun + j;
                if (y < H) coef[(size_t)y * W + x] = acc[j];
            }
        }
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
