// Shared device helpers and kernel argument blocks for the gbdic library.
//
// Rounding contract: the bit-exact units are compiled with --fmad=false, so a*b+c is
// only fused where the source writes fmaf(); every other float operation is
// one IEEE binary32 operation rounded to nearest (no fast-math, IEEE
// division and square root).  The arithmetic order of each kernel is fixed
// in its comments so that results are reproducible bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gbdic {

constexpr int kModelAffine = 0;
constexpr int kModelTranslation = 1;
constexpr int kModelQuadratic = 2;
constexpr int kInterpBspline = 0;
constexpr int kInterpLinear = 1;
constexpr int kInterpKeys = 2;
constexpr unsigned kFullMask = 0xffffffffu;

__host__ __device__ constexpr int parameter_count(int model) { return model == kModelQuadratic ? 12 : 6; }
__host__ __device__ constexpr int state_stride(int model) { return model == kModelQuadratic ? 16 : 8; }
__host__ __device__ constexpr int meta_stride(int model) { return model == kModelQuadratic ? 28 : 16; }
__host__ __device__ constexpr int status_slot(int model) { return model == kModelQuadratic ? 12 : 6; }

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// One reflection without edge repetition, then clamp (icgn.wgsl:128-143).
__device__ __forceinline__ int mirror_clamp(int c, int n) {
    int r = c < 0 ? -c : (c >= n ? 2 * n - 2 - c : c);
    return clampi(r, 0, n - 1);
}

// Uniform cubic B-spline weights, Horner forms, 1/6 as a binary32 product.
__device__ __forceinline__ void bspline_weights(float t, float w[4]) {
    const float k6 = 1.0f / 6.0f;
    float t2 = t * t, t3 = t2 * t, s = 1.0f - t;
    w[0] = ((s * s) * s) * k6;
    w[1] = fmaf(fmaf(3.0f, t, -6.0f), t2, 4.0f) * k6;
    w[2] = fmaf(fmaf(fmaf(-3.0f, t, 3.0f), t, 3.0f), t, 1.0f) * k6;
    w[3] = t3 * k6;
}

// Keys cubic convolution weights (a = -0.5).
__device__ __forceinline__ void keys_weights(float t, float w[4]) {
    float t2 = t * t;
    w[0] = fmaf(fmaf(-0.5f, t, 1.0f), t, -0.5f) * t;
    w[1] = fmaf(fmaf(1.5f, t, -2.5f), t2, 1.0f);
    w[2] = fmaf(fmaf(-1.5f, t, 2.0f), t, 0.5f) * t;
    w[3] = fmaf(0.5f, t, -0.5f) * t2;
}

// a*(1-t) + b*t with the last product fused.
__device__ __forceinline__ float mixf(float a, float b, float t) { return fmaf(b, t, a * (1.0f - t)); }

// Target sample at (px, py).  CLAMP keeps every tap inside the plane; the
// affine and translation solvers omit it because their bounds check already
// guarantees a one-pixel margin around every 4x4 footprint.
template <int INTERP, bool CLAMP>
__device__ __forceinline__ float sample_target(const float *__restrict__ coef,
                                               const uint8_t *__restrict__ img, int W, int H,
                                               float px, float py) {
    float fx = floorf(px), fy = floorf(py);
    int bx = (int)fx, by = (int)fy;
    float tx = px - fx, ty = py - fy;
    if (INTERP == kInterpLinear) {
        int x0 = bx, x1 = bx + 1, y0 = by, y1 = by + 1;
        if (CLAMP) {
            x0 = clampi(x0, 0, W - 1); x1 = clampi(x1, 0, W - 1);
            y0 = clampi(y0, 0, H - 1); y1 = clampi(y1, 0, H - 1);
        }
        float a = __ldg(img + (size_t)y0 * W + x0), b = __ldg(img + (size_t)y0 * W + x1);
        float c = __ldg(img + (size_t)y1 * W + x0), d = __ldg(img + (size_t)y1 * W + x1);
        return mixf(mixf(a, b, tx), mixf(c, d, tx), ty);
    }
    float wx[4], wy[4];
    if (INTERP == kInterpKeys) {
        keys_weights(tx, wx);
        keys_weights(ty, wy);
    } else {
        bspline_weights(tx, wx);
        bspline_weights(ty, wy);
    }
    int xs[4], ys[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        xs[i] = CLAMP ? clampi(bx + i - 1, 0, W - 1) : bx + i - 1;
        ys[i] = CLAMP ? clampi(by + i - 1, 0, H - 1) : by + i - 1;
    }
    float value = 0.0f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float row = 0.0f;
        if (INTERP == kInterpKeys) {
            const uint8_t *r = img + (size_t)ys[j] * W;
#pragma unroll
            for (int i = 0; i < 4; ++i) row = fmaf(wx[i], (float)__ldg(r + xs[i]), row);
        } else {
            const float *r = coef + (size_t)ys[j] * W;
#pragma unroll
            for (int i = 0; i < 4; ++i) row = fmaf(wx[i], __ldg(r + xs[i]), row);
        }
        value = fmaf(wy[j], row, value);
    }
    return value;
}

struct Warp {
    float t0, t1;           // tx, ty
    float l0, l1, l2, l3;   // ux, uy, vx, vy
    float c0, c1, c2, c3, c4, c5;  // uxx, uxy, uyy, vxx, vxy, vyy
};

// Displacement at local (lx, ly); hx2 = lx^2/2, xy = lx*ly, hy2 = ly^2/2.
template <int MODEL>
__device__ __forceinline__ void displacement(const Warp &w, float lx, float ly, float hx2,
                                             float xy, float hy2, float &dx, float &dy) {
    if (MODEL == kModelTranslation) {
        dx = w.t0;
        dy = w.t1;
        return;
    }
    float ax = w.t0 + fmaf(w.l0, lx, w.l1 * ly);
    float ay = w.t1 + fmaf(w.l2, lx, w.l3 * ly);
    if (MODEL == kModelQuadratic) {
        ax = ax + fmaf(w.c0, hx2, fmaf(w.c1, xy, w.c2 * hy2));
        ay = ay + fmaf(w.c3, hx2, fmaf(w.c4, xy, w.c5 * hy2));
    }
    dx = ax;
    dy = ay;
}

__device__ __forceinline__ float length2(float a, float b) { return sqrtf(fmaf(a, a, b * b)); }

// Arguments of one IC-GN launch over one level.
struct SolveArgs {
    const float *coef;         // B-spline coefficient plane (bspline mode)
    const uint8_t *img;        // target bytes (direct modes)
    const float4 *plane;       // reference plane [f, gx, gy, 0]
    const float *meta;         // metadata rows
    const float *inv;          // inverse Hessians
    const float *weights;      // S*S integration weights (Gaussian mode)
    const float *seed;         // seed states or nullptr (zero seed)
    const uint32_t *active;    // per-subset activity (seeded entries)
    float *state;              // output states
    unsigned *work_counter;    // persistent launch queue head
    int W, H, grid_w, count, S, stride;
    int iterations;
    float tolerance, zncc_min, weight_sum;
    int roi_enabled, preserve_disabled, use_mean;
    int div_patience, div_min;
    int persistent;
    unsigned long long *iteration_total;  // profiling: sum of executed iterations, or nullptr
    // Partial-support windows (partial solver only): group g solves window
    // partial_index[g] over the pixels set in its support words, bounded by
    // its support box (x0, y0, x1, y1); count = number of partial windows.
    const int *partial_index;
    const uint32_t *support;
    const float4 *support_box;
    int support_words;
    // Fast pixel loop (solver_fast.cu): row segments per column, or 0 for the
    // exact loop.
    int fast_segments;
    // Staged tiles (solver_staged.cu): 0 off, 1 compact (56 x 44 floats per
    // warp), 2 wide (72 x 56).
    int staged_tile;
    // List mode (exact loop, complete windows): group g solves subset
    // subset_list[g] for g < count, or g < min(count, *list_count) when
    // list_count is set (a device count written by an earlier kernel).
    const int *subset_list;
    const unsigned *list_count;
};

}  // namespace gbdic
