// IC-GN subset solver (reference: shaders/icgn.wgsl:595-1017).
//
// One group of LANES threads solves one subset.  Pixel p of the S x S subset
// belongs to lane p % LANES; each lane accumulates its pixels in increasing p
// order, and the lane partial sums are combined by the pairwise tree of
// icgn.wgsl:782-799 (stride LANES/2 .. 1, lane i += lane i + stride).  For
// LANES <= 32 the tree is a __shfl_down ladder inside a warp; for 64 and 128
// the strides >= 32 go through shared memory first.  After the reduction the
// totals are broadcast and every lane evaluates the same Gauss-Newton update
// (identical operands, identical results), so the warp state never leaves
// registers.
//
// Work distribution: a "unit" is a warp (LANES <= 32) or a 128-thread block
// (LANES > 32) holding 128/LANES or 32/LANES groups.  Grid mode maps units to
// the launch grid; persistent mode keeps one resident grid and lets every
// unit pull the next batch of subsets from an atomic queue head, so subsets
// with long iteration counts do not hold up a statically assigned tile.
#pragma once

#include "gbdic_common.cuh"

// Resident CTAs per SM the translation / affine solver is compiled for
// (register budget 65536 / (128 x this)); the quadratic solver uses 5.
#ifndef GBDIC_SOLVER_MIN_BLOCKS
#define GBDIC_SOLVER_MIN_BLOCKS 5
#endif
// Packed-pair pixel loop (FADD2 / FMUL2 / FFMA2) for B-spline windows.
#ifndef GBDIC_QUAD_MIN_BLOCKS
#define GBDIC_QUAD_MIN_BLOCKS 5
#endif
#ifndef GBDIC_QUAD_PAIRS
#define GBDIC_QUAD_PAIRS 1
#endif
#ifndef GBDIC_SOLVER_PAIRS
#define GBDIC_SOLVER_PAIRS 1
#endif

namespace gbdic {

template <int MODEL>
struct SumCount {
    static constexpr int value = MODEL == kModelQuadratic ? 15 : (MODEL == kModelTranslation ? 5 : 9);
};

// Tree reduction inside a warp segment of LANES lanes, then broadcast of the
// segment's lane-0 totals to the whole segment.
template <int LANES, int N>
__device__ __forceinline__ void reduce_warp(float (&s)[N], int lane_in_warp) {
#pragma unroll
    for (int off = LANES / 2; off >= 1; off >>= 1) {
#pragma unroll
        for (int k = 0; k < N; ++k) s[k] = s[k] + __shfl_down_sync(kFullMask, s[k], off, LANES);
    }
    const int src = lane_in_warp & ~(LANES - 1);
#pragma unroll
    for (int k = 0; k < N; ++k) s[k] = __shfl_sync(kFullMask, s[k], src);
}

// Same tree for 64 or 128 lanes: shared-memory strides down to 32, then the
// shuffle ladder in the group's first warp; totals broadcast through `red`.
template <int LANES, int N>
__device__ __forceinline__ void reduce_block(float (&s)[N], float *red, int glane) {
#pragma unroll
    for (int k = 0; k < N; ++k) red[k * LANES + glane] = s[k];
    __syncthreads();
#pragma unroll
    for (int stride = LANES / 2; stride >= 32; stride >>= 1) {
        if (glane < stride) {
#pragma unroll
            for (int k = 0; k < N; ++k)
                red[k * LANES + glane] = red[k * LANES + glane] + red[k * LANES + glane + stride];
        }
        __syncthreads();
    }
    if (glane < 32) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            float v = red[k * LANES + glane];
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_down_sync(kFullMask, v, off);
            if (glane == 0) red[k * LANES] = v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) s[k] = red[k * LANES];
    __syncthreads();
}

// Bounds check of icgn.wgsl:647-690: the warped corner (affine) or 3x3
// control points (quadratic) must lie in [2, W-3] x [2, H-3].
template <int MODEL>
__device__ __forceinline__ bool warp_inside(const Warp &w, int px0, int py0, int S, float half,
                                            int W, int H) {
    const float xmax = (float)W - 3.0f, ymax = (float)H - 3.0f;
    if (MODEL == kModelTranslation) {
        float x0 = (float)px0 + w.t0, y0 = (float)py0 + w.t1;
        float x1 = (float)(px0 + S - 1) + w.t0, y1 = (float)(py0 + S - 1) + w.t1;
        return x0 >= 2.0f && y0 >= 2.0f && x1 <= xmax && y1 <= ymax;
    }
    bool inside = true;
    constexpr int count = MODEL == kModelQuadratic ? 9 : 4;
#pragma unroll
    for (int p = 0; p < count; ++p) {
        float lx, ly;
        if (MODEL == kModelQuadratic) {
            lx = (float)(p % 3 - 1) * half;
            ly = (float)(p / 3 - 1) * half;
        } else {
            lx = (p == 1 || p == 3) ? half : -half;
            ly = (p >= 2) ? half : -half;
        }
        float dx, dy;
        displacement<MODEL>(w, lx, ly, 0.5f * lx * lx, lx * ly, 0.5f * ly * ly, dx, dy);
        float px = ((float)px0 + (half + lx)) + dx;
        float py = ((float)py0 + (half + ly)) + dy;
        inside = inside && px >= 2.0f && py >= 2.0f && px <= xmax && py <= ymax;
    }
    return inside;
}

// Partial-support variant of warp_inside (icgn.wgsl:635-690 with
// PARTIAL_SUPPORT): the support box's corners instead of the window's.
template <int MODEL>
__device__ __forceinline__ bool warp_inside_box(const Warp &w, int px0, int py0, float half, float4 box, int W,
                                                int H) {
    const float xmax = (float)W - 3.0f, ymax = (float)H - 3.0f;
    if (MODEL == kModelTranslation) {
        const float x0 = ((float)px0 + box.x) + w.t0, y0 = ((float)py0 + box.y) + w.t1;
        const float x1 = ((float)px0 + box.z) + w.t0, y1 = ((float)py0 + box.w) + w.t1;
        return x0 >= 2.0f && y0 >= 2.0f && x1 <= xmax && y1 <= ymax;
    }
    const float lx0 = box.x - half, ly0 = box.y - half, lx1 = box.z - half, ly1 = box.w - half;
    bool inside = true;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        const float lx = (p == 1 || p == 3) ? lx1 : lx0;
        const float ly = (p >= 2) ? ly1 : ly0;
        float dx, dy;
        displacement<MODEL>(w, lx, ly, 0.5f * lx * lx, lx * ly, 0.5f * ly * ly, dx, dy);
        const float px = ((float)px0 + (half + lx)) + dx;
        const float py = ((float)py0 + (half + ly)) + dy;
        inside = inside && px >= 2.0f && py >= 2.0f && px <= xmax && py <= ymax;
    }
    return inside;
}

// Quadratic inverse composition (icgn.wgsl:393-513): lifted 6x6 warp matrix
// of the increment, pivoted Gauss-Jordan in binary32 on the augmented 6x12
// matrix [M | I].  The matrix is spread over a 16-lane segment of the warp,
// lane e (< 12) holding column e, so no lane keeps more than six of its
// entries: the pivot column is broadcast by shuffles, every lane applies
// the row swap, the pivot-row division and the eliminations
// m[r][e] = fma(-m[r][col], m[col][e], m[r][e]) to its own column.  Each
// entry sees exactly the operations of the row-by-row elimination, so the
// result is bitwise that of a single-thread elimination.  `sl` is the lane
// index within the segment; `mask` names the lanes executing the call.
__device__ __forceinline__ bool compose_quadratic(Warp &w, const float (&d)[12], int sl, unsigned mask) {
    const float u = d[0], ux = d[1], uy = d[2], v = d[3], vx = d[4], vy = d[5];
    const float uxx = d[6], uxy = d[7], uyy = d[8], vxx = d[9], vxy = d[10], vyy = d[11];
    float L[6][6];
    L[0][0] = fmaf(u, uxx, fmaf(ux, ux, 1.0f + 2.0f * ux));
    L[0][1] = fmaf(2.0f * (1.0f + ux), uy, 2.0f * u * uxy);
    L[0][2] = fmaf(u, uyy, uy * uy);
    L[0][3] = 2.0f * u * (1.0f + ux);
    L[0][4] = 2.0f * u * uy;
    L[0][5] = u * u;
    L[1][0] = 0.5f * fmaf(u, vxx, fmaf(2.0f * (1.0f + ux), vx, v * uxx));
    L[1][1] = (fmaf(u, vxy, fmaf(v, uxy, fmaf(ux, vy, fmaf(uy, vx, 1.0f)))) + vy) + ux;
    L[1][2] = 0.5f * fmaf(u, vyy, fmaf(2.0f * uy, 1.0f + vy, v * uyy));
    L[1][3] = fmaf(u, vx, fmaf(v, ux, v));
    L[1][4] = fmaf(u, vy, fmaf(v, uy, u));
    L[1][5] = u * v;
    L[2][0] = fmaf(v, vxx, vx * vx);
    L[2][1] = fmaf(2.0f * vx, 1.0f + vy, 2.0f * v * vxy);
    L[2][2] = fmaf(v, vyy, fmaf(vy, vy, 1.0f + 2.0f * vy));
    L[2][3] = 2.0f * v * vx;
    L[2][4] = 2.0f * v * (1.0f + vy);
    L[2][5] = v * v;
    L[3][0] = 0.5f * uxx; L[3][1] = uxy; L[3][2] = 0.5f * uyy;
    L[3][3] = 1.0f + ux;  L[3][4] = uy;  L[3][5] = u;
    L[4][0] = 0.5f * vxx; L[4][1] = vxy; L[4][2] = 0.5f * vyy;
    L[4][3] = vx;         L[4][4] = 1.0f + vy; L[4][5] = v;
    L[5][0] = 0.0f; L[5][1] = 0.0f; L[5][2] = 0.0f; L[5][3] = 0.0f; L[5][4] = 0.0f; L[5][5] = 1.0f;
    const int e = sl < 12 ? sl : 11;  // lanes 12-15 shadow column 11
    float c[6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        float x = (e - 6 == r) ? 1.0f : 0.0f;
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (e == k) x = L[r][k];
        c[r] = x;
    }
#pragma unroll
    for (int col = 0; col < 6; ++col) {
        float pc[6];  // pivot column before the swap
#pragma unroll
        for (int r = 0; r < 6; ++r) pc[r] = __shfl_sync(mask, c[r], col, 16);
        int prow = col;
        float psize = fabsf(pc[col]);
#pragma unroll
        for (int cand = col + 1; cand < 6; ++cand) {
            const float cs = fabsf(pc[cand]);
            if (cs > psize) { prow = cand; psize = cs; }
        }
        if (psize < 1e-8f) return false;
        float pivot = pc[col];
#pragma unroll
        for (int cand = col + 1; cand < 6; ++cand) {
            if (cand == prow) {
                const float t = c[col];
                c[col] = c[cand];
                c[cand] = t;
                const float tp = pc[col];
                pc[col] = pc[cand];
                pc[cand] = tp;
                pivot = pc[col];
            }
        }
        c[col] = c[col] / pivot;
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            if (r == col) continue;
            c[r] = fmaf(-pc[r], c[col], c[r]);
        }
    }
    // nu[k] = sum_e cu[e] m[e][6 + k] (ascending e), on lane 6 + k.
    const float cu[6] = {0.5f * w.c0, w.c1, 0.5f * w.c2, 1.0f + w.l0, w.l1, w.t0};
    const float cv[6] = {0.5f * w.c3, w.c4, 0.5f * w.c5, w.l2, 1.0f + w.l3, w.t1};
    float au = 0.0f, av = 0.0f;
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        au = fmaf(cu[r], c[r], au);
        av = fmaf(cv[r], c[r], av);
    }
    float nu[6], nv[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        nu[k] = __shfl_sync(mask, au, 6 + k, 16);
        nv[k] = __shfl_sync(mask, av, 6 + k, 16);
    }
    w.c0 = 2.0f * nu[0]; w.c1 = nu[1]; w.c2 = 2.0f * nu[2];
    w.c3 = 2.0f * nv[0]; w.c4 = nv[1]; w.c5 = 2.0f * nv[2];
    w.t0 = nu[5];
    w.t1 = nv[5];
    w.l0 = nu[3] - 1.0f; w.l1 = nu[4];
    w.l2 = nv[3];        w.l3 = nv[4] - 1.0f;
    return true;
}

// icgn.wgsl:103-111 optional stagnation check (status 3 internal).
__device__ __forceinline__ float divergence_status(const SolveArgs &a, float change, unsigned count,
                                                   float status, float &previous, unsigned &stalled) {
    if (a.div_patience == 0 || status != 0.0f) return status;
    if (count >= (unsigned)a.div_min) stalled = (change >= previous) ? stalled + 1u : 0u;
    previous = change;
    return (stalled >= (unsigned)a.div_patience) ? 3.0f : status;
}

// Gauss-Newton update from the reduced totals (icgn.wgsl:801-921).  Returns
// the new status; modifies the warp on a successful composition.
// Quadratic: `sl` / `mask` as for compose_quadratic; lane r of each 16-lane
// segment forms row r of H^-1 r and the rows are exchanged by shuffles.
template <int MODEL>
__device__ __forceinline__ float gn_update(const SolveArgs &a, const float (&t)[SumCount<MODEL>::value],
                                           const float *__restrict__ md, const float *__restrict__ hi,
                                           float wsum, float half, unsigned it1, Warp &w,
                                           float &prev_change, unsigned &stalled, int sl, unsigned mask) {
    constexpr int n = parameter_count(MODEL);
    // Totals layout: 0 sum g, 1 sum g^2, 2 sum f g, then J^T g.
    float jg[12];
    if (MODEL == kModelTranslation) {
        jg[0] = t[3]; jg[3] = t[4];
        jg[1] = jg[2] = jg[4] = jg[5] = 0.0f;
    } else {
#pragma unroll
        for (int k = 0; k < SumCount<MODEL>::value - 3; ++k) jg[k] = t[3 + k];
    }
    const float mean_g = t[0] / wsum;
    const float norm_g = sqrtf(fmaxf(0.0f, fmaf(-t[0], mean_g, t[1])));
    const float norm_f = __ldg(md + 0);
    if (norm_g < 1e-9f || norm_f < 1e-9f) return -2.0f;
    const float ratio = norm_f / norm_g;
    const int sum_off = 2 + n;
    float delta[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) delta[k] = 0.0f;
    if (MODEL == kModelTranslation) {
        float r0 = fmaf(-ratio, fmaf(-mean_g, __ldg(md + sum_off + 0), jg[0]), __ldg(md + 2));
        float r3 = fmaf(-ratio, fmaf(-mean_g, __ldg(md + sum_off + 3), jg[3]), __ldg(md + 5));
        float a0 = __ldg(hi + 0) * r0;
        a0 = fmaf(__ldg(hi + 3), r3, a0);
        float a3 = __ldg(hi + 18) * r0;
        a3 = fmaf(__ldg(hi + 21), r3, a3);
        delta[0] = -a0;
        delta[3] = -a3;
    } else {
        float res[n];
#pragma unroll
        for (int k = 0; k < n; ++k)
            res[k] = fmaf(-ratio, fmaf(-mean_g, __ldg(md + sum_off + k), jg[k]), __ldg(md + 2 + k));
        if (MODEL == kModelQuadratic) {
            const int row = sl < n ? sl : 0;
            float acc = 0.0f;
#pragma unroll
            for (int k = 0; k < n; ++k) acc = fmaf(__ldg(hi + row * n + k), res[k], acc);
#pragma unroll
            for (int r = 0; r < n; ++r) delta[r] = -__shfl_sync(mask, acc, r, 16);
        } else {
#pragma unroll
            for (int r = 0; r < n; ++r) {
                float acc = 0.0f;
#pragma unroll
                for (int k = 0; k < n; ++k) acc = fmaf(__ldg(hi + r * n + k), res[k], acc);
                delta[r] = -acc;
            }
        }
    }
    float change;
    if (MODEL == kModelQuadratic) {
        if (!compose_quadratic(w, delta, sl, mask)) return -1.0f;
        change = 0.0f;
#pragma unroll
        for (int p = 0; p < 9; ++p) {
            float x = (float)(p % 3 - 1) * half, y = (float)(p / 3 - 1) * half;
            float hx2 = 0.5f * x * x, xy = x * y, hy2 = 0.5f * y * y;
            float ca = fmaf(delta[2], y, fmaf(delta[1], x, delta[0]));
            ca = ca + fmaf(delta[6], hx2, fmaf(delta[7], xy, delta[8] * hy2));
            float cb = fmaf(delta[5], y, fmaf(delta[4], x, delta[3]));
            cb = cb + fmaf(delta[9], hx2, fmaf(delta[10], xy, delta[11] * hy2));
            change = fmaxf(change, length2(ca, cb));
        }
    } else if (MODEL == kModelTranslation) {
        w.t0 = w.t0 - delta[0];
        w.t1 = w.t1 - delta[3];
        change = length2(delta[0], delta[3]);
    } else {
        const float det = fmaf(1.0f + delta[1], 1.0f + delta[5], -(delta[2] * delta[4]));
        if (fabsf(det) < 1e-8f) return -1.0f;
        const float i11 = (1.0f + delta[5]) / det, i12 = -delta[2] / det;
        const float i21 = -delta[4] / det, i22 = (1.0f + delta[1]) / det;
        const float w11 = 1.0f + w.l0, w12 = w.l1, w21 = w.l2, w22 = 1.0f + w.l3;
        const float itx = -fmaf(i11, delta[0], i12 * delta[3]);
        const float ity = -fmaf(i21, delta[0], i22 * delta[3]);
        w.t0 = w.t0 + fmaf(w11, itx, w12 * ity);
        w.t1 = w.t1 + fmaf(w21, itx, w22 * ity);
        const float u11 = fmaf(w11, i11, w12 * i21), u12 = fmaf(w11, i12, w12 * i22);
        const float u21 = fmaf(w21, i11, w22 * i21), u22 = fmaf(w21, i12, w22 * i22);
        w.l0 = u11 - 1.0f; w.l1 = u12; w.l2 = u21; w.l3 = u22 - 1.0f;
        change = 0.0f;
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            float x = (p == 1 || p == 3) ? half : -half;
            float y = (p >= 2) ? half : -half;
            float ca = fmaf(delta[2], y, fmaf(delta[1], x, delta[0]));
            float cb = fmaf(delta[5], y, fmaf(delta[4], x, delta[3]));
            change = fmaxf(change, length2(ca, cb));
        }
    }
    const float zncc = t[2] / (norm_f * norm_g);
    const float conv = (change >= a.tolerance) ? 0.0f : (zncc >= a.zncc_min ? 1.0f : -2.0f);
    return divergence_status(a, change, it1, conv, prev_change, stalled);
}

// One pixel's contribution to the lane's sums (icgn.wgsl:712-780), in the
// reference's order: sum w g, w g^2, w f g, then the Jacobian-weighted terms.
template <int MODEL, bool GAUSS, int N>
__device__ __forceinline__ void accumulate_pixel(float (&s)[N], const SolveArgs &a, float g, unsigned ridx, int p,
                                                 float lx, float ly, float ref_mean, float hx2, float xy,
                                                 float hy2) {
    const float4 rv = __ldg(a.plane + ridx);
    const float f = rv.x - ref_mean;
    float wc = g, wf = f;
    if (GAUSS) {
        const float wt = __ldg(a.weights + p);
        wc = wt * g;
        wf = wt * f;
    }
    const float gxg = rv.y * wc, gyg = rv.z * wc;
    s[0] = s[0] + wc;
    s[1] = fmaf(wc, g, s[1]);
    s[2] = fmaf(wf, g, s[2]);
    if (MODEL == kModelTranslation) {
        s[3] = s[3] + gxg;
        s[4] = s[4] + gyg;
    } else {
        s[3] = s[3] + gxg;
        s[4] = fmaf(gxg, lx, s[4]);
        s[5] = fmaf(gxg, ly, s[5]);
        s[6] = s[6] + gyg;
        s[7] = fmaf(gyg, lx, s[7]);
        s[8] = fmaf(gyg, ly, s[8]);
        if (MODEL == kModelQuadratic) {
            s[9] = fmaf(gxg, hx2, s[9]);
            s[10] = fmaf(gxg, xy, s[10]);
            s[11] = fmaf(gxg, hy2, s[11]);
            s[12] = fmaf(gyg, hx2, s[12]);
            s[13] = fmaf(gyg, xy, s[13]);
            s[14] = fmaf(gyg, hy2, s[14]);
        }
    }
}

// Packed FP32 pairs (sm_100 FADD2 / FMUL2 / FFMA2): component k of every
// operation is the scalar operation of pixel k, rounded identically.
__device__ __forceinline__ float2 pair(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// bspline_weights() of two fractions.  1 - t and px - fx are formed as
// fma(t, -1, 1) and fma(fx, -1, px): exact products, so each equals the
// scalar subtraction bit for bit.
__device__ __forceinline__ void bspline_weights2(float2 t, float2 w[4]) {
    const float2 k6 = pair(1.0f / 6.0f), one = pair(1.0f), m1 = pair(-1.0f), three = pair(3.0f);
    const float2 t2 = mul2(t, t), t3 = mul2(t2, t), s = fma2(t, m1, one);
    w[0] = mul2(mul2(mul2(s, s), s), k6);
    w[1] = mul2(fma2(fma2(three, t, pair(-6.0f)), t2, pair(4.0f)), k6);
    w[2] = mul2(fma2(fma2(fma2(pair(-3.0f), t, three), t, three), t, one), k6);
    w[3] = mul2(t3, k6);
}

// sample_target<kInterpBspline, false> of two positions: the 4x4 coefficient
// taps of each pixel in one register pair per tap, the row and column sums
// as packed FMAs in the scalar order.
template <bool CLAMP>
__device__ __forceinline__ float2 sample_bspline_pair(const float *__restrict__ coef, int W, int H, float2 px,
                                                      float2 py) {
    const float fxa = floorf(px.x), fxb = floorf(px.y), fya = floorf(py.x), fyb = floorf(py.y);
    const float2 m1 = pair(-1.0f);
    float2 wx[4], wy[4];
    bspline_weights2(fma2(make_float2(fxa, fxb), m1, px), wx);
    bspline_weights2(fma2(make_float2(fya, fyb), m1, py), wy);
    const int bxa = (int)fxa, bxb = (int)fxb, bya = (int)fya, byb = (int)fyb;
    float2 value = pair(0.0f);
    // Clamping changes a tap only when a footprint reaches the plane border;
    // footprints inside take the unclamped addressing below (same taps).
    const bool border = CLAMP && (min(bxa, bxb) < 1 || max(bxa, bxb) > W - 3 || min(bya, byb) < 1 ||
                                  max(bya, byb) > H - 3);
    if (border) {
        // Every tap index clamped to the plane, as sample_target<.., true>.
        int xa[4], xb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            xa[i] = clampi(bxa + i - 1, 0, W - 1);
            xb[i] = clampi(bxb + i - 1, 0, W - 1);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float *ra = coef + (size_t)clampi(bya + j - 1, 0, H - 1) * W;
            const float *rb = coef + (size_t)clampi(byb + j - 1, 0, H - 1) * W;
            float2 row = pair(0.0f);
#pragma unroll
            for (int i = 0; i < 4; ++i) row = fma2(wx[i], make_float2(__ldg(ra + xa[i]), __ldg(rb + xb[i])), row);
            value = fma2(wy[j], row, value);
        }
        return value;
    }
    const float *ra = coef + (size_t)(bya - 1) * W + (bxa - 1);
    const float *rb = coef + (size_t)(byb - 1) * W + (bxb - 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float2 row = pair(0.0f);
#pragma unroll
        for (int i = 0; i < 4; ++i) row = fma2(wx[i], make_float2(__ldg(ra + i), __ldg(rb + i)), row);
        value = fma2(wy[j], row, value);
        ra += W;
        rb += W;
    }
    return value;
}

// ---------------------------------------------------------------- staged tiles
// Staged solver modes: each warp keeps one shared-memory tile of the
// coefficient plane, TW x TH floats loaded by TMA (cp.async.bulk.tensor),
// that covers the tap footprints of its subsets; the pixel loop samples from
// the tile instead of global memory.  The tile is reloaded only when a
// subset's footprint leaves it, so over a subset's iterations (whose warps
// move by fractions of a pixel) it is usually loaded once.  A subset whose
// footprint does not fit the tile samples from global memory that
// iteration.  Values and arithmetic are those of the exact loop: results are
// bit-identical to it.
struct StageTile {
    const void *map;  // CUtensorMap of the coefficient plane (box TW x TH)
    float *tile;      // the warp's tile, TW x TH row-major, 128-byte aligned
    uint64_t *bar;    // its mbarrier (one arrival + the tile's bytes)
};
struct StageState {
    int tx0, ty0;     // tile origin (tx0 % 4 == 0: 16-byte TMA coordinate)
    unsigned phase;   // parity of the next load's completion
    bool valid;       // the tile holds the plane at (tx0, ty0)
    bool broken;      // a load's wait expired: no further staging in this warp
    bool pending;     // a load may still be landing (after an expired wait)
};
constexpr uint32_t kStageSpinLimit = 1u << 22;

__device__ __forceinline__ bool stage_wait(uint64_t *bar, unsigned parity) {
    const uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
    for (uint32_t i = 0; i < kStageSpinLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Taps a subset's samples can touch under warp w, with a one-pixel margin:
// x in [b0, b1], y in [b2, b3] (b0 > b1 when `none`).  The sample positions
// are origin + (lx, ly) + displacement over |lx|, |ly| <= half.
template <int MODEL>
__device__ __forceinline__ void stage_box(const Warp &w, float ox, float oy, float half, bool none, int (&b)[4]) {
    b[0] = 1 << 29; b[1] = -(1 << 29); b[2] = 1 << 29; b[3] = -(1 << 29);
    if (none) return;
    const float ex = half * (fabsf(1.0f + w.l0) + fabsf(w.l1));
    const float ey = half * (fabsf(w.l2) + fabsf(1.0f + w.l3));
    const float cx = ox + w.t0, cy = oy + w.t1;
    const float x0 = floorf(cx - ex) - 2.0f, x1 = floorf(cx + ex) + 3.0f;
    const float y0 = floorf(cy - ey) - 2.0f, y1 = floorf(cy + ey) + 3.0f;
    if (!(x0 > -1e6f && x1 < 1e6f && y0 > -1e6f && y1 < 1e6f)) {
        b[0] = -(1 << 29); b[1] = 1 << 29;  // never fits: sampled from global memory
        b[2] = -(1 << 29); b[3] = 1 << 29;
        return;
    }
    b[0] = (int)x0; b[1] = (int)x1; b[2] = (int)y0; b[3] = (int)y1;
}

// Tile origin for box b, or false when b does not fit a TW x TH tile.
template <int TW, int TH>
__device__ __forceinline__ bool stage_origin(const int (&b)[4], int &tx0, int &ty0) {
    if (b[1] - b[0] + 1 > TW || b[3] - b[2] + 1 > TH) return false;
    const int cx = b[0] - (TW - (b[1] - b[0] + 1)) / 2;
    tx0 = cx - (((cx % 4) + 4) % 4);
    ty0 = b[2] - (TH - (b[3] - b[2] + 1)) / 2;
    return b[0] >= tx0 && b[1] < tx0 + TW;
}

template <int TW, int TH>
__device__ __forceinline__ bool stage_contains(const StageState &ss, const int (&b)[4]) {
    return ss.valid && b[0] >= ss.tx0 && b[1] < ss.tx0 + TW && b[2] >= ss.ty0 && b[3] < ss.ty0 + TH;
}

// Warp-uniform tile update at the top of an iteration: gathers the warp's
// subset boxes (two per warp for 16 lanes), reloads the tile when a live
// subset's box is outside it (over the union of the boxes when that fits,
// else the first live subset's box) and returns whether this lane's subset
// samples from the tile.
template <int LANES, int TW, int TH>
__device__ __forceinline__ bool stage_update(const StageTile &st, StageState &ss, const int (&b)[4],
                                             int lane_in_warp) {
    int A[4], B[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int o = LANES == 16 ? __shfl_xor_sync(kFullMask, b[k], 16) : b[k];
        const bool upper = LANES == 16 && (lane_in_warp & 16);
        A[k] = upper ? o : b[k];
        B[k] = upper ? b[k] : o;
    }
    const bool liveA = A[0] <= A[1], liveB = LANES == 16 && B[0] <= B[1];
    const bool need = (liveA && !stage_contains<TW, TH>(ss, A)) || (liveB && !stage_contains<TW, TH>(ss, B));
    if (need && !ss.broken) {
        int U[4] = {min(A[0], B[0]), max(A[1], B[1]), min(A[2], B[2]), max(A[3], B[3])};
        if (!liveA) { U[0] = B[0]; U[1] = B[1]; U[2] = B[2]; U[3] = B[3]; }
        if (!liveB) { U[0] = A[0]; U[1] = A[1]; U[2] = A[2]; U[3] = A[3]; }
        int tx0 = 0, ty0 = 0;
        bool ok = stage_origin<TW, TH>(U, tx0, ty0);
        if (!ok && liveA) ok = stage_origin<TW, TH>(A, tx0, ty0);
        if (!ok && liveB) ok = stage_origin<TW, TH>(B, tx0, ty0);
        if (ok) {
            // Every lane's reads of the old tile precede the asynchronous
            // writes of the new one.
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            const uint32_t bar = static_cast<uint32_t>(__cvta_generic_to_shared(st.bar));
            if (lane_in_warp == 0) {
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                             "r"((uint32_t)(TW * TH * 4))
                             : "memory");
                asm volatile(
                    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
                    "%4}], [%2];" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(st.tile))),
                    "l"(reinterpret_cast<uint64_t>(st.map)), "r"(bar), "r"(tx0), "r"(ty0)
                    : "memory");
            }
            int landed = 0;
            if (lane_in_warp == 0) landed = stage_wait(st.bar, ss.phase) ? 1 : 0;
            landed = __shfl_sync(kFullMask, landed, 0);
            __syncwarp();
            if (landed) {
                ss.phase ^= 1u;
                ss.valid = true;
                ss.tx0 = tx0;
                ss.ty0 = ty0;
            } else {
                ss.valid = false;
                ss.broken = true;
                ss.pending = true;
            }
        }
        // else: no box fits; this iteration samples from global memory and
        // the tile is kept for later subsets
    }
    return b[0] <= b[1] && stage_contains<TW, TH>(ss, b);
}

// sample_bspline_pair<false> from a staged tile whose origin is (tx0, ty0):
// the same taps at tile-relative addresses, the same arithmetic.
template <int TW>
__device__ __forceinline__ float2 sample_bspline_pair_tile(const float *tile, int tx0, int ty0, float2 px, float2 py) {
    const float fxa = floorf(px.x), fxb = floorf(px.y), fya = floorf(py.x), fyb = floorf(py.y);
    const float2 m1 = pair(-1.0f);
    float2 wx[4], wy[4];
    bspline_weights2(fma2(make_float2(fxa, fxb), m1, px), wx);
    bspline_weights2(fma2(make_float2(fya, fyb), m1, py), wy);
    const float *ra = tile + ((int)fya - 1 - ty0) * TW + ((int)fxa - 1 - tx0);
    const float *rb = tile + ((int)fyb - 1 - ty0) * TW + ((int)fxb - 1 - tx0);
    float2 value = pair(0.0f);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float2 row = pair(0.0f);
#pragma unroll
        for (int i = 0; i < 4; ++i) row = fma2(wx[i], make_float2(ra[i], rb[i]), row);
        value = fma2(wy[j], row, value);
        ra += TW;
        rb += TW;
    }
    return value;
}

template <int MODEL, int INTERP, int LANES, bool GAUSS, bool PART = false, int TW = 0, int TH = 0>
__device__ __forceinline__ void solve_group(const SolveArgs &a, int group, int glane, int lane_in_warp,
                                            float *red, const StageTile *st = nullptr, StageState *ss = nullptr) {
    constexpr int N = SumCount<MODEL>::value;
    constexpr bool kBlock = LANES > 32;
    constexpr bool kClamp = MODEL == kModelQuadratic;
    // Pixel pairs with packed FP32 arithmetic: B-spline sampling of
    // complete windows.
    constexpr bool kPair = GBDIC_SOLVER_PAIRS && INTERP == kInterpBspline && !PART &&
                           (MODEL != kModelQuadratic || GBDIC_QUAD_PAIRS);
    const int live = (!PART && a.list_count != nullptr) ? min(a.count, (int)__ldg(a.list_count)) : a.count;
    const bool exists = group < live;
    // Partial windows: group -> window index; support words and box.  List
    // mode: group -> listed subset.
    const int idx = PART ? (exists ? __ldg(a.partial_index + group) : 0)
                         : (a.subset_list != nullptr ? (exists ? __ldg(a.subset_list + group) : 0) : group);
    const uint32_t *support = PART ? a.support + (size_t)(exists ? group : 0) * a.support_words : nullptr;
    const float4 box = PART ? __ldg(a.support_box + (exists ? group : 0)) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int sidx = exists ? idx : 0;
    const float *md = a.meta + (size_t)sidx * meta_stride(MODEL);
    const float *hi = a.inv + (size_t)sidx * parameter_count(MODEL) * parameter_count(MODEL);
    Warp w = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    bool enabled = exists;
    if (a.seed != nullptr && exists) {
        const float4 *s = reinterpret_cast<const float4 *>(a.seed + (size_t)sidx * state_stride(MODEL));
        float4 s0 = __ldg(s), s1 = __ldg(s + 1);
        w.t0 = s0.x; w.l0 = s0.y; w.l1 = s0.z; w.t1 = s0.w;
        w.l2 = s1.x; w.l3 = s1.y;
        if (MODEL == kModelQuadratic) {
            float4 s2 = __ldg(s + 2);
            w.c0 = s1.z; w.c1 = s1.w; w.c2 = s2.x; w.c3 = s2.y; w.c4 = s2.z; w.c5 = s2.w;
        }
        enabled = __ldg(a.active + sidx) != 0u;
    }
    if (MODEL == kModelTranslation) { w.l0 = w.l1 = w.l2 = w.l3 = 0.0f; }
    const float mvalid = __ldg(md + 1);
    const bool valid = enabled && (PART ? mvalid == -4.0f : mvalid >= 0.5f);
    const float rejected = (a.roi_enabled && !PART) ? fminf(-1.0f, mvalid) : -1.0f;
    float status = valid ? 0.0f : rejected;
    float iters = 0.0f;
    bool done = !exists;
    const int S = a.S;
    const int gx = sidx % a.grid_w, gy = sidx / a.grid_w;
    const int px0 = gx * a.stride, py0 = gy * a.stride;
    const float half = 0.5f * ((float)S - 1.0f);
    const float ref_mean = (a.use_mean || PART) ? __ldg(md + (MODEL == kModelQuadratic ? 26 : 14)) : 0.0f;
    const float wsum = (GAUSS || PART) ? __ldg(md + 3 + 2 * parameter_count(MODEL)) : (float)(S * S);
    float prev_change = 3.402823e38f;
    unsigned stalled = 0u;
    const int npix = S * S;
    const int ldiv = LANES / S, lmod = LANES % S;
    const int col0 = glane % S, row0 = glane / S;
    const int W = a.W, H = a.H;
    // Pixel bookkeeping without conversions: column / row as exact small
    // float integers, the window origin plus `half` (so origin + lx is the
    // pixel's integer coordinate exactly), and the reference-plane index.
    const float fS = (float)S, flmod = (float)lmod, fldiv = (float)ldiv;
    const float fcol0 = (float)col0, frow0 = (float)row0;
    const float ox = (float)px0 + half, oy = (float)py0 + half;
    const unsigned ridx0 = (unsigned)(py0 + row0) * (unsigned)W + (unsigned)(px0 + col0);
    const unsigned rstep = (unsigned)lmod + (unsigned)ldiv * (unsigned)W, rwrap = (unsigned)(W - S);
    // Lanes that run the update together: the group's half warp for 16-lane
    // groups (groups are uniform in `done`), else the whole warp.
    const unsigned seg_mask = LANES == 16 ? (0xffffu << (lane_in_warp & 16)) : kFullMask;

    for (int it = 0; it < 30; ++it) {
        if (!done) {
            if (!(a.div_patience != 0 && status == 3.0f)) {
                const bool in = PART ? warp_inside_box<MODEL>(w, px0, py0, half, box, W, H)
                                     : warp_inside<MODEL>(w, px0, py0, S, half, W, H);
                if (!in) {
                    if (!a.roi_enabled || status > -2.5f) status = -1.0f;
                }
            }
            if (it >= a.iterations || fabsf(status) > 0.5f) done = true;
        }
        if (kBlock) {
            if (!__syncthreads_or(!done)) break;
        } else {
            if (__all_sync(kFullMask, done)) break;
        }
        // Staged modes: the warp's tile covers this subset's taps this
        // iteration (warp-uniform update; complete windows only).
        bool staged = false;
        if constexpr (TW > 0) {
            int box[4];
            stage_box<MODEL>(w, ox, oy, half, done, box);
            staged = stage_update<LANES, TW, TH>(*st, *ss, box, lane_in_warp);
        }
        float s[N];
#pragma unroll
        for (int k = 0; k < N; ++k) s[k] = 0.0f;
        if (!done) {
            float fcol = fcol0, frow = frow0;
            unsigned ridx = ridx0;
            int p = glane;
            if (kPair) {
                // Two consecutive pixels of the lane per step (p and
                // p + LANES), sampled with packed FP32 pairs and accumulated
                // one after the other, as in the scalar loop.
                const float2 nh = pair(-half), ox2 = pair(ox), oy2 = pair(oy);
                const float2 t0 = pair(w.t0), t1 = pair(w.t1);
                const float2 l0 = pair(w.l0), l1 = pair(w.l1), l2 = pair(w.l2), l3 = pair(w.l3);
                const float2 half2 = pair(0.5f);
                for (; p + LANES < npix; p += 2 * LANES) {
                    float fcolb = fcol + flmod, frowb = frow + fldiv;
                    unsigned ridxb = ridx + rstep;
                    if (fcolb >= fS) { fcolb -= fS; frowb += 1.0f; ridxb += rwrap; }
                    const float2 lx = add2(make_float2(fcol, fcolb), nh), ly = add2(make_float2(frow, frowb), nh);
                    float2 dx = t0, dy = t1;
                    float2 hx2 = pair(0.0f), xy = pair(0.0f), hy2 = pair(0.0f);
                    if (MODEL != kModelTranslation) {
                        dx = add2(t0, fma2(l0, lx, mul2(l1, ly)));
                        dy = add2(t1, fma2(l2, lx, mul2(l3, ly)));
                    }
                    if (MODEL == kModelQuadratic) {
                        // displacement<kModelQuadratic> on both pixels.
                        hx2 = mul2(mul2(half2, lx), lx);
                        xy = mul2(lx, ly);
                        hy2 = mul2(mul2(half2, ly), ly);
                        dx = add2(dx, fma2(pair(w.c0), hx2, fma2(pair(w.c1), xy, mul2(pair(w.c2), hy2))));
                        dy = add2(dy, fma2(pair(w.c3), hx2, fma2(pair(w.c4), xy, mul2(pair(w.c5), hy2))));
                    }
                    const float2 spx = add2(add2(ox2, lx), dx), spy = add2(add2(oy2, ly), dy);
                    float2 g;
                    if constexpr (TW > 0) {
                        g = staged ? sample_bspline_pair_tile<TW>(st->tile, ss->tx0, ss->ty0, spx, spy)
                                   : sample_bspline_pair<kClamp>(a.coef, W, H, spx, spy);
                    } else {
                        g = sample_bspline_pair<kClamp>(a.coef, W, H, spx, spy);
                    }
                    accumulate_pixel<MODEL, GAUSS, N>(s, a, g.x, ridx, p, lx.x, ly.x, ref_mean, hx2.x, xy.x, hy2.x);
                    accumulate_pixel<MODEL, GAUSS, N>(s, a, g.y, ridxb, p + LANES, lx.y, ly.y, ref_mean, hx2.y, xy.y,
                                                      hy2.y);
                    fcol = fcolb + flmod;
                    frow = frowb + fldiv;
                    ridx = ridxb + rstep;
                    if (fcol >= fS) { fcol -= fS; frow += 1.0f; ridx += rwrap; }
                }
            }
            for (; p < npix; p += LANES) {
                if (PART && !((__ldg(support + (p >> 5)) >> (p & 31)) & 1u)) {
                    fcol += flmod;
                    frow += fldiv;
                    ridx += rstep;
                    if (fcol >= fS) { fcol -= fS; frow += 1.0f; ridx += rwrap; }
                    continue;
                }
                const float lx = fcol - half, ly = frow - half;
                float hx2 = 0.0f, xy = 0.0f, hy2 = 0.0f;
                if (MODEL == kModelQuadratic) {
                    hx2 = 0.5f * lx * lx;
                    xy = lx * ly;
                    hy2 = 0.5f * ly * ly;
                }
                float dx, dy;
                displacement<MODEL>(w, lx, ly, hx2, xy, hy2, dx, dy);
                const float g = sample_target<INTERP, kClamp>(a.coef, a.img, W, H, (ox + lx) + dx, (oy + ly) + dy);
                accumulate_pixel<MODEL, GAUSS, N>(s, a, g, ridx, p, lx, ly, ref_mean, hx2, xy, hy2);
                fcol += flmod;
                frow += fldiv;
                ridx += rstep;
                if (fcol >= fS) { fcol -= fS; frow += 1.0f; ridx += rwrap; }
            }
        }
        if (kBlock) reduce_block<LANES, N>(s, red, glane);
        else reduce_warp<LANES, N>(s, lane_in_warp);
        if (!done) {
            iters = (float)(it + 1);
            status = gn_update<MODEL>(a, s, md, hi, wsum, half, (unsigned)(it + 1), w, prev_change, stalled,
                                      lane_in_warp & 15, seg_mask);
        }
    }
    if (a.iteration_total != nullptr && exists && glane == 0 && iters > 0.0f)
        atomicAdd(a.iteration_total, (unsigned long long)iters);
    if (exists && (enabled || !a.preserve_disabled) && glane == 0) {
        const float final_status = (a.div_patience != 0 && status == 3.0f) ? 0.0f : status;
        float4 *o = reinterpret_cast<float4 *>(a.state + (size_t)idx * state_stride(MODEL));
        o[0] = make_float4(w.t0, w.l0, w.l1, w.t1);
        if (MODEL == kModelQuadratic) {
            o[1] = make_float4(w.l2, w.l3, w.c0, w.c1);
            o[2] = make_float4(w.c2, w.c3, w.c4, w.c5);
            o[3] = make_float4(final_status, iters, 0.0f, 0.0f);
        } else {
            o[1] = make_float4(w.l2, w.l3, final_status, iters);
        }
    }
}

template <int MODEL, int INTERP, int LANES, bool GAUSS, bool PART = false>
__global__ void __launch_bounds__(128, MODEL == kModelQuadratic ? GBDIC_QUAD_MIN_BLOCKS : GBDIC_SOLVER_MIN_BLOCKS) icgn_kernel(SolveArgs a) {
    constexpr bool kBlock = LANES > 32;
    constexpr int kUnitThreads = kBlock ? 128 : 32;
    constexpr int kGroups = kUnitThreads / LANES;
    constexpr int N = SumCount<MODEL>::value;
    __shared__ float red_smem[kBlock ? 128 * N : 1];
    __shared__ int unit_base;
    const int tid = threadIdx.x;
    const int glane = tid % LANES;
    const int group_in_unit = (tid % kUnitThreads) / LANES;
    const int lane_in_warp = tid & 31;
    const int units_per_block = 128 / kUnitThreads;
    const long long unit = (long long)blockIdx.x * units_per_block + tid / kUnitThreads;
    float *red = red_smem + (kBlock ? group_in_unit * LANES * N : 0);
    const int count = (!PART && a.list_count != nullptr) ? min(a.count, (int)__ldg(a.list_count)) : a.count;
    for (;;) {
        int base;
        if (a.persistent) {
            if (kBlock) {
                if (tid == 0) unit_base = (int)atomicAdd(a.work_counter, (unsigned)kGroups);
                __syncthreads();
                base = unit_base;
                __syncthreads();
            } else {
                int v = 0;
                if (lane_in_warp == 0) v = (int)atomicAdd(a.work_counter, (unsigned)kGroups);
                base = __shfl_sync(kFullMask, v, 0);
            }
        } else {
            base = unit * kGroups < (long long)count ? (int)(unit * kGroups) : count;
        }
        if (base >= count) break;
        solve_group<MODEL, INTERP, LANES, GAUSS, PART>(a, base + group_in_unit, glane, lane_in_warp, red);
        if (!a.persistent) break;
    }
}

#define GBDIC_SOLVER_CASE(MODEL, INTERP, LANES)                                                   \
    if (interp == INTERP && lanes == LANES) {                                                     \
        if (occupancy_only) {                                                                      \
            int blocks = 0;                                                                        \
            if (gauss)                                                                             \
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                     \
                    &blocks, icgn_kernel<MODEL, INTERP, LANES, true>, 128, 0);                     \
            else                                                                                   \
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                     \
                    &blocks, icgn_kernel<MODEL, INTERP, LANES, false>, 128, 0);                    \
            *occupancy_only = blocks;                                                              \
            return cudaSuccess;                                                                    \
        }                                                                                          \
        if (gauss)                                                                                 \
            icgn_kernel<MODEL, INTERP, LANES, true><<<grid, 128, 0, stream>>>(a);                  \
        else                                                                                       \
            icgn_kernel<MODEL, INTERP, LANES, false><<<grid, 128, 0, stream>>>(a);                 \
        return cudaGetLastError();                                                                 \
    }

// Launcher for one model (instantiated in solver_<model>.cu).  With
// occupancy_only set, nothing is launched and the resident CTA count per SM
// of the selected variant is stored there instead.
#define GBDIC_SOLVER_MODEL(MODEL)                                                                 \
    template <>                                                                                    \
    cudaError_t launch_icgn_model<MODEL>(const SolveArgs &a, int interp, int lanes, bool gauss,    \
                                         int grid, cudaStream_t stream, int *occupancy_only) {     \
        GBDIC_SOLVER_CASE(MODEL, kInterpBspline, 16)                                               \
        GBDIC_SOLVER_CASE(MODEL, kInterpBspline, 32)                                               \
        GBDIC_SOLVER_CASE(MODEL, kInterpBspline, 64)                                               \
        GBDIC_SOLVER_CASE(MODEL, kInterpBspline, 128)                                              \
        GBDIC_SOLVER_CASE(MODEL, kInterpLinear, 16)                                                \
        GBDIC_SOLVER_CASE(MODEL, kInterpLinear, 32)                                                \
        GBDIC_SOLVER_CASE(MODEL, kInterpLinear, 64)                                                \
        GBDIC_SOLVER_CASE(MODEL, kInterpLinear, 128)                                               \
        GBDIC_SOLVER_CASE(MODEL, kInterpKeys, 16)                                                  \
        GBDIC_SOLVER_CASE(MODEL, kInterpKeys, 32)                                                  \
        GBDIC_SOLVER_CASE(MODEL, kInterpKeys, 64)                                                  \
        GBDIC_SOLVER_CASE(MODEL, kInterpKeys, 128)                                                 \
        return cudaErrorInvalidValue;                                                              \
    }

}  // namespace gbdic
