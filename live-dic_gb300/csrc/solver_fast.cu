// Sliding-window IC-GN solver ("fast" mode) for complete B-spline windows of
// the translation and affine models (reference operations:
// shaders/icgn.wgsl:230-319 sample_cubic, 712-799 the pixel loop and its
// reduction; the Gauss-Newton update of 801-921 is shared with the exact
// solver, solver_impl.cuh).
//
// The exact solver keeps the reference's pixel-to-lane order (pixel p on lane
// p mod LANES): a lane's consecutive pixels are LANES columns apart, every
// sample gathers its 16 coefficients afresh and the L1 data pipe is the
// limiter.  Here the pixels are owned by vertical runs instead:
//
//  * Each of the S columns is cut into m row segments of L = ceil(S / m)
//    rows; run q covers column q mod S, segment q / S.  A lane walks two runs
//    at once (slots A and B: runs (2 ph) LANES + lane and (2 ph + 1) LANES +
//    lane of phase ph), one row per step, so at every step the group's lanes
//    read neighbouring columns of one row.  m is chosen on the host to
//    minimise the steps, phases x L (icgn_fast_segments).
//  * Consecutive samples of a run are one row apart; under a warp whose
//    gradient is small their 4 x 4 tap footprints share three rows.  The taps
//    of both runs live in a ring of five rows of float2 registers (run A in
//    .x, run B in .y): four rows form the current sample's window, and while
//    it is computed the fifth receives the next sample's new bottom row (four
//    loads) when that sample's footprint is exactly one row lower, so the
//    loads of a step overlap the arithmetic of the one before.  A sample
//    whose footprint jumped (a run's first, or a column change under the
//    warp's gradient) loads its sixteen taps itself.  The ring's rotation is
//    resolved at compile time by unrolling the steps five at a time.
//  * Positions are window-local, q(k) = q0 + k s with the per-row step
//    s = (du/dy, 1 + dv/dy): one packed FMA per axis and sample, no large
//    coordinates and no int/float conversions beyond the floors.
//  * B-spline weights, the 4 x 4 tap sums and the lane's partial sums run on
//    packed FP32 pairs (FFMA2 / FMUL2 / FADD2), A and B in the two halves;
//    the halves are added before the reduction across lanes.
//  * This unit compiles with FMA contraction.
//
// The summation order therefore differs from the reference's.  Results agree
// with the exact solver within the parity tolerances (statuses identical
// except threshold-borderline windows, |du| <= 1e-3 px, |grad u| <= 1e-5;
// tests/test_gpu_fast_solver.py).  The bounds check (every warped corner in
// [2, W-3] x [2, H-3]) keeps every footprint inside the plane, as in the
// exact solver, so the ring loads need no clamping.
#include <climits>

#include "gbdic_kernels.h"
#include "solver_impl.cuh"

#ifndef GBDIC_FAST_MIN_BLOCKS
#define GBDIC_FAST_MIN_BLOCKS 4
#endif

namespace gbdic {

int icgn_fast_segments(int S, int lanes) {
    int best = 1, best_steps = INT_MAX;
    for (int m = 1; m <= S; ++m) {
        const int L = (S + m - 1) / m;
        const int phases = (S * m + 2 * lanes - 1) / (2 * lanes);
        const int steps = phases * L;
        if (steps < best_steps) {
            best_steps = steps;
            best = m;
        }
        if (L == 1) break;
    }
    return best;
}

bool icgn_fast_supported(int model, int interp, int lanes) {
    return interp == kInterpBspline && (model == kModelAffine || model == kModelTranslation) &&
           (lanes == 16 || lanes == 32);
}

namespace {

// One run walked by one half (slot) of the packed pairs.
struct Slot {
    int rows;     // rows in this run (0: idle)
    int ix, iy;   // floor of the current sample's window-local position
    int ridx;     // reference-plane index of the current sample
    bool fresh;   // the current sample's taps must be loaded in full
};

// Ring rows j = 0..3 of the window at rotation R are ring[(R + j) % 5]; the
// fifth row receives the next sample's new bottom row while the current
// sample is computed.
template <bool HI>
__device__ __forceinline__ void put(float2 &d, float v) {
    if (HI) d.y = v;
    else d.x = v;
}

template <int R, bool HI>
__device__ __forceinline__ void load_window(float2 (&ring)[5][4], const float *__restrict__ p, int W) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
        for (int i = 0; i < 4; ++i) put<HI>(ring[(R + j) % 5][i], __ldg(p + (size_t)j * W + i));
    }
}

template <int R, bool HI>
__device__ __forceinline__ void load_next_row(float2 (&ring)[5][4], const float *__restrict__ p) {
#pragma unroll
    for (int i = 0; i < 4; ++i) put<HI>(ring[(R + 4) % 5][i], __ldg(p + i));
}

// Walker state shared by both slots: window-local positions
// q(k) = q0 + k s of the current sample (x and y, slot A in .x, B in .y)
// and their floors.
struct Walk {
    float2 q0x, q0y, sx, sy;  // start positions and per-row steps
    float2 fx, fy;            // floors of the current positions
    float2 qx, qy;            // current positions
};

template <int MODEL, bool GAUSS, int N, int R>
__device__ __forceinline__ void fast_step(float2 (&acc)[N], float2 (&ring)[5][4], Slot &A, Slot &B, Walk &wk,
                                          float kf, int k, const SolveArgs &a, const float2 lx, float2 &ly,
                                          int px0, int py0, int wA, int wB, float ref_mean) {
    const bool actA = k < A.rows, actB = k < B.rows;
    if (!(actA || actB)) return;
    const int W = a.W;
    // Taps of the current sample that the previous step could not prefetch.
    if (actA && A.fresh) load_window<R, false>(ring, a.coef + (size_t)(py0 + A.iy - 1) * W + (px0 + A.ix - 1), W);
    if (actB && B.fresh) load_window<R, true>(ring, a.coef + (size_t)(py0 + B.iy - 1) * W + (px0 + B.ix - 1), W);
    // The next sample: position, floors, and its new row when it slides.
    const float2 kn = pair(kf + 1.0f);
    const float2 nqx = fma2(kn, wk.sx, wk.q0x), nqy = fma2(kn, wk.sy, wk.q0y);
    const float2 nfx = make_float2(floorf(nqx.x), floorf(nqx.y)), nfy = make_float2(floorf(nqy.x), floorf(nqy.y));
    const int nixA = (int)nfx.x, nixB = (int)nfx.y, niyA = (int)nfy.x, niyB = (int)nfy.y;
    const bool slideA = k + 1 < A.rows && nixA == A.ix && niyA == A.iy + 1;
    const bool slideB = k + 1 < B.rows && nixB == B.ix && niyB == B.iy + 1;
    if (slideA) load_next_row<R, false>(ring, a.coef + (size_t)(py0 + niyA + 2) * W + (px0 + nixA - 1));
    if (slideB) load_next_row<R, true>(ring, a.coef + (size_t)(py0 + niyB + 2) * W + (px0 + nixB - 1));
    // The current sample.  (Loading the plane entries one step ahead as
    // well costs more occupancy in registers than it hides in latency.)
    float4 ra = make_float4(0.0f, 0.0f, 0.0f, 0.0f), rb = ra;
    float wa = 0.0f, wb = 0.0f;
    if (actA) {
        ra = __ldg(a.plane + A.ridx);
        wa = GAUSS ? __ldg(a.weights + wA + k * a.S) : 1.0f;
    }
    if (actB) {
        rb = __ldg(a.plane + B.ridx);
        wb = GAUSS ? __ldg(a.weights + wB + k * a.S) : 1.0f;
    }
    float2 wx[4], wy[4];
    bspline_weights2(add2(wk.qx, mul2(wk.fx, pair(-1.0f))), wx);
    bspline_weights2(add2(wk.qy, mul2(wk.fy, pair(-1.0f))), wy);
    float2 g = pair(0.0f);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float2 row = mul2(wx[0], ring[(R + j) % 5][0]);
#pragma unroll
        for (int i = 1; i < 4; ++i) row = fma2(wx[i], ring[(R + j) % 5][i], row);
        g = fma2(wy[j], row, g);
    }
    // An idle slot contributes nothing: zero weight, zero sample.
    g = make_float2(actA ? g.x : 0.0f, actB ? g.y : 0.0f);
    const float2 wt = make_float2(wa, wb);
    const float2 f = mul2(add2(make_float2(ra.x, rb.x), pair(-ref_mean)), wt);
    const float2 wc = mul2(wt, g);
    acc[0] = add2(acc[0], wc);
    acc[1] = fma2(wc, g, acc[1]);
    acc[2] = fma2(f, g, acc[2]);
    const float2 gxg = mul2(make_float2(ra.y, rb.y), wc), gyg = mul2(make_float2(ra.z, rb.z), wc);
    if (MODEL == kModelTranslation) {
        acc[3] = add2(acc[3], gxg);
        acc[4] = add2(acc[4], gyg);
    } else {
        acc[3] = add2(acc[3], gxg);
        acc[4] = fma2(gxg, lx, acc[4]);
        acc[5] = fma2(gxg, ly, acc[5]);
        acc[6] = add2(acc[6], gyg);
        acc[7] = fma2(gyg, lx, acc[7]);
        acc[8] = fma2(gyg, ly, acc[8]);
    }
    // Advance both slots to the next sample.
    ly = add2(ly, pair(1.0f));
    wk.qx = nqx;
    wk.qy = nqy;
    wk.fx = nfx;
    wk.fy = nfy;
    A.fresh = !slideA;
    B.fresh = !slideB;
    A.ix = nixA;
    A.iy = niyA;
    B.ix = nixB;
    B.iy = niyB;
    A.ridx += W;
    B.ridx += W;
}

template <int MODEL, int LANES, bool GAUSS>
__device__ __forceinline__ void solve_group_fast(const SolveArgs &a, int group, int glane, int lane_in_warp) {
    constexpr int N = SumCount<MODEL>::value;
    const bool exists = group < a.count;
    const int sidx = exists ? group : 0;
    const float *md = a.meta + (size_t)sidx * meta_stride(MODEL);
    const float *hi = a.inv + (size_t)sidx * parameter_count(MODEL) * parameter_count(MODEL);
    Warp w = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    bool enabled = exists;
    if (a.seed != nullptr && exists) {
        const float4 *s = reinterpret_cast<const float4 *>(a.seed + (size_t)sidx * state_stride(MODEL));
        const float4 s0 = __ldg(s), s1 = __ldg(s + 1);
        w.t0 = s0.x; w.l0 = s0.y; w.l1 = s0.z; w.t1 = s0.w;
        w.l2 = s1.x; w.l3 = s1.y;
        enabled = __ldg(a.active + sidx) != 0u;
    }
    if (MODEL == kModelTranslation) { w.l0 = w.l1 = w.l2 = w.l3 = 0.0f; }
    const float mvalid = __ldg(md + 1);
    const bool valid = enabled && mvalid >= 0.5f;
    const float rejected = a.roi_enabled ? fminf(-1.0f, mvalid) : -1.0f;
    float status = valid ? 0.0f : rejected;
    float iters = 0.0f;
    bool done = !exists;
    const int S = a.S;
    const int px0 = (sidx % a.grid_w) * a.stride, py0 = (sidx / a.grid_w) * a.stride;
    const float half = 0.5f * ((float)S - 1.0f);
    const float ref_mean = a.use_mean ? __ldg(md + 14) : 0.0f;
    const float wsum = GAUSS ? __ldg(md + 3 + 2 * parameter_count(MODEL)) : (float)(S * S);
    float prev_change = 3.402823e38f;
    unsigned stalled = 0u;
    const int m = a.fast_segments;
    const int L = (S + m - 1) / m;
    const int runs = S * m;
    const int phases = (runs + 2 * LANES - 1) / (2 * LANES);
    const unsigned seg_mask = LANES == 16 ? (0xffffu << (lane_in_warp & 16)) : kFullMask;

    for (int it = 0; it < 30; ++it) {
        if (!done) {
            if (!(a.div_patience != 0 && status == 3.0f)) {
                if (!warp_inside<MODEL>(w, px0, py0, S, half, a.W, a.H)) {
                    if (!a.roi_enabled || status > -2.5f) status = -1.0f;
                }
            }
            if (it >= a.iterations || fabsf(status) > 0.5f) done = true;
        }
        if (__all_sync(kFullMask, done)) break;
        float s[N];
#pragma unroll
        for (int k = 0; k < N; ++k) s[k] = 0.0f;
        if (!done) {
            float2 acc[N];
#pragma unroll
            for (int k = 0; k < N; ++k) acc[k] = pair(0.0f);
            for (int ph = 0; ph < phases; ++ph) {
                // Runs of the two slots: column q mod S, segment q / S.
                const int qa = (2 * ph) * LANES + glane, qb = qa + LANES;
                const int colA = qa % S, colB = qb % S;
                const int r0A = (qa / S) * L, r0B = (qb / S) * L;
                Slot A, B;
                A.rows = qa < runs ? min(L, S - r0A) : 0;
                B.rows = qb < runs ? min(L, S - r0B) : 0;
                A.ridx = (py0 + r0A) * a.W + px0 + colA;
                B.ridx = (py0 + r0B) * a.W + px0 + colB;
                A.fresh = B.fresh = true;
                const float2 lx = make_float2((float)colA - half, (float)colB - half);
                float2 ly = make_float2((float)r0A - half, (float)r0B - half);
                // Window-local position of a run's first sample (the window's
                // pixel (c, r) sits at local (c, r)) and its step per row.
                Walk wk;
                float2 dx = pair(w.t0), dy = pair(w.t1);
                if (MODEL != kModelTranslation) {
                    dx = add2(dx, fma2(pair(w.l0), lx, mul2(pair(w.l1), ly)));
                    dy = add2(dy, fma2(pair(w.l2), lx, mul2(pair(w.l3), ly)));
                }
                wk.q0x = add2(make_float2((float)colA, (float)colB), dx);
                wk.q0y = add2(make_float2((float)r0A, (float)r0B), dy);
                wk.sx = pair(MODEL == kModelTranslation ? 0.0f : w.l1);
                wk.sy = pair(MODEL == kModelTranslation ? 1.0f : 1.0f + w.l3);
                wk.qx = wk.q0x;
                wk.qy = wk.q0y;
                wk.fx = make_float2(floorf(wk.qx.x), floorf(wk.qx.y));
                wk.fy = make_float2(floorf(wk.qy.x), floorf(wk.qy.y));
                A.ix = (int)wk.fx.x; A.iy = (int)wk.fy.x;
                B.ix = (int)wk.fx.y; B.iy = (int)wk.fy.y;
                const int wA = GAUSS ? r0A * S + colA : 0, wB = GAUSS ? r0B * S + colB : 0;
                float2 ring[5][4];
#pragma unroll
                for (int j = 0; j < 5; ++j)
#pragma unroll
                    for (int i = 0; i < 4; ++i) ring[j][i] = pair(0.0f);
                float kf = 0.0f;
                for (int k = 0; k < L; k += 5) {
                    fast_step<MODEL, GAUSS, N, 0>(acc, ring, A, B, wk, kf, k, a, lx, ly, px0, py0, wA, wB, ref_mean);
                    fast_step<MODEL, GAUSS, N, 1>(acc, ring, A, B, wk, kf + 1.0f, k + 1, a, lx, ly, px0, py0, wA, wB,
                                                  ref_mean);
                    fast_step<MODEL, GAUSS, N, 2>(acc, ring, A, B, wk, kf + 2.0f, k + 2, a, lx, ly, px0, py0, wA, wB,
                                                  ref_mean);
                    fast_step<MODEL, GAUSS, N, 3>(acc, ring, A, B, wk, kf + 3.0f, k + 3, a, lx, ly, px0, py0, wA, wB,
                                                  ref_mean);
                    fast_step<MODEL, GAUSS, N, 4>(acc, ring, A, B, wk, kf + 4.0f, k + 4, a, lx, ly, px0, py0, wA, wB,
                                                  ref_mean);
                    kf += 5.0f;
                }
            }
#pragma unroll
            for (int k = 0; k < N; ++k) s[k] = acc[k].x + acc[k].y;
        }
        reduce_warp<LANES, N>(s, lane_in_warp);
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
        float4 *o = reinterpret_cast<float4 *>(a.state + (size_t)sidx * state_stride(MODEL));
        o[0] = make_float4(w.t0, w.l0, w.l1, w.t1);
        o[1] = make_float4(w.l2, w.l3, final_status, iters);
    }
}

template <int MODEL, int LANES, bool GAUSS>
__global__ void __launch_bounds__(128, GBDIC_FAST_MIN_BLOCKS) icgn_fast_kernel(SolveArgs a) {
    constexpr int kGroups = 32 / LANES;
    const int tid = threadIdx.x;
    const int lane_in_warp = tid & 31;
    const int glane = tid % LANES;
    const int group_in_unit = lane_in_warp / LANES;
    const long long unit = (long long)blockIdx.x * 4 + tid / 32;
    for (;;) {
        int base;
        if (a.persistent) {
            int v = 0;
            if (lane_in_warp == 0) v = (int)atomicAdd(a.work_counter, (unsigned)kGroups);
            base = __shfl_sync(kFullMask, v, 0);
        } else {
            base = unit * kGroups < (long long)a.count ? (int)(unit * kGroups) : a.count;
        }
        if (base >= a.count) break;
        solve_group_fast<MODEL, LANES, GAUSS>(a, base + group_in_unit, glane, lane_in_warp);
        if (!a.persistent) break;
    }
}

template <int MODEL, int LANES>
cudaError_t launch_lanes(const SolveArgs &a, bool gauss, int grid, cudaStream_t stream, int *occupancy_only) {
    if (occupancy_only) {
        int blocks = 0;
        if (gauss)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_fast_kernel<MODEL, LANES, true>, 128, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_fast_kernel<MODEL, LANES, false>, 128, 0);
        *occupancy_only = blocks;
        return cudaSuccess;
    }
    if (gauss) icgn_fast_kernel<MODEL, LANES, true><<<grid, 128, 0, stream>>>(a);
    else icgn_fast_kernel<MODEL, LANES, false><<<grid, 128, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_icgn_fast(const SolveArgs &a, int model, int lanes, bool gauss, int grid, cudaStream_t stream,
                             int *occupancy_only) {
    if (!icgn_fast_supported(model, kInterpBspline, lanes)) return cudaErrorInvalidValue;
    if (!occupancy_only && (a.fast_segments < 1 || a.fast_segments > a.S)) return cudaErrorInvalidValue;
    if (model == kModelAffine)
        return lanes == 16 ? launch_lanes<kModelAffine, 16>(a, gauss, grid, stream, occupancy_only)
                           : launch_lanes<kModelAffine, 32>(a, gauss, grid, stream, occupancy_only);
    return lanes == 16 ? launch_lanes<kModelTranslation, 16>(a, gauss, grid, stream, occupancy_only)
                       : launch_lanes<kModelTranslation, 32>(a, gauss, grid, stream, occupancy_only);
}

}  // namespace gbdic
