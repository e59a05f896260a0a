// Quadratic reference preparation by window rows (reference:
// wgpu_backend.py:_reference_arrays, 589-823, quadratic shape function; the
// per-window path for every other configuration is refprep.cu's
// subset_prep_kernel, whose moment layout and finishing steps this follows).
//
// With uniform weights, or Gaussian weights w = wx(x) wy(y), each moment of
// a window is a double sum
//     sum_rows sum_cols w Q(X, Y) x^a y^b
// of a pixel quantity Q (I, I^2, gx I, gy I, gx, gy, gx^2, gx gy, gy^2)
// times window-local monomials.  The windows of one grid row share their
// rows and overlapping windows share columns, so
//   1. quadratic_row_moments_kernel, one CTA per segment of a window row:
//      a. column sums V[Q, b](X) = sum_rows wy Q(X, Y) y^b, one thread per
//         column, 29 Kahan sums over the S rows (packed FP32 pairs),
//         into shared memory as head + tail;
//      b. window sums sum_cols wx x^a V[Q, b] for a = 0 .. 4 - b (or 2 - b),
//         one (column sum, window) item per thread, Kahan sums in FP32
//         pairs of powers of x, into shared memory as head + tail;
//      c. per window: the moments of f = I - mean from those of I by
//         expanding the mean (sum (I - m) Q = sum I Q - m sum Q, carried in
//         double-float), rounded to binary32 in subset_prep_kernel's order
//         and written with the mean to a [moment][window] buffer;
//   2. quadratic_finish_kernel, one window per thread: the Jacobi-scaled
//      12x12 Cholesky inverse in binary64 on a packed triangle in shared
//      memory (the factor, L^-1 and L^-T L^-1 in place), validity, metadata
//      and the inverse rows (written by the warp, one window at a time).
// About S x 29 products per column and S x 71 per window replace the
// S^2 x 70 of the per-window sums, and one thread per window keeps every
// lane of the FP64 pipe busy instead of the 12-24 of a warp per window.
#include <algorithm>
#include <cfloat>

#include "gbdic_common.cuh"
#include "gbdic_kernels.h"

namespace gbdic {

namespace {

constexpr int kSlots = 29;        // column sums per column
constexpr int kWindowSums = 71;   // window sums (x^a of each column sum)
constexpr int kMoments = 71;      // binary32 outputs per window: 70 moments + mean
constexpr int kRowWindows = 16;   // windows per CTA (at most)
constexpr int kRowMaxCols = 256;  // columns per CTA (one thread each)
constexpr int kFinishThreads = 32;   // one warp per CTA: 20.6 KB of triangles, 11 CTAs per SM
constexpr int kN = 12, kTri = kN * (kN + 1) / 2;

// Column sums ("slots") in the order phase a produces them, FP32 pairs
// (0,1) (2,3) ...: quantity and power of y.  Quantities: 0 I, 1 I^2, 2 gx I,
// 3 gy I, 4 gx, 5 gy, 6 gx^2, 7 gx gy, 8 gy^2.
//   pairs: (I, I^2) (gxI, gyI) gxI(y, y^2) gyI(y, y^2) (gx, gy) gx(y, y^2)
//          gy(y, y^2) (gx^2, gxgy) gx^2(y, y^2) gx^2(y^3, y^4) gxgy(y, y^2)
//          gxgy(y^3, y^4) gy^2(y, y^2) gy^2(y^3, y^4) (gy^2, -)
__host__ __device__ constexpr int slot_quantity(int s) {
    constexpr int q[kSlots] = {0, 1, 2, 3, 2, 2, 3, 3, 4, 5, 4, 4, 5, 5, 6, 7, 6, 6, 6, 6, 7, 7, 7, 7, 8, 8, 8, 8, 8};
    return q[s];
}
__host__ __device__ constexpr int slot_power(int s) {
    constexpr int b[kSlots] = {0, 0, 0, 0, 1, 2, 1, 2, 0, 0, 1, 2, 1, 2, 0, 0, 1, 2, 3, 4, 1, 2, 3, 4, 1, 2, 3, 4, 0};
    return b[s];
}
// Highest power of x summed for a slot: the monomials of the moments it
// feeds (degree <= 2 for J^T f and sum J, <= 4 for the Hessian).
__host__ __device__ constexpr int slot_degree(int s) {
    return (slot_quantity(s) < 2 ? 0 : slot_quantity(s) < 6 ? 2 : 4) - slot_power(s);
}
__host__ __device__ constexpr int slot_base(int s) {
    int base = 0;
    for (int k = 0; k < s; ++k) base += slot_degree(k) + 1;
    return base;
}
__host__ __device__ constexpr int slot_of(int quantity, int b) {
    for (int s = 0; s < kSlots; ++s)
        if (slot_quantity(s) == quantity && slot_power(s) == b) return s;
    return -1;
}
// Window sum of quantity Q times x^a y^b.
__host__ __device__ constexpr int window_sum(int quantity, int a, int b) { return slot_base(slot_of(quantity, b)) + a; }
static_assert(slot_base(kSlots - 1) + slot_degree(kSlots - 1) + 1 == kWindowSums, "window sums");
constexpr int kSumI = window_sum(0, 0, 0);  // sum I, for the window mean

__constant__ int c_slot_degree[kSlots] = {
    slot_degree(0),  slot_degree(1),  slot_degree(2),  slot_degree(3),  slot_degree(4),  slot_degree(5),
    slot_degree(6),  slot_degree(7),  slot_degree(8),  slot_degree(9),  slot_degree(10), slot_degree(11),
    slot_degree(12), slot_degree(13), slot_degree(14), slot_degree(15), slot_degree(16), slot_degree(17),
    slot_degree(18), slot_degree(19), slot_degree(20), slot_degree(21), slot_degree(22), slot_degree(23),
    slot_degree(24), slot_degree(25), slot_degree(26), slot_degree(27), slot_degree(28)};
__constant__ int c_slot_base[kSlots] = {
    slot_base(0),  slot_base(1),  slot_base(2),  slot_base(3),  slot_base(4),  slot_base(5),  slot_base(6),
    slot_base(7),  slot_base(8),  slot_base(9),  slot_base(10), slot_base(11), slot_base(12), slot_base(13),
    slot_base(14), slot_base(15), slot_base(16), slot_base(17), slot_base(18), slot_base(19), slot_base(20),
    slot_base(21), slot_base(22), slot_base(23), slot_base(24), slot_base(25), slot_base(26), slot_base(27),
    slot_base(28)};

// Column sums by decreasing degree, so that the items of a warp in the
// window-sum phase mostly share one degree.
__host__ __device__ constexpr int slot_order(int pos) {
    for (int d = 4; d >= 0; --d)
        for (int s = 0; s < kSlots; ++s)
            if (slot_degree(s) == d && pos-- == 0) return s;
    return -1;
}
__constant__ int c_slot_order[kSlots] = {
    slot_order(0),  slot_order(1),  slot_order(2),  slot_order(3),  slot_order(4),  slot_order(5),
    slot_order(6),  slot_order(7),  slot_order(8),  slot_order(9),  slot_order(10), slot_order(11),
    slot_order(12), slot_order(13), slot_order(14), slot_order(15), slot_order(16), slot_order(17),
    slot_order(18), slot_order(19), slot_order(20), slot_order(21), slot_order(22), slot_order(23),
    slot_order(24), slot_order(25), slot_order(26), slot_order(27), slot_order(28)};

// Quadratic Jacobian column q = (gradient block, monomial m_i), monomials
// (1, x, y, x^2/2, xy, y^2/2): [gx m0..m2, gy m0..m2, gx m3..m5, gy m3..m5].
__host__ __device__ constexpr int column_block(int q) { return (q < 3 || (q >= 6 && q < 9)) ? 0 : 1; }
__host__ __device__ constexpr int column_monomial(int q) { return q < 3 ? q : (q < 6 ? q - 3 : (q < 9 ? q - 3 : q - 6)); }
__host__ __device__ constexpr int mono_x(int i) { return i == 1 ? 1 : i == 3 ? 2 : i == 4 ? 1 : 0; }
__host__ __device__ constexpr int mono_y(int i) { return i == 2 ? 1 : i == 4 ? 1 : i == 5 ? 2 : 0; }
__host__ __device__ constexpr float mono_scale(int i) { return i == 3 || i == 5 ? 0.5f : 1.0f; }
// index of x^a y^b among the 15 monomials of degree <= 4
__host__ __device__ constexpr int degree4_index(int a, int b) { return (a + b) * (a + b + 1) / 2 + b; }
// packed lower triangle, i >= j
__host__ __device__ constexpr int tri(int i, int j) { return i * (i + 1) / 2 + j; }
// (a, b) of the monomial with degree4_index k
__host__ __device__ constexpr int degree4_b(int k) {
    int d = 0;
    while ((d + 1) * (d + 2) / 2 <= k) ++d;
    return k - d * (d + 1) / 2;
}
__host__ __device__ constexpr int degree4_a(int k) {
    int d = 0;
    while ((d + 1) * (d + 2) / 2 <= k) ++d;
    return d - degree4_b(k);
}

// Binary32 moment k of the per-window layout (0 f^2; 1-6 gx f m; 7-12 gy f m;
// 13-18 gx m; 19-24 gy m; 25-69 gx^2, gx gy, gy^2 times the monomials of
// degree <= 4; 70 the mean) from the window sums: scale x (primary -
// mean x secondary), secondary -1 for none.  Moment 0 is
// sum I^2 - 2 m sum I + m^2 N (primary sum I^2, secondary sum I).
__host__ __device__ constexpr int first_order_quantity(int k) { return 2 + (k - 1) / 6; }  // gxI gyI gx gy
__host__ __device__ constexpr int moment_primary(int k) {
    return k == 0    ? window_sum(1, 0, 0)
           : k < 25  ? window_sum(first_order_quantity(k), mono_x((k - 1) % 6), mono_y((k - 1) % 6))
           : k < 70  ? window_sum(6 + (k - 25) / 15, degree4_a((k - 25) % 15), degree4_b((k - 25) % 15))
                     : window_sum(0, 0, 0);
}
__host__ __device__ constexpr int moment_secondary(int k) {
    return k == 0 ? window_sum(0, 0, 0)
           : k < 13 ? window_sum(first_order_quantity(k) + 2, mono_x((k - 1) % 6), mono_y((k - 1) % 6))
                    : -1;
}
__host__ __device__ constexpr float moment_scale(int k) { return k >= 1 && k < 25 ? mono_scale((k - 1) % 6) : 1.0f; }

#define GBDIC_TABLE10(f, b) f(b), f(b + 1), f(b + 2), f(b + 3), f(b + 4), f(b + 5), f(b + 6), f(b + 7), f(b + 8), f(b + 9)
#define GBDIC_TABLE71(f)                                                                                        \
    GBDIC_TABLE10(f, 0), GBDIC_TABLE10(f, 10), GBDIC_TABLE10(f, 20), GBDIC_TABLE10(f, 30), GBDIC_TABLE10(f, 40), \
        GBDIC_TABLE10(f, 50), GBDIC_TABLE10(f, 60), f(70)
__constant__ int c_moment_primary[kMoments] = {GBDIC_TABLE71(moment_primary)};
__constant__ int c_moment_secondary[kMoments] = {GBDIC_TABLE71(moment_secondary)};
__constant__ float c_moment_scale[kMoments] = {GBDIC_TABLE71(moment_scale)};
#undef GBDIC_TABLE71
#undef GBDIC_TABLE10

// Double-float value hi + lo.  Every operation is an explicit _rn
// intrinsic, so contraction cannot merge the error-free transforms.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_normalise(float hi, float lo) {
    const float s = __fadd_rn(hi, lo);
    return {s, __fsub_rn(lo, __fsub_rn(s, hi))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bp = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b.hi, bp));
    return df_normalise(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF df_scale(DF a, float b) {
    const float p = __fmul_rn(a.hi, b);
    const float e = __fmaf_rn(a.lo, b, __fmaf_rn(a.hi, b, -p));
    return df_normalise(p, e);
}
__device__ __forceinline__ float df_round(DF a) { return __fadd_rn(a.hi, a.lo); }

__device__ __forceinline__ void kahan_pair(float2 &s, float2 &c, float2 v) {
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const float2 y = __ffma2_rn(c, m1, v);
    const float2 t = __fadd2_rn(s, y);
    c = __ffma2_rn(y, m1, __ffma2_rn(s, m1, t));
    s = t;
}

// Window sums of one column sum (head, tail) times wx x^0 .. wx x^D over the
// S columns of a window: Kahan sums in FP32 pairs (x^0, x^1) (x^2, x^3)
// (x^4, -), each term fl(head p + tail p) with p = wx x^a from the column's
// power table (xpow03 = wx (1, x, x^2, x^3), xpow4 = wx x^4).  Written as
// head s, tail -c.
template <int D>
__device__ __forceinline__ void window_sums(const float2 *col, const float4 *xpow03, const float *xpow4, int S,
                                            float2 *out) {
    constexpr int P = D / 2 + 1;
    float2 s[P], c[P];
#pragma unroll
    for (int p = 0; p < P; ++p) { s[p] = make_float2(0.0f, 0.0f); c[p] = make_float2(0.0f, 0.0f); }
    for (int j = 0; j < S; ++j) {
        const float2 v = col[j];
        const float4 x = xpow03[j];
        const float2 hi = make_float2(v.x, v.x), lo = make_float2(v.y, v.y);
        const float2 pw[3] = {make_float2(x.x, x.y), make_float2(x.z, x.w),
                              make_float2(D >= 4 ? xpow4[j] : 0.0f, 0.0f)};
#pragma unroll
        for (int p = 0; p < P; ++p) kahan_pair(s[p], c[p], __ffma2_rn(lo, pw[p], __fmul2_rn(hi, pw[p])));
    }
#pragma unroll
    for (int k = 0; k <= D; ++k)
        out[k] = (k & 1) ? make_float2(s[k / 2].y, -c[k / 2].y) : make_float2(s[k / 2].x, -c[k / 2].x);
}

// 96 registers: three 192-thread CTAs per SM (the shared-memory limit as well).
template <bool GAUSS>
__global__ void __maxnreg__(96) quadratic_row_moments_kernel(PrepArgs a, int windows_per_cta, int pitch) {
    extern __shared__ float2 s_col[];  // [slot][pitch] column sums (head, tail)
    __shared__ float2 s_win[kRowWindows][kWindowSums];
    __shared__ float4 s_xpow03[kRowMaxCols];  // wx (1, x, x^2, x^3) of window column j
    __shared__ float s_xpow4[kRowMaxCols];    // wx x^4
    __shared__ float s_wy[kRowMaxCols];       // wy of window row r
    const int tid = threadIdx.x;
    const int ix0 = blockIdx.x * windows_per_cta, iy = blockIdx.y;
    const int nw = min(windows_per_cta, a.grid_w - ix0);
    const int S = a.S, st = a.stride;
    const int cols = (nw - 1) * st + S;
    const int gx0 = ix0 * st, gy0 = iy * st;
    const float half = 0.5f * ((float)S - 1.0f);
    if (GAUSS && tid < S) s_wy[tid] = a.axis_weights[tid];
    if (GAUSS) __syncthreads();

    // a. column sums over the window row's S image rows
    if (tid < cols) {
        float2 s[15], c[15];
#pragma unroll
        for (int k = 0; k < 15; ++k) { s[k] = make_float2(0.0f, 0.0f); c[k] = make_float2(0.0f, 0.0f); }
        const float4 *src = a.plane + (size_t)gy0 * a.W + gx0 + tid;
#pragma unroll 2
        for (int r = 0; r < S; ++r) {
            const float4 v = src[(size_t)r * a.W];
            const float y = (float)r - half, y2 = y * y;
            float2 y12 = make_float2(y, y2), y34 = make_float2(y2 * y, y2 * y2);
            const float I = v.x, gx = v.y, gy = v.z;
            const float2 gI = __fmul2_rn(make_float2(gx, gy), make_float2(I, I));
            const float2 G01 = __fmul2_rn(make_float2(gx, gx), make_float2(gx, gy));
            const float G2 = gy * gy;
            // y^0 terms times wy; wy folded into the powers of y for the others
            float2 t0 = make_float2(I, I * I), t1 = gI, t4 = make_float2(gx, gy), t7 = G01,
                   t14 = make_float2(G2, 0.0f);
            if (GAUSS) {
                const float2 wy = make_float2(s_wy[r], s_wy[r]);
                y12 = __fmul2_rn(y12, wy);
                y34 = __fmul2_rn(y34, wy);
                t0 = __fmul2_rn(t0, wy);
                t1 = __fmul2_rn(t1, wy);
                t4 = __fmul2_rn(t4, wy);
                t7 = __fmul2_rn(t7, wy);
                t14 = __fmul2_rn(t14, wy);
            }
            kahan_pair(s[0], c[0], t0);
            kahan_pair(s[1], c[1], t1);
            kahan_pair(s[2], c[2], __fmul2_rn(make_float2(gI.x, gI.x), y12));
            kahan_pair(s[3], c[3], __fmul2_rn(make_float2(gI.y, gI.y), y12));
            kahan_pair(s[4], c[4], t4);
            kahan_pair(s[5], c[5], __fmul2_rn(make_float2(gx, gx), y12));
            kahan_pair(s[6], c[6], __fmul2_rn(make_float2(gy, gy), y12));
            kahan_pair(s[7], c[7], t7);
            kahan_pair(s[8], c[8], __fmul2_rn(make_float2(G01.x, G01.x), y12));
            kahan_pair(s[9], c[9], __fmul2_rn(make_float2(G01.x, G01.x), y34));
            kahan_pair(s[10], c[10], __fmul2_rn(make_float2(G01.y, G01.y), y12));
            kahan_pair(s[11], c[11], __fmul2_rn(make_float2(G01.y, G01.y), y34));
            kahan_pair(s[12], c[12], __fmul2_rn(make_float2(G2, G2), y12));
            kahan_pair(s[13], c[13], __fmul2_rn(make_float2(G2, G2), y34));
            kahan_pair(s[14], c[14], t14);
        }
        // a Kahan sum is s - c: stored as head s, tail -c
#pragma unroll
        for (int k = 0; k < 15; ++k) {
            s_col[(2 * k) * pitch + tid] = make_float2(s[k].x, -c[k].x);
            if (2 * k + 1 < kSlots) s_col[(2 * k + 1) * pitch + tid] = make_float2(s[k].y, -c[k].y);
        }
    }
    if (tid < S) {
        const float x = (float)tid - half, x2 = x * x;
        if (GAUSS) {
            const float wx = a.axis_weights[tid];
            s_xpow03[tid] = make_float4(wx, wx * x, wx * x2, wx * (x2 * x));
            s_xpow4[tid] = wx * (x2 * x2);
        } else {
            s_xpow03[tid] = make_float4(1.0f, x, x2, x2 * x);
            s_xpow4[tid] = x2 * x2;
        }
    }
    __syncthreads();

    // b. window sums: item (column sum, window), column sums by decreasing
    // degree, windows fastest
    for (int item = tid; item < nw * kSlots; item += blockDim.x) {
        const int pos = item / nw, w = item - pos * nw;
        const int slot = c_slot_order[pos];
        const float2 *col = s_col + slot * pitch + w * st;
        float2 *out = &s_win[w][c_slot_base[slot]];
        switch (c_slot_degree[slot]) {
        case 0: window_sums<0>(col, s_xpow03, s_xpow4, S, out); break;
        case 1: window_sums<1>(col, s_xpow03, s_xpow4, S, out); break;
        case 2: window_sums<2>(col, s_xpow03, s_xpow4, S, out); break;
        case 3: window_sums<3>(col, s_xpow03, s_xpow4, S, out); break;
        default: window_sums<4>(col, s_xpow03, s_xpow4, S, out); break;
        }
    }
    __syncthreads();

    // c. the window means, then the binary32 moments in the order of the
    // per-window path, one (moment, window) item per thread (windows fastest,
    // so the stores to the [moment][window] buffer are contiguous)
    __shared__ float s_mean[kRowWindows];
    if (tid < nw) {
        const float2 sI = s_win[tid][kSumI];
        s_mean[tid] = df_round(DF{sI.x, sI.y}) / a.weight_sum;
    }
    __syncthreads();
    const size_t idx0 = (size_t)iy * a.grid_w + ix0;
    for (int item = tid; item < nw * kMoments; item += blockDim.x) {
        const int k = item / nw, w = item - k * nw;
        const float mean = s_mean[w];
        const float2 p = s_win[w][c_moment_primary[k]];
        const int sec = c_moment_secondary[k];
        float v;
        if (k == 70) {
            v = mean;
        } else if (k == 0) {
            // sum (I - m)^2 = sum I^2 - 2 m sum I + m^2 N
            const float2 q = s_win[w][sec];
            const float mm = __fmul_rn(mean, mean);
            const DF m2{mm, __fmaf_rn(mean, mean, -mm)};
            const DF e = df_add(df_add(DF{p.x, p.y}, df_scale(DF{q.x, q.y}, -2.0f * mean)), df_scale(m2, a.weight_sum));
            v = df_round(e);
        } else if (sec >= 0) {
            const float2 q = s_win[w][sec];
            v = c_moment_scale[k] * df_round(df_add(DF{p.x, p.y}, df_scale(DF{q.x, q.y}, -mean)));
        } else {
            v = c_moment_scale[k] * df_round(DF{p.x, p.y});
        }
        a.moments[(size_t)k * a.count + idx0 + w] = v;
    }
}

// 168 registers (a few spilled): the shared triangles, not the registers,
// bound the resident warps (0.36 -> 0.30 ms on the UHD S41/s10 grid).
__global__ void __maxnreg__(168) quadratic_finish_kernel(PrepArgs a) {
    extern __shared__ double s_tri[];  // element e of thread t at e * (blockDim + 1) + t
    const int tid = threadIdx.x, lane = tid & 31;
    const int ld = blockDim.x + 1;
    const int idx = blockIdx.x * blockDim.x + tid;
    const bool live = idx < a.count;
    const size_t n = (size_t)a.count;
    const float *t = a.moments + (live ? idx : 0);
    double *T = s_tri + tid;
    const float energy = live ? t[0] : 0.0f;

    // Hessian from the monomial moments, Jacobi scaling (diagonal first)
    bool ok = live;
    double d[kN];
#pragma unroll
    for (int i = 0; i < kN; ++i) {
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            const int bi = column_block(i), bj = column_block(j), mi = column_monomial(i), mj = column_monomial(j);
            const int k = 25 + (bi + bj) * 15 + degree4_index(mono_x(mi) + mono_x(mj), mono_y(mi) + mono_y(mj));
            const float v = live ? mono_scale(mi) * mono_scale(mj) * t[k * n] : 0.0f;
            T[tri(i, j) * ld] = (double)v;
        }
        const double aii = T[tri(i, i) * ld];
        ok = ok && aii > 0.0;
        d[i] = aii > 0.0 ? rsqrt(aii) : 0.0;
    }
#pragma unroll
    for (int i = 0; i < kN; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) T[tri(i, j) * ld] = T[tri(i, j) * ld] * d[i] * d[j];

    // Cholesky factor in place; r[k] = 1 / L_kk
    double r[kN];
#pragma unroll
    for (int k = 0; k < kN; ++k) {
        const double pivot = T[tri(k, k) * ld];
        ok = ok && pivot > 0.0;
        r[k] = pivot > 0.0 ? rsqrt(pivot) : 0.0;
        T[tri(k, k) * ld] = pivot * r[k];
#pragma unroll
        for (int i = k + 1; i < kN; ++i) T[tri(i, k) * ld] = T[tri(i, k) * ld] * r[k];
#pragma unroll
        for (int i = k + 1; i < kN; ++i) {
            const double lik = T[tri(i, k) * ld];
#pragma unroll
            for (int j = k + 1; j <= i; ++j) T[tri(i, j) * ld] = T[tri(i, j) * ld] - lik * T[tri(j, k) * ld];
        }
    }
    // L^-1 in place, column by column: X_jj = r_j, X_ij = -(sum_{k=j}^{i-1} L_ik X_kj) r_i
#pragma unroll
    for (int j = 0; j < kN; ++j) {
        T[tri(j, j) * ld] = r[j];
#pragma unroll
        for (int i = j + 1; i < kN; ++i) {
            double acc = 0.0;
#pragma unroll
            for (int k = j; k < i; ++k) acc = acc + T[tri(i, k) * ld] * T[tri(k, j) * ld];
            T[tri(i, j) * ld] = -acc * r[i];
        }
    }
    // A^-1 = D L^-T L^-1 D in place, row by row: (i, j) = sum_{k>=i} X_ki X_kj,
    // stored rounded to binary32 in the low word of its slot (read back by the
    // warp's row writes below); a value beyond the binary32 range rounds to
    // infinity and makes the window invalid
    bool finite = true;
#pragma unroll
    for (int i = 0; i < kN; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            double acc = 0.0;
#pragma unroll
            for (int k = i; k < kN; ++k) acc = acc + T[tri(k, i) * ld] * T[tri(k, j) * ld];
            const float v = (float)(acc * d[i] * d[j]);
            finite = finite && isfinite(v);
            reinterpret_cast<float *>(&T[tri(i, j) * ld])[0] = v;
        }
    const bool valid = live && energy > 1e-12f && ok && finite;
    const bool selected = live && (a.selected == nullptr || a.selected[idx] != 0);

    if (live) {
        float *md = a.meta + (size_t)idx * meta_stride(kModelQuadratic);
        md[0] = sqrtf(fmaxf(energy, 0.0f));
        md[1] = selected ? (valid ? 1.0f : 0.0f) : -3.0f;
#pragma unroll
        for (int q = 0; q < kN; ++q) {
            md[2 + q] = t[(1 + column_block(q) * 6 + column_monomial(q)) * n];
            md[2 + kN + q] = t[(13 + column_block(q) * 6 + column_monomial(q)) * n];
        }
        md[2 + 2 * kN] = t[70 * n];
        md[3 + 2 * kN] = a.weight_sum;
        a.admissible[idx] = valid ? 1 : 0;
    }
    const unsigned counted = __ballot_sync(kFullMask, valid && selected);
    if (lane == 0 && counted) atomicAdd(a.valid_count, (unsigned)__popc(counted));

    // inverse rows, one window of the warp at a time (coalesced rows of 144)
    __syncwarp();
    const int warp0 = tid - lane;
    for (int w = 0; w < 32; ++w) {
        const int widx = blockIdx.x * blockDim.x + warp0 + w;
        const bool wvalid = __shfl_sync(kFullMask, valid, w);
        if (widx >= a.count) break;  // warp-uniform
        float *inv = a.inv + (size_t)widx * kN * kN;
        for (int e = lane; e < kN * kN; e += 32) {
            const int row = e / kN, colm = e - row * kN;
            const int hi = row > colm ? row : colm, lo = row > colm ? colm : row;
            inv[e] = wvalid ? reinterpret_cast<const float *>(&s_tri[tri(hi, lo) * ld + warp0 + w])[0] : 0.0f;
        }
    }
}

}  // namespace

// GBDIC_QUAD_ROW_PREP=0 (a -D tuning macro) keeps every configuration on
// the per-window path, for comparisons.
#ifndef GBDIC_QUAD_ROW_PREP
#define GBDIC_QUAD_ROW_PREP 1
#endif

bool quadratic_row_prep_supported(int model, int gaussian_weighting, int S, int stride, int grid_h) {
    return GBDIC_QUAD_ROW_PREP && model == kModelQuadratic && (gaussian_weighting == 0 || gaussian_weighting == 1) &&
           stride < S && S <= kRowMaxCols && grid_h <= 65535;
}

size_t quadratic_row_prep_moment_floats(int count) { return (size_t)kMoments * (size_t)count; }

cudaError_t launch_quadratic_row_prep(const PrepArgs &a, cudaStream_t stream) {
    if (!quadratic_row_prep_supported(a.model, a.gaussian_weighting, a.S, a.stride, a.grid_h) || !a.moments)
        return cudaErrorInvalidValue;
    if (a.count <= 0) return cudaSuccess;
    const int wpc = std::min(kRowWindows, (kRowMaxCols - a.S) / a.stride + 1);
    const int pitch = (wpc - 1) * a.stride + a.S;
    const int threads = (pitch + 31) / 32 * 32;
    const size_t shared = (size_t)kSlots * pitch * sizeof(float2);
    const bool gauss = a.gaussian_weighting == 1;
    if (gauss && !a.axis_weights) return cudaErrorInvalidValue;
    auto kernel = gauss ? quadratic_row_moments_kernel<true> : quadratic_row_moments_kernel<false>;
    cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared);
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   (int)cudaSharedmemCarveoutMaxShared);
    if (err != cudaSuccess) return err;
    const dim3 grid((a.grid_w + wpc - 1) / wpc, a.grid_h);
    kernel<<<grid, threads, shared, stream>>>(a, wpc, pitch);
    const size_t tri_shared = (size_t)kTri * (kFinishThreads + 1) * sizeof(double);
    quadratic_finish_kernel<<<(a.count + kFinishThreads - 1) / kFinishThreads, kFinishThreads, tri_shared, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace gbdic
