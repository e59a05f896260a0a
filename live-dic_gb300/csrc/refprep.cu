// GPU reference preparation (reference: wgpu_backend.py:_reference_arrays,
// 544-823, and its browser GPU twin shaders/reference.wgsl:59-277).
//
// Stages, all on the engine stream:
//   1. gauss7      mirrored 7-tap sigma-one Gaussian (B-spline mode) or byte
//                  copy (direct modes) -> intensity plane (float32)
//   2. spline      exact recursive cubic B-spline prefilter, rows then
//                  columns: each line is split in 64-sample chunks; a chunk's
//                  causal pass starts 24 samples early (z^24 < 1e-13) and its
//                  anticausal pass 24 samples late, so chunks are independent
//                  threads; rows go through shared-memory tile transposes so
//                  that every pass reads and writes coalesced columns
//   3. gradients   [1,4,1]/6-smoothed central differences of the coefficients
//                  (B-spline) or central differences of the bytes -> plane
//   4. subsets     one warp per subset: Kahan-compensated binary32 moments of
//                  the weighted steepest-descent images, tree-combined with
//                  TwoSum, Jacobi-scaled Cholesky factor and inverse of the
//                  Hessian (binary32 for 6x6 and 2x2, binary64 for 12x12),
//                  metadata row and validity.
#include <cfloat>
#include <type_traits>

#include "gbdic_common.cuh"
#include "gbdic_kernels.h"

namespace gbdic {

namespace {

__constant__ float c_gauss[7];

constexpr int kTile = 32;

// ---------------------------------------------------------------- stage 1
__global__ void gauss7_kernel(const uint8_t *__restrict__ img, int W, int H, int pitch, int smooth,
                              float *__restrict__ out) {
    constexpr int R = 3, TW = 64, TH = 32, IW = TW + 2 * R, IH = TH + 2 * R;
    __shared__ float s_in[IH * IW];
    __shared__ float s_x[IH * TW];
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH, tid = threadIdx.x;
    if (!smooth) {
        for (int i = tid; i < TW * TH; i += blockDim.x) {
            const int x = x0 + i % TW, y = y0 + i / TW;
            if (x < W && y < H) out[(size_t)y * W + x] = (float)img[(size_t)y * pitch + x];
        }
        return;
    }
    for (int i = tid; i < IH * IW; i += blockDim.x) {
        const int r = i / IW, c = i % IW;
        s_in[i] = (float)img[(size_t)mirror_clamp(y0 + r - R, H) * pitch + mirror_clamp(x0 + c - R, W)];
    }
    __syncthreads();
    for (int i = tid; i < IH * TW; i += blockDim.x) {
        const int r = i / TW, c = i % TW;
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 7; ++k) acc = fmaf(c_gauss[k], s_in[r * IW + c + k], acc);
        s_x[i] = acc;
    }
    __syncthreads();
    for (int i = tid; i < TH * TW; i += blockDim.x) {
        const int r = i / TW, c = i % TW, x = x0 + c, y = y0 + r;
        if (x >= W || y >= H) continue;
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 7; ++k) acc = fmaf(c_gauss[k], s_x[(r + k) * TW + c], acc);
        out[(size_t)y * W + x] = acc;
    }
}

// ---------------------------------------------------------------- stage 2
// out[c][r] = in[r][c] for an (rows x cols) input.
__global__ void transpose_kernel(const float *__restrict__ in, int rows, int cols, float *__restrict__ out) {
    __shared__ float tile[kTile][kTile + 1];
    const int bx = blockIdx.x * kTile, by = blockIdx.y * kTile;
    for (int j = threadIdx.y; j < kTile; j += blockDim.y) {
        const int r = by + j, c = bx + threadIdx.x;
        if (r < rows && c < cols) tile[j][threadIdx.x] = in[(size_t)r * cols + c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < kTile; j += blockDim.y) {
        const int c = bx + j, r = by + threadIdx.x;
        if (c < cols && r < rows) out[(size_t)c * rows + r] = tile[threadIdx.x][j];
    }
}

constexpr int kChunk = 64;
constexpr int kWarm = 24;

// Recursive cubic B-spline prefilter along the columns of an (n x cols)
// row-major array; thread = (column, chunk of kChunk rows).
__global__ void spline_columns_kernel(const float *__restrict__ in, int n, int cols, float *__restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = blockIdx.y * kChunk;
    if (c >= cols || a >= n || n < 2) return;
    const float z = -0.26794919243112270f;  // sqrt(3) - 2
    const float gain = 6.0f;                // (1 - z)(1 - 1/z)
    const int b = min(a + kChunk, n);
    const int e = min(b + kWarm, n);
    // causal results are kept for [a0, e); a0 <= n - 2 so that the exact
    // anticausal start value, which needs c+[n-2], is always available
    const int a0 = a > n - 2 ? n - 2 : a;
    const int s = a0 - kWarm > 0 ? a0 - kWarm : 0;
    float cp[kChunk + kWarm + 1];
    float prev;
    int k;
    if (s == 0) {
        const int horizon = n < 21 ? n : 21;
        float acc = 0.0f, power = 1.0f;
        for (int i = 0; i < horizon; ++i) {
            acc = fmaf(gain * in[(size_t)i * cols + c], power, acc);
            power = power * z;
        }
        prev = acc;
        if (a0 == 0) cp[0] = prev;
        k = 1;
    } else {
        prev = 0.0f;
        k = s;
    }
    for (; k < e; ++k) {
        prev = fmaf(z, prev, gain * in[(size_t)k * cols + c]);
        if (k >= a0) cp[k - a0] = prev;
    }
    float next;
    int j;
    if (e == n) {
        next = (z / (z * z - 1.0f)) * fmaf(z, cp[n - 2 - a0], cp[n - 1 - a0]);
        if (n - 1 >= a && n - 1 < b) out[(size_t)(n - 1) * cols + c] = next;
        j = n - 2;
    } else {
        next = 0.0f;
        j = e - 1;
    }
    for (; j >= a; --j) {
        next = z * (next - cp[j - a0]);
        if (j < b) out[(size_t)j * cols + c] = next;
    }
}

// ---------------------------------------------------------------- stage 3
__global__ void gradient_kernel(const float *__restrict__ intensity, const float *__restrict__ src,
                                int W, int H, int bspline, float4 *__restrict__ plane) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W || y >= H) return;
    const int xm = mirror_clamp(x - 1, W), xp = mirror_clamp(x + 1, W);
    const int ym = mirror_clamp(y - 1, H), yp = mirror_clamp(y + 1, H);
    const float *r0 = src + (size_t)ym * W, *r1 = src + (size_t)y * W, *r2 = src + (size_t)yp * W;
    float gx = 0.5f * (r1[xp] - r1[xm]);
    float gy = 0.5f * (r2[x] - r0[x]);
    if (bspline) {
        const float ga = 0.5f * (r0[xp] - r0[xm]), gb = 0.5f * (r2[xp] - r2[xm]);
        const float ha = 0.5f * (r2[xm] - r0[xm]), hb = 0.5f * (r2[xp] - r0[xp]);
        gx = fmaf(4.0f, gx, ga) + gb;
        gy = fmaf(4.0f, gy, ha) + hb;
        gx = gx / 6.0f;
        gy = gy / 6.0f;
    }
    plane[(size_t)y * W + x] = make_float4(intensity[(size_t)y * W + x], gx, gy, 0.0f);
}

// ---------------------------------------------------------------- stage 4
// Pair index (i <= j) -> position in the upper-triangular list.
__host__ __device__ constexpr int pair_index(int nm, int i, int j) {
    return i * nm - i * (i - 1) / 2 + (j - i);
}

// Quadratic Hessian moments by monomial: the products m_i m_j of the six
// monomials (1, x, y, x^2/2, xy, y^2/2) are c x^a y^b with a + b <= 4, 15
// distinct monomials, so each gradient product needs 15 sums instead of 21
// (c is 1, 1/2 or 1/4, exact).  x, y are integer or half-integer offsets, so
// every monomial of a window up to 41 px is an exact binary32 value.
__host__ __device__ constexpr int mono_exp_x(int i) { return i == 1 ? 1 : i == 3 ? 2 : i == 4 ? 1 : 0; }
__host__ __device__ constexpr int mono_exp_y(int i) { return i == 2 ? 1 : i == 4 ? 1 : i == 5 ? 2 : 0; }
// index of x^a y^b in (1, x, y, x^2, xy, y^2, x^3, x^2y, xy^2, y^3, x^4, ...)
__host__ __device__ constexpr int monomial_index(int a, int b) {
    return (a + b) * (a + b + 1) / 2 + b;
}
__host__ __device__ constexpr float pair_scale(int i, int j) {
    return (i == 3 || i == 5 ? 0.5f : 1.0f) * (j == 3 || j == 5 ? 0.5f : 1.0f);
}

template <int MODEL>
struct Moments {
    static constexpr int nm = MODEL == kModelQuadratic ? 6 : (MODEL == kModelTranslation ? 1 : 3);
    static constexpr int pairs = nm * (nm + 1) / 2;
    // Hessian sums per gradient product: pairs of monomials, or for the
    // quadratic model the 15 monomials of degree <= 4
    static constexpr int hess = MODEL == kModelQuadratic ? 15 : pairs;
    static constexpr int count = 1 + 4 * nm + 3 * hess;  // 8, 31, 70
};

// Position of Hessian entry (i <= j) among a gradient product's sums, and
// its scale.
template <int MODEL>
__host__ __device__ constexpr int hess_index(int i, int j) {
    return MODEL == kModelQuadratic ? monomial_index(mono_exp_x(i) + mono_exp_x(j), mono_exp_y(i) + mono_exp_y(j))
                                    : pair_index(Moments<MODEL>::nm, i, j);
}
template <int MODEL>
__host__ __device__ constexpr float hess_scale(int i, int j) {
    return MODEL == kModelQuadratic ? pair_scale(i, j) : 1.0f;
}


// All moments of one pixel in the order of Moments (f^2; gx f m; gy f m;
// gx m; gy m; then gx^2, gx gy, gy^2 times m_i m_j for i <= j), with
// compile-time indices so that a pass keeps only the values it sums.
template <int MODEL>
__device__ __forceinline__ void moment_values(float w, float f, float gx, float gy, const float *m,
                                              float (&out)[Moments<MODEL>::count]) {
    constexpr int nm = Moments<MODEL>::nm;
    out[0] = (w * f) * f;
    const float wgxf = (w * gx) * f, wgyf = (w * gy) * f, wgx = w * gx, wgy = w * gy;
#pragma unroll
    for (int q = 0; q < nm; ++q) {
        out[1 + q] = wgxf * m[q];
        out[1 + nm + q] = wgyf * m[q];
        out[1 + 2 * nm + q] = wgx * m[q];
        out[1 + 3 * nm + q] = wgy * m[q];
    }
    int k = 1 + 4 * nm;
    if constexpr (MODEL == kModelQuadratic) {
        // x = m[1], y = m[2]: the 15 monomials x^a y^b (a + b <= 4), exact
        const float x = m[1], y = m[2], x2 = x * x, xy = x * y, y2 = y * y;
        const float mono[15] = {1.0f, x, y, x2, xy, y2, x2 * x, x2 * y, x * y2, y2 * y,
                                x2 * x2, x2 * xy, x2 * y2, xy * y2, y2 * y2};
#pragma unroll
        for (int block = 0; block < 3; ++block) {
            const float wg = w * (block == 0 ? gx * gx : (block == 1 ? gx * gy : gy * gy));
#pragma unroll
            for (int q = 0; q < 15; ++q) out[k++] = wg * mono[q];
        }
    } else {
#pragma unroll
        for (int block = 0; block < 3; ++block) {
            const float wg = w * (block == 0 ? gx * gx : (block == 1 ? gx * gy : gy * gy));
#pragma unroll
            for (int i = 0; i < nm; ++i) {
                const float wgi = wg * m[i];
#pragma unroll
                for (int j = i; j < nm; ++j) out[k++] = wgi * m[j];
            }
        }
    }
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// Combine two sums held as head + tail (s + c) with an exact TwoSum of the
// heads.
__device__ __forceinline__ void twosum_merge(float &s, float &c, float s2, float c2) {
    const float t = s + s2;
    const float bp = t - s;
    const float err = (s - (t - bp)) + (s2 - bp);
    s = t;
    c = (c + c2) + err;
}

// Warp total of per-lane Kahan sums.  On entry a lane's sum is s - c (c is
// the compensation kahan_add carries: the excess of the last addition); on
// return lane 0 holds the total as a head and an additive tail, s + c.
__device__ __forceinline__ void warp_compensated_sum(float &s, float &c) {
    c = -c;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const float s2 = __shfl_down_sync(kFullMask, s, off);
        const float c2 = __shfl_down_sync(kFullMask, c, off);
        twosum_merge(s, c, s2, c2);
    }
}

// Warp-cooperative Cholesky inverse of an SPD n x n matrix held in shared
// memory (row-major A), with Jacobi scaling d_i = 1/sqrt(A_ii).  On return
// X holds A^-1; returns false if A is not numerically positive definite.
// Used for the FP32 6x6 Hessians; the FP64 12x12 quadratic ones go through
// cholesky_inverse_split.
template <typename T>
__device__ bool cholesky_inverse(T *A, T *X, T *d, int n, int lane) {
    bool ok = true;
    if (lane < n) {
        const T aii = A[lane * n + lane];
        ok = aii > T(0);
        d[lane] = ok ? T(1) / sqrt(aii) : T(0);
    }
    ok = __all_sync(kFullMask, ok);
    if (!ok) return false;
    __syncwarp();
    if (lane < n)
        for (int j = 0; j < n; ++j) A[lane * n + j] = A[lane * n + j] * d[lane] * d[j];
    __syncwarp();
    for (int k = 0; k < n; ++k) {
        T pivot = A[k * n + k];
        ok = pivot > T(0);
        if (!__all_sync(kFullMask, ok)) return false;
        const T lkk = sqrt(pivot);
        __syncwarp();
        if (lane == k) A[k * n + k] = lkk;
        if (lane > k && lane < n) A[lane * n + k] = A[lane * n + k] / lkk;
        __syncwarp();
        if (lane > k && lane < n) {
            const T lik = A[lane * n + k];
            for (int j = k + 1; j <= lane; ++j) A[lane * n + j] = A[lane * n + j] - lik * A[j * n + k];
        }
        __syncwarp();
    }
    // lane j: column j of L^-1 (forward substitution) into X (lower part)
    if (lane < n) {
        const int j = lane;
        for (int i = 0; i < n; ++i) X[i * n + j] = T(0);
        X[j * n + j] = T(1) / A[j * n + j];
        for (int i = j + 1; i < n; ++i) {
            T acc = T(0);
            for (int k = j; k < i; ++k) acc = acc + A[i * n + k] * X[k * n + j];
            X[i * n + j] = -acc / A[i * n + i];
        }
    }
    __syncwarp();
    // A^-1 = L^-T L^-1; lane i writes row i into A (A no longer needed).
    if (lane < n) {
        const int i = lane;
        for (int j = 0; j < n; ++j) {
            const int k0 = i > j ? i : j;
            T acc = T(0);
            for (int k = k0; k < n; ++k) acc = acc + X[k * n + i] * X[k * n + j];
            A[i * n + j] = acc * d[i] * d[j];
        }
    }
    __syncwarp();
    if (lane < n)
        for (int j = 0; j < n; ++j) X[lane * n + j] = A[lane * n + j];
    __syncwarp();
    return true;
}

// FP64 Cholesky inverse of the 12x12 quadratic Hessian with two lanes per
// row (lane & 15 = row, lane >> 4 = half): the Jacobi-scaled factorisation,
// L^-1 and L^-T L^-1 of cholesky_inverse, with every row's j loops and
// k sums split by parity between the two halves (partial sums combined by
// one shuffle), so the warp issues about half the FP64 instructions.
__device__ bool cholesky_inverse_split(double *A, double *X, double *d, int n, int lane) {
    __shared__ double s_r[4][12];
    double *rdiag = s_r[(threadIdx.x >> 5) & 3];
    const int row = lane & 15, half = lane >> 4;
    const bool mine = row < n;
    bool ok = true;
    if (mine && half == 0) {
        const double aii = A[row * n + row];
        ok = aii > 0.0;
        d[row] = ok ? rsqrt(aii) : 0.0;
    }
    if (!__all_sync(kFullMask, ok)) return false;
    __syncwarp();
    if (mine)
        for (int j = half; j < n; j += 2) A[row * n + j] = A[row * n + j] * d[row] * d[j];
    __syncwarp();
    for (int k = 0; k < n; ++k) {
        const double pivot = A[k * n + k];
        if (!__all_sync(kFullMask, pivot > 0.0)) return false;
        __syncwarp();
        const double r = rsqrt(pivot);
        if (half == 0 && row == k) { A[k * n + k] = pivot * r; rdiag[k] = r; }
        if (half == 0 && mine && row > k) A[row * n + k] = A[row * n + k] * r;
        __syncwarp();
        if (mine && row > k) {
            const double lik = A[row * n + k];
            for (int j = k + 1 + half; j <= row; j += 2) A[row * n + j] = A[row * n + j] - lik * A[j * n + k];
        }
        __syncwarp();
    }
    // L^-1, column `row`: X[i][row] = -(sum_k L[i][k] X[k][row]) / L[i][i]
    if (mine && half == 0) {
        for (int i = 0; i < n; ++i) X[i * n + row] = 0.0;
        X[row * n + row] = rdiag[row];
    }
    __syncwarp();
    for (int i = 1; i < n; ++i) {
        double acc = 0.0;
        if (mine && i > row)
            for (int k = row + half; k < i; k += 2) acc = acc + A[i * n + k] * X[k * n + row];
        acc = acc + __shfl_xor_sync(kFullMask, acc, 16);
        if (mine && half == 0 && i > row) X[i * n + row] = -acc * rdiag[i];
        __syncwarp();
    }
    // A^-1 = D L^-T L^-1 D; row `row`, columns split by parity, into A.
    if (mine) {
        for (int j = half; j < n; j += 2) {
            const int k0 = row > j ? row : j;
            double acc = 0.0;
            for (int k = k0; k < n; ++k) acc = acc + X[k * n + row] * X[k * n + j];
            A[row * n + j] = acc * d[row] * d[j];
        }
    }
    __syncwarp();
    if (mine)
        for (int j = half; j < n; j += 2) X[row * n + j] = A[row * n + j];
    __syncwarp();
    return true;
}

template <int MODEL>
__global__ void __launch_bounds__(128) subset_prep_kernel(PrepArgs a) {
    using T = typename std::conditional<MODEL == kModelQuadratic, double, float>::type;
    constexpr int n = parameter_count(MODEL);
    constexpr int nm = Moments<MODEL>::nm, P = Moments<MODEL>::hess, NM = Moments<MODEL>::count;
    constexpr int kChunkM = MODEL == kModelTranslation ? 8 : (MODEL == kModelQuadratic ? 36 : 32);
    __shared__ float s_tot[4][NM];
    __shared__ T s_A[4][n * n];
    __shared__ T s_X[4][n * n];
    __shared__ T s_d[4][n];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * 4 + warp;
    if (idx >= a.count) return;  // warp-uniform
    const int S = a.S, npix = S * S;
    const int gx0 = (idx % a.grid_w) * a.stride, gy0 = (idx / a.grid_w) * a.stride;
    const float half = 0.5f * ((float)S - 1.0f);
    // pass 1: weighted mean of the intensity
    // Pixel p = lane + 32 k of the window, tracked without divisions.
    const int ldiv = 32 / S, lmod = 32 % S, col0 = lane % S, row0 = lane / S;
    float s = 0.0f, c = 0.0f;
    {
        int col = col0, row = row0;
        for (int p = lane; p < npix; p += 32) {
            const float I = a.plane[(size_t)(gy0 + row) * a.W + gx0 + col].x;
            kahan_add(s, c, a.weights[p] * I);
            col += lmod;
            row += ldiv;
            if (col >= S) { col -= S; ++row; }
        }
    }
    warp_compensated_sum(s, c);
    const float mean = __shfl_sync(kFullMask, s + c, 0) / a.weight_sum;
    // passes over the moments, kChunkM at a time (unrolled: constant indices)
#pragma unroll
    for (int base = 0; base < NM; base += kChunkM) {
        // Kahan sums of moment pairs in packed FP32 (FADD2 / FFMA2): every
        // component follows kahan_add's sequence, a - b written as
        // fma(b, -1, a) (an exact product, so the same rounding).
        float2 ms2[kChunkM / 2], mc2[kChunkM / 2];
#pragma unroll
        for (int q = 0; q < kChunkM / 2; ++q) { ms2[q] = make_float2(0.0f, 0.0f); mc2[q] = make_float2(0.0f, 0.0f); }
        int col = col0, row = row0;
        for (int p = lane; p < npix; p += 32) {
            const float4 v = a.plane[(size_t)(gy0 + row) * a.W + gx0 + col];
            const float f = v.x - mean;
            const float w = a.weights[p];
            const float x = (float)col - half, y = (float)row - half;
            float m[6] = {1.0f, x, y, 0.5f * x * x, x * y, 0.5f * y * y};
            float mv[NM];
            moment_values<MODEL>(w, f, v.y, v.z, m, mv);
            const float2 m1 = make_float2(-1.0f, -1.0f);
#pragma unroll
            for (int q = 0; q < kChunkM / 2; ++q) {
                if (base + 2 * q < NM) {
                    const float2 val = make_float2(mv[base + 2 * q], base + 2 * q + 1 < NM ? mv[base + 2 * q + 1] : 0.0f);
                    const float2 y = __ffma2_rn(mc2[q], m1, val);
                    const float2 t = __fadd2_rn(ms2[q], y);
                    mc2[q] = __ffma2_rn(y, m1, __ffma2_rn(ms2[q], m1, t));
                    ms2[q] = t;
                }
            }
            col += lmod;
            row += ldiv;
            if (col >= S) { col -= S; ++row; }
        }
#pragma unroll
        for (int q = 0; q < kChunkM; ++q) {
            if (base + q < NM) {
                float sq = (q & 1) ? ms2[q / 2].y : ms2[q / 2].x, cq = (q & 1) ? mc2[q / 2].y : mc2[q / 2].x;
                warp_compensated_sum(sq, cq);
                if (lane == 0) s_tot[warp][base + q] = sq + cq;
            }
        }
    }
    __syncwarp();
    // centre the plane for tiled (non-overlapping) grids
    if (a.stride == S) {
        for (int p = lane; p < npix; p += 32) {
            const int col = p % S, row = p / S;
            float4 *dst = a.plane + (size_t)(gy0 + row) * a.W + gx0 + col;
            dst->x = dst->x - mean;
        }
    }
    const float *t = s_tot[warp];
    const float energy = t[0];
    T *A = s_A[warp];
    T *X = s_X[warp];
    float jtf[n], sj[n];
#pragma unroll
    for (int q = 0; q < n; ++q) { jtf[q] = 0.0f; sj[q] = 0.0f; }
    bool valid = energy > 1e-12f;
    if (MODEL == kModelTranslation) {
        // moments: 0 f^2, 1 gx f, 2 gy f, 3 gx, 4 gy, 5 gx^2, 6 gx gy, 7 gy^2
        jtf[0] = t[1]; jtf[3] = t[2]; sj[0] = t[3]; sj[3] = t[4];
        const float hxx = t[5], hxy = t[6], hyy = t[7];
        const float det = fmaf(hxx, hyy, -(hxy * hxy));
        const float scale = fmaxf(fabsf(hxx * hyy), 1.0f);
        valid = valid && isfinite(det) && fabsf(det) > FLT_EPSILON * scale;
        if (lane == 0) {
            for (int q = 0; q < n * n; ++q) X[q] = T(0);
            if (valid) {
                X[0] = hyy / det;
                X[3] = -hxy / det;
                X[3 * n] = -hxy / det;
                X[3 * n + 3] = hxx / det;
            }
        }
        __syncwarp();
    } else {
        // Jacobian column q = (gradient block, monomial): affine
        // [gx m0..m2, gy m0..m2]; quadratic [gx m0..m2, gy m0..m2, gx m3..m5, gy m3..m5]
        auto blk = [](int q) { return MODEL == kModelQuadratic ? ((q < 3 || (q >= 6 && q < 9)) ? 0 : 1) : (q < 3 ? 0 : 1); };
        auto mono = [](int q) {
            return MODEL == kModelQuadratic ? (q < 3 ? q : (q < 6 ? q - 3 : (q < 9 ? q - 3 : q - 6))) : (q < 3 ? q : q - 3);
        };
#pragma unroll
        for (int q = 0; q < n; ++q) {
            const int b = blk(q), i = mono(q);
            jtf[q] = t[1 + b * nm + i];
            sj[q] = t[1 + 2 * nm + b * nm + i];
        }
        if (lane < n) {
            const int bq = blk(lane), iq = mono(lane);
            for (int r = 0; r < n; ++r) {
                const int br = blk(r), ir = mono(r);
                const int lo = iq < ir ? iq : ir, hi = iq < ir ? ir : iq;
                A[lane * n + r] = (T)(hess_scale<MODEL>(lo, hi) * t[1 + 4 * nm + (bq + br) * P + hess_index<MODEL>(lo, hi)]);
            }
        }
        __syncwarp();
        bool ok;
        if constexpr (std::is_same<T, double>::value) ok = cholesky_inverse_split(A, X, s_d[warp], n, lane);
        else ok = cholesky_inverse<T>(A, X, s_d[warp], n, lane);
        valid = valid && ok;
        if (ok) {
            bool finite = true;
            for (int q = lane; q < n * n; q += 32) {
                const double v = (double)X[q];
                finite = finite && isfinite(v) && fabs(v) <= (double)FLT_MAX;
            }
            valid = valid && __all_sync(kFullMask, finite);
        }
    }
    const bool selected = a.selected == nullptr || a.selected[idx] != 0;
    float *inv = a.inv + (size_t)idx * n * n;
    for (int q = lane; q < n * n; q += 32) inv[q] = valid ? (float)X[q] : 0.0f;
    if (lane == 0) {
        float *md = a.meta + (size_t)idx * meta_stride(MODEL);
        md[0] = sqrtf(fmaxf(energy, 0.0f));
        md[1] = selected ? (valid ? 1.0f : 0.0f) : -3.0f;
        for (int q = 0; q < n; ++q) {
            md[2 + q] = jtf[q];
            md[2 + n + q] = sj[q];
        }
        md[2 + 2 * n] = a.stride == S ? 0.0f : mean;
        md[3 + 2 * n] = a.weight_sum;
        for (int q = 4 + 2 * n; q < meta_stride(MODEL); ++q) md[q] = 0.0f;
        if (valid && selected) atomicAdd(a.valid_count, 1u);
        a.admissible[idx] = valid ? 1 : 0;
    }
}

}  // namespace

cudaError_t set_gauss_taps(const float *taps7) { return cudaMemcpyToSymbol(c_gauss, taps7, 7 * sizeof(float)); }

cudaError_t launch_reference_prep(const PrepArgs &a, cudaStream_t stream) {
    const int W = a.W, H = a.H;
    const bool bspline = a.interp == kInterpBspline;
    dim3 gg((W + 63) / 64, (H + 31) / 32);
    gauss7_kernel<<<gg, 256, 0, stream>>>(a.img, W, H, a.pitch, bspline ? 1 : 0, a.intensity);
    const float *grad_src = a.intensity;
    if (bspline) {
        // rows: transpose (H x W -> W x H), filter columns of length W, transpose back
        dim3 tb(kTile, 8);
        transpose_kernel<<<dim3((W + kTile - 1) / kTile, (H + kTile - 1) / kTile), tb, 0, stream>>>(
            a.intensity, H, W, a.scratch);
        spline_columns_kernel<<<dim3((H + 127) / 128, (W + kChunk - 1) / kChunk), 128, 0, stream>>>(
            a.scratch, W, H, a.spline);
        transpose_kernel<<<dim3((H + kTile - 1) / kTile, (W + kTile - 1) / kTile), tb, 0, stream>>>(
            a.spline, W, H, a.scratch);
        spline_columns_kernel<<<dim3((W + 127) / 128, (H + kChunk - 1) / kChunk), 128, 0, stream>>>(
            a.scratch, H, W, a.spline);
        grad_src = a.spline;
    }
    gradient_kernel<<<dim3((W + 127) / 128, H), 128, 0, stream>>>(a.intensity, grad_src, W, H,
                                                                    bspline ? 1 : 0, a.plane);
    const int blocks = (a.count + 3) / 4;
    if (blocks > 0 && a.moments) {
        const cudaError_t err = launch_quadratic_row_prep(a, stream);
        if (err != cudaSuccess) return err;
    } else if (blocks > 0) {
        switch (a.model) {
        case kModelTranslation: subset_prep_kernel<kModelTranslation><<<blocks, 128, 0, stream>>>(a); break;
        case kModelQuadratic: subset_prep_kernel<kModelQuadratic><<<blocks, 128, 0, stream>>>(a); break;
        default: subset_prep_kernel<kModelAffine><<<blocks, 128, 0, stream>>>(a); break;
        }
    }
    return cudaGetLastError();
}

}  // namespace gbdic
