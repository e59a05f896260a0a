// Data-movement and element-wise kernels of the learned seed network.  The
// contractions (convolutions as implicit GEMMs, the final linear layer and
// all their gradients) run on the tensor cores in tc_gemm.cu; everything here
// is HBM-bound glue around them:
//   patch extraction and normalisation, 3x3 stride-2 im2col (and its
//   transpose for the weight gradient), the gather of output gradients for
//   the data gradient, BF16 transposes, ReLU backward fused with the bias
//   gradient and the output-gradient transpose, split-K reduction of weight
//   gradients, Adam, weight packing and the regression loss.
// Activations are NHWC BF16 (rows = pixels, channels contiguous); weights are
// [Cout][(ky, kx, ci)] with the reduction index padded to the GEMM tile.
#include <cuda_bf16.h>

#include <algorithm>

#include <cstdint>

#include "gbdic_kernels.h"

namespace gbdic {
namespace {

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// One CTA (256 threads) per patch: 64 x 64 pixels of the reference and target
// level images around (cx, cy), each channel normalised to zero mean and unit
// variance, written as [64][64][2] BF16.
__global__ void __launch_bounds__(256) patch_kernel(NnPatchArgs a) {
    const int b = blockIdx.x;
    if (b >= a.count) return;
    const int img = a.image_index ? a.image_index[b] : 0;
    const uint8_t *ref = a.refs[img], *tgt = a.tgts[img];
    const float cx = a.centres[2 * b], cy = a.centres[2 * b + 1];
    const int x0 = (int)floorf(cx + 0.5f) - 32, y0 = (int)floorf(cy + 0.5f) - 32;
    // Target window: optionally displaced by a previous prediction.
    float sx = 0.0f, sy = 0.0f;
    if (a.shift) {
        sx = a.shift[(size_t)b * a.shift_ld] * a.shift_scale;
        sy = a.shift[(size_t)b * a.shift_ld + 3] * a.shift_scale;
        if (!(fabsf(sx) < 1e4f)) sx = 0.0f;
        if (!(fabsf(sy) < 1e4f)) sy = 0.0f;
    }
    const int tx0 = (int)floorf(cx + sx + 0.5f) - 32, ty0 = (int)floorf(cy + sy + 0.5f) - 32;
    float vr[16], vt[16];
    float sr = 0.0f, st = 0.0f, qr = 0.0f, qt = 0.0f;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int p = threadIdx.x + 256 * i;
        const int x = min(max(x0 + (p & 63), 0), a.W - 1), y = min(max(y0 + (p >> 6), 0), a.H - 1);
        const int u = min(max(tx0 + (p & 63), 0), a.W - 1), v = min(max(ty0 + (p >> 6), 0), a.H - 1);
        vr[i] = (float)ref[(size_t)y * a.W + x];
        vt[i] = (float)tgt[(size_t)v * a.W + u];
        sr += vr[i]; st += vt[i]; qr += vr[i] * vr[i]; qt += vt[i] * vt[i];
    }
    __shared__ float red[4][8];
    float v4[4] = {sr, st, qr, qt};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float v = v4[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    float tot[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float v = 0.0f;
        for (int w = 0; w < 8; ++w) v += red[k][w];
        tot[k] = v;
    }
    const float mr = tot[0] / 4096.0f, mt = tot[1] / 4096.0f;
    const float ir = rsqrtf(fmaxf(tot[2] / 4096.0f - mr * mr, 1e-2f));
    const float it = rsqrtf(fmaxf(tot[3] / 4096.0f - mt * mt, 1e-2f));
    __nv_bfloat162 *out = reinterpret_cast<__nv_bfloat162 *>(a.out) + (size_t)b * 4096;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int p = threadIdx.x + 256 * i;
        out[p] = __floats2bfloat162_rn((vr[i] - mr) * ir, (vt[i] - mt) * it);
    }
}

// A[m][k] for m = (b, oy, ox), k = (ky, kx, ci) < 9 C; zero for k >= 9 C.
__global__ void im2col_kernel(NnConvShape s, const __nv_bfloat16 *x, __nv_bfloat16 *A) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rows = (long long)s.B * s.OH * s.OW;
    if (idx >= rows * s.Kp) return;
    const int k = (int)(idx % s.Kp);
    const long long m = idx / s.Kp;
    __nv_bfloat16 v = __float2bfloat16(0.0f);
    if (k < 9 * s.C) {
        const int tap = k / s.C, ci = k % s.C, ky = tap / 3, kx = tap % 3;
        const int ox = (int)(m % s.OW), oy = (int)((m / s.OW) % s.OH), b = (int)(m / ((long long)s.OW * s.OH));
        const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
        if (iy >= 0 && iy < s.H && ix >= 0 && ix < s.W) v = x[(((size_t)b * s.H + iy) * s.W + ix) * s.C + ci];
    }
    A[idx] = v;
}

// Vectorised im2col for C a multiple of 8: thread (m, q) writes the 16 bytes
// A[m][8q .. 8q+7], which lie in one tap (ci0 = 8q mod C) and so come from
// one 16-byte load of the input pixel, or are zero (padding tap or k >= 9 C).
__global__ void im2col_vec_kernel(NnConvShape s, const uint4 *x, uint4 *A) {
    const int chunks = s.Kp / 8;
    const int rows = s.B * s.OH * s.OW;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= rows * chunks) return;
    const int q = idx % chunks, m = idx / chunks;
    const int k0 = 8 * q;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (k0 < 9 * s.C) {
        const int tap = k0 / s.C, ci0 = k0 - tap * s.C, ky = tap / 3, kx = tap - 3 * ky;
        const int ox = m % s.OW, t = m / s.OW, oy = t % s.OH, b = t / s.OH;
        const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
        if (iy >= 0 && iy < s.H && ix >= 0 && ix < s.W)
            v = __ldg(x + ((((size_t)b * s.H + iy) * s.W + ix) * s.C + ci0) / 8);
    }
    A[idx] = v;
}

// im2col for the 2-channel input layer: one row (Kp bf16) per thread, each
// tap's channel pair one 4-byte load, the row written as 16-byte stores.
__global__ void im2col_c2_kernel(NnConvShape s, const uint32_t *x, uint4 *A) {
    const int rows = s.B * s.OH * s.OW;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= rows) return;
    const int ox = m % s.OW, t = m / s.OW, oy = t % s.OH, b = t / s.OH;
    uint32_t w[12];
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
        const int ky = tap / 3, kx = tap - 3 * ky;
        const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
        w[tap] = (iy >= 0 && iy < s.H && ix >= 0 && ix < s.W) ? __ldg(x + ((size_t)b * s.H + iy) * s.W + ix) : 0u;
    }
    w[9] = w[10] = w[11] = 0u;
    uint4 *row = A + (size_t)m * (s.Kp / 8);
    row[0] = make_uint4(w[0], w[1], w[2], w[3]);
    row[1] = make_uint4(w[4], w[5], w[6], w[7]);
    row[2] = make_uint4(w[8], w[9], w[10], w[11]);
    for (int q = 3; q < s.Kp / 8; ++q) row[q] = make_uint4(0u, 0u, 0u, 0u);
}

// G[m][k] for input pixel m = (b, iy, ix) and k = (ky, kx, co) < 9 Cout: the
// output gradient at (oy, ox) = ((iy + 1 - ky) / 2, (ix + 1 - kx) / 2) when
// both are integral and inside the output, else zero.
__global__ void dgrad_gather_kernel(NnConvShape s, const __nv_bfloat16 *dz, __nv_bfloat16 *G) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rows = (long long)s.B * s.H * s.W;
    const int kg = 9 * s.Cout;
    if (idx >= rows * kg) return;
    const int k = (int)(idx % kg);
    const long long m = idx / kg;
    const int tap = k / s.Cout, co = k % s.Cout, ky = tap / 3, kx = tap % 3;
    const int ix = (int)(m % s.W), iy = (int)((m / s.W) % s.H), b = (int)(m / ((long long)s.W * s.H));
    const int ty = iy + 1 - ky, tx = ix + 1 - kx;
    __nv_bfloat16 v = __float2bfloat16(0.0f);
    if (ty >= 0 && tx >= 0 && !(ty & 1) && !(tx & 1) && (ty >> 1) < s.OH && (tx >> 1) < s.OW)
        v = dz[(((size_t)b * s.OH + (ty >> 1)) * s.OW + (tx >> 1)) * s.Cout + co];
    G[idx] = v;
}

// Vectorised dgrad_gather for Cout a multiple of 8: 16 bytes (8 output
// channels of one tap) per thread.
__global__ void dgrad_gather_vec_kernel(NnConvShape s, const uint4 *dz, uint4 *G) {
    const int chunks = 9 * s.Cout / 8;
    const int rows = s.B * s.H * s.W;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= rows * chunks) return;
    const int q = idx % chunks, m = idx / chunks;
    const int k0 = 8 * q, tap = k0 / s.Cout, co0 = k0 - tap * s.Cout, ky = tap / 3, kx = tap - 3 * ky;
    const int ix = m % s.W, t = m / s.W, iy = t % s.H, b = t / s.H;
    const int ty = iy + 1 - ky, tx = ix + 1 - kx;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (ty >= 0 && tx >= 0 && !(ty & 1) && !(tx & 1) && (ty >> 1) < s.OH && (tx >> 1) < s.OW)
        v = __ldg(dz + ((((size_t)b * s.OH + (ty >> 1)) * s.OW + (tx >> 1)) * s.Cout + co0) / 8);
    G[idx] = v;
}

// dst[c][r] = src[r][c] for r < R, c < C; zero in the padding up to Rp x Cp.
__global__ void transpose_kernel(const __nv_bfloat16 *src, int R, int C, int ld_src, __nv_bfloat16 *dst, int Rp,
                                 int Cp) {
    __shared__ __nv_bfloat16 tile[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        tile[i][threadIdx.x] = (r < R && c < C) ? src[(size_t)r * ld_src + c] : __float2bfloat16(0.0f);
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (c < Cp && r < Rp) dst[(size_t)c * Rp + r] = tile[threadIdx.x][i];
    }
}

// dZ = dY * (Y > 0) as BF16; rows x C, dY with row stride ld.
__global__ void relu_backward_kernel(const float *dy, int ld, const __nv_bfloat16 *y, __nv_bfloat16 *dz, long long rows,
                                     int C) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= rows * C) return;
    const long long r = idx / C;
    const int c = (int)(idx % C);
    const float g = bf(y[idx]) > 0.0f ? dy[r * ld + c] : 0.0f;
    dz[idx] = __float2bfloat16(g);
}

// db[c] = sum over rows of dY[r][c] * (Y[r][c] > 0) (Y == nullptr: no mask),
// one CTA per column, fixed summation order.
__global__ void __launch_bounds__(256) bias_grad_kernel(const float *dy, int ld, const __nv_bfloat16 *y, long long rows,
                                                        int C, float *db) {
    const int c = blockIdx.x;
    float acc = 0.0f;
    for (long long r = threadIdx.x; r < rows; r += 256) {
        const float g = dy[r * ld + c];
        acc += (y == nullptr || bf(y[r * C + c]) > 0.0f) ? g : 0.0f;
    }
    __shared__ float red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[c] = red[0];
}

// ReLU backward, bias gradient and the transposed output gradient in one
// pass over dY: dZ = dY where Y > 0 (everywhere when y == nullptr), written
// BF16 as [rows][C] and, when dzt != nullptr, as [C][rows]; the FP32 column
// sums of each 64-row tile go to partial[c * tiles + tile] (rows ascending
// per thread, then the threads of a column in order).  256 threads, C a
// power of two from 4 to 256; the reads (float4 of dY) and both writes are
// contiguous, the transpose staged in shared memory.
__global__ void __launch_bounds__(256) relu_bias_backward_kernel(const float *dy, int ld, const __nv_bfloat16 *y,
                                                                 long long rows, int C, __nv_bfloat16 *dz,
                                                                 __nv_bfloat16 *dzt, float *partial, int tiles) {
    extern __shared__ __align__(16) uint8_t nn_smem[];
    float4 *red = reinterpret_cast<float4 *>(nn_smem);                       // [256]
    __nv_bfloat16 *tile = reinterpret_cast<__nv_bfloat16 *>(nn_smem + 256 * sizeof(float4));  // [C][72]
    const int t = threadIdx.x, groups = C / 4, c4 = t % groups, rstep = 256 / groups;
    const long long r0 = (long long)blockIdx.x * 64;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int r = t / groups; r < 64 && r0 + r < rows; r += rstep) {
        const long long row = r0 + r;
        float4 g = *reinterpret_cast<const float4 *>(dy + row * ld + 4 * c4);
        if (y != nullptr) {
            const uint2 yy = *reinterpret_cast<const uint2 *>(y + row * C + 4 * c4);
            const __nv_bfloat162 y01 = *reinterpret_cast<const __nv_bfloat162 *>(&yy.x);
            const __nv_bfloat162 y23 = *reinterpret_cast<const __nv_bfloat162 *>(&yy.y);
            if (!(bf(y01.x) > 0.0f)) g.x = 0.0f;
            if (!(bf(y01.y) > 0.0f)) g.y = 0.0f;
            if (!(bf(y23.x) > 0.0f)) g.z = 0.0f;
            if (!(bf(y23.y) > 0.0f)) g.w = 0.0f;
        }
        acc.x += g.x; acc.y += g.y; acc.z += g.z; acc.w += g.w;
        const __nv_bfloat162 lo = __floats2bfloat162_rn(g.x, g.y), hi = __floats2bfloat162_rn(g.z, g.w);
        uint2 out;
        out.x = *reinterpret_cast<const uint32_t *>(&lo);
        out.y = *reinterpret_cast<const uint32_t *>(&hi);
        *reinterpret_cast<uint2 *>(dz + row * C + 4 * c4) = out;
        if (dzt != nullptr) {
            tile[(4 * c4 + 0) * 72 + r] = lo.x;
            tile[(4 * c4 + 1) * 72 + r] = lo.y;
            tile[(4 * c4 + 2) * 72 + r] = hi.x;
            tile[(4 * c4 + 3) * 72 + r] = hi.y;
        }
    }
    red[t] = acc;
    __syncthreads();
    if (t < groups) {
        float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int q = t; q < 256; q += groups) {
            const float4 v = red[q];
            sum.x += v.x; sum.y += v.y; sum.z += v.z; sum.w += v.w;
        }
        partial[(size_t)(4 * t + 0) * tiles + blockIdx.x] = sum.x;
        partial[(size_t)(4 * t + 1) * tiles + blockIdx.x] = sum.y;
        partial[(size_t)(4 * t + 2) * tiles + blockIdx.x] = sum.z;
        partial[(size_t)(4 * t + 3) * tiles + blockIdx.x] = sum.w;
    }
    if (dzt != nullptr) {
        // rows % 8 == 0: every 8-row chunk is complete or absent
        for (int idx = t; idx < C * 8; idx += 256) {
            const int c = idx >> 3, ch = idx & 7;
            if (r0 + 8 * ch >= rows) continue;
            *reinterpret_cast<uint4 *>(dzt + (size_t)c * rows + r0 + 8 * ch) =
                *reinterpret_cast<const uint4 *>(tile + c * 72 + 8 * ch);
        }
    }
}

// y[m][n] = BF16(relu(sum_s partial[s][m][n] + bias[n])) for split-K
// convolution outputs (splits ascending), 4 columns per thread.
__global__ void splitk_bias_relu_kernel(const float *partial, int splits, long long rows, int N,
                                        long long split_stride, const float *bias, int relu, __nv_bfloat16 *y) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // float4 index
    if (q >= rows * N / 4) return;
    float4 acc = reinterpret_cast<const float4 *>(partial)[q];
    for (int s = 1; s < splits; ++s) {
        const float4 v = reinterpret_cast<const float4 *>(partial + s * split_stride)[q];
        acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
    }
    const int n = (int)((4 * q) % N);
    if (bias) { acc.x += bias[n]; acc.y += bias[n + 1]; acc.z += bias[n + 2]; acc.w += bias[n + 3]; }
    if (relu) { acc.x = fmaxf(acc.x, 0.0f); acc.y = fmaxf(acc.y, 0.0f); acc.z = fmaxf(acc.z, 0.0f); acc.w = fmaxf(acc.w, 0.0f); }
    const __nv_bfloat162 lo = __floats2bfloat162_rn(acc.x, acc.y), hi = __floats2bfloat162_rn(acc.z, acc.w);
    uint2 out;
    out.x = *reinterpret_cast<const uint32_t *>(&lo);
    out.y = *reinterpret_cast<const uint32_t *>(&hi);
    reinterpret_cast<uint2 *>(y)[q] = out;
}

// db[c] = sum over tiles of partial[c * tiles + tile]: one CTA per column,
// thread t the tiles t, t + 256, ... in order, then a fixed tree.
__global__ void __launch_bounds__(256) bias_reduce_kernel(const float *partial, int tiles, float *db) {
    const int c = blockIdx.x;
    float acc = 0.0f;
    for (int i = threadIdx.x; i < tiles; i += 256) acc += partial[(size_t)c * tiles + i];
    __shared__ float red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[c] = red[0];
}

// Transposed im2col At[k][m] = A[m][k] (A as im2col_kernel writes it, zero
// for k >= 9 C) for k < Kt, m < M = B OH OW: one CTA per 64 k x 64 m tile,
// staged in shared memory so that the reads (a pixel's channels) and the
// writes (64 consecutive m of one k, 128 bytes) are both contiguous.  The
// weight-gradient GEMM reads At; A itself is never written.
__global__ void __launch_bounds__(256) im2col_t_kernel(NnConvShape s, const __nv_bfloat16 *x, __nv_bfloat16 *At,
                                                       int Kt) {
    __shared__ __align__(16) __nv_bfloat16 tile[64 * 72];  // [k][m], rows padded to 72
    const int M = s.B * s.OH * s.OW;
    const int m0 = blockIdx.x * 64, k0 = blockIdx.y * 64, t = threadIdx.x;
    if (s.C % 8 == 0) {
        for (int i = 0; i < 2; ++i) {
            const int j = t & 7, ml = (t >> 3) + 32 * i, m = m0 + ml, k = k0 + 8 * j;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (m < M && k < 9 * s.C) {
                const int tap = k / s.C, ci0 = k - tap * s.C, ky = tap / 3, kx = tap - 3 * ky;
                const int ox = m % s.OW, tt = m / s.OW, oy = tt % s.OH, b = tt / s.OH;
                const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
                if (iy >= 0 && iy < s.H && ix >= 0 && ix < s.W)
                    v = __ldg(reinterpret_cast<const uint4 *>(x + (((size_t)b * s.H + iy) * s.W + ix) * s.C + ci0));
            }
            const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
            for (int q = 0; q < 8; ++q) tile[(8 * j + q) * 72 + ml] = e[q];
        }
    } else if (s.C == 2 && k0 == 0) {
        // 2 channels: one 4-byte load per (pixel, tap); rows 18 .. 63 zero
        for (int i = t; i < 64 * 9; i += 256) {
            const int ml = i & 63, tap = i >> 6, m = m0 + ml, ky = tap / 3, kx = tap - 3 * ky;
            uint32_t v = 0u;
            if (m < M) {
                const int ox = m % s.OW, tt = m / s.OW, oy = tt % s.OH, b = tt / s.OH;
                const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
                if (iy >= 0 && iy < s.H && ix >= 0 && ix < s.W)
                    v = __ldg(reinterpret_cast<const uint32_t *>(x + (((size_t)b * s.H + iy) * s.W + ix) * 2));
            }
            const __nv_bfloat162 pr = *reinterpret_cast<const __nv_bfloat162 *>(&v);
            tile[(2 * tap) * 72 + ml] = pr.x;
            tile[(2 * tap + 1) * 72 + ml] = pr.y;
        }
        for (int i = t; i < 64 * 46; i += 256) tile[(18 + (i >> 6)) * 72 + (i & 63)] = __float2bfloat16(0.0f);
    } else {
        for (int i = 0; i < 16; ++i) {
            const int kl = t & 63, ml = (t >> 6) + 4 * i, m = m0 + ml, k = k0 + kl;
            __nv_bfloat16 v = __float2bfloat16(0.0f);
            if (m < M && k < 9 * s.C) {
                const int tap = k / s.C, ci = k - tap * s.C, ky = tap / 3, kx = tap - 3 * ky;
                const int ox = m % s.OW, tt = m / s.OW, oy = tt % s.OH, b = tt / s.OH;
                const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
                if (iy >= 0 && iy < s.H && ix >= 0 && ix < s.W) v = x[(((size_t)b * s.H + iy) * s.W + ix) * s.C + ci];
            }
            tile[kl * 72 + ml] = v;
        }
    }
    __syncthreads();
    for (int i = 0; i < 2; ++i) {
        const int ch = t & 7, kl = (t >> 3) + 32 * i, k = k0 + kl, m = m0 + 8 * ch;
        if (k < Kt && m < M)
            *reinterpret_cast<uint4 *>(At + (size_t)k * M + m) = *reinterpret_cast<const uint4 *>(tile + kl * 72 + 8 * ch);
    }
}

// out[n][k] = sum_s partial[s][k][n] (s ascending) for k < Kp, n < N.
// Consecutive threads take consecutive n (contiguous partial reads); the
// loads of four splits are issued before their ordered additions.
__global__ void splitk_reduce_kernel(const float *partial, int splits, int Kp_rows, int N, int Kp, float *out) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N * Kp) return;
    const int k = idx / N, n = idx - k * N;
    const size_t stride = (size_t)Kp_rows * N;
    const float *p = partial + (size_t)k * N + n;
    float acc = 0.0f;
    int s = 0;
    for (; s + 4 <= splits; s += 4) {
        const float v0 = __ldg(p + s * stride), v1 = __ldg(p + (s + 1) * stride);
        const float v2 = __ldg(p + (s + 2) * stride), v3 = __ldg(p + (s + 3) * stride);
        acc += v0;
        acc += v1;
        acc += v2;
        acc += v3;
    }
    for (; s < splits; ++s) acc += __ldg(p + s * stride);
    out[(size_t)n * Kp + k] = acc;
}

// One Adam element update (shared by both kernels so that they compile to
// the same arithmetic).
__device__ __forceinline__ void adam_element(float *param, const float *grad, float *m_, float *v_, long long j,
                                             float lr, float beta1, float beta2, float eps, float bias1, float bias2,
                                             float weight_decay) {
    const float g = grad[j] + weight_decay * param[j];
    const float m = beta1 * m_[j] + (1.0f - beta1) * g;
    const float v = beta2 * v_[j] + (1.0f - beta2) * g * g;
    m_[j] = m;
    v_[j] = v;
    param[j] -= lr * (m / bias1) / (sqrtf(v / bias2) + eps);
}

// Adam over up to kMaxAdamTensors tensors in one launch: element i of the
// concatenation belongs to the tensor whose offset range holds it.
__global__ void adam_many_kernel(NnAdamMany a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.offset[a.n]) return;
    int t = 0;
    while (i >= a.offset[t + 1]) ++t;
    adam_element(a.param[t], a.grad[t], a.m[t], a.v[t], i - a.offset[t], a.lr, a.beta1, a.beta2, a.eps, a.bias1,
                 a.bias2, a.weight_decay);
}

__global__ void adam_kernel(NnAdamArgs a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    adam_element(a.param, a.grad, a.m, a.v, i, a.lr, a.beta1, a.beta2, a.eps, a.bias1, a.bias2, a.weight_decay);
}

// W [Cout][Kp] FP32 -> BF16 copy, and the data-gradient operand
// Wt[ci][(ky, kx, co)] = W[co][(ky, kx, ci)] (when wt != nullptr).
__global__ void pack_weights_kernel(const float *w, int Cout, int Cin, int Kp, __nv_bfloat16 *wb, __nv_bfloat16 *wt,
                                    int Kt) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= Cout * Kp) return;
    const int co = idx / Kp, k = idx % Kp;
    const __nv_bfloat16 v = __float2bfloat16(w[idx]);
    wb[idx] = v;
    if (wt != nullptr && k < 9 * Cin) {
        const int tap = k / Cin, ci = k % Cin;
        wt[(size_t)ci * Kt + tap * Cout + co] = v;
    }
}

// Loss 0.5 / B sum (pred - target)^2 over the first `outputs` columns and
// its gradient (pred - target) / B as BF16 [B][ldg] (zero elsewhere); one CTA.
__global__ void __launch_bounds__(1024) regression_loss_kernel(const float *pred, int ldp, const float *target,
                                                               int outputs, int B, __nv_bfloat16 *grad,
                                                               float *grad_f32, int ldg, float *loss) {
    float acc = 0.0f;
    for (int i = threadIdx.x; i < B * ldg; i += 1024) {
        const int b = i / ldg, j = i % ldg;
        float g = 0.0f;
        if (j < outputs) {
            const float d = pred[(size_t)b * ldp + j] - target[(size_t)b * outputs + j];
            acc += 0.5f * d * d;
            g = d / (float)B;
        }
        grad[i] = __float2bfloat16(g);
        if (grad_f32) grad_f32[i] = g;
    }
    __shared__ float red[1024];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int off = 512; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = red[0] / (float)B;
}

// Seeds of every subset from a lattice of every `step`-th subset: bilinear
// weights over the four surrounding lattice nodes, each node's affine warp
// Taylor-recentred to the subset centre (offset (gx - lx step) stride).  With
// `base` (a first pass), translations are base + residual.
__global__ void lattice_seed_kernel(NnLatticeArgs a) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= a.grid_w * a.grid_h) return;
    const int gx = idx % a.grid_w, gy = idx / a.grid_w;
    const float u = (float)gx / (float)a.step, v = (float)gy / (float)a.step;
    const int lx = a.lattice_w > 1 ? min(max((int)floorf(u), 0), a.lattice_w - 2) : 0;
    const int ly = a.lattice_h > 1 ? min(max((int)floorf(v), 0), a.lattice_h - 2) : 0;
    const float fx = a.lattice_w > 1 ? fminf(fmaxf(u - (float)lx, 0.0f), 1.0f) : 0.0f;
    const float fy = a.lattice_h > 1 ? fminf(fmaxf(v - (float)ly, 0.0f), 1.0f) : 0.0f;
    float acc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int corner = 0; corner < 4; ++corner) {
        const int cx = min(lx + (corner & 1), a.lattice_w - 1), cy = min(ly + (corner >> 1), a.lattice_h - 1);
        const float w = ((corner & 1) ? fx : 1.0f - fx) * ((corner & 2) ? fy : 1.0f - fy);
        const size_t row = (size_t)(cy * a.lattice_w + cx) * a.ldp;
        const float *p = a.pred + row;
        const float bx = a.base ? a.base[row] : 0.0f, by = a.base ? a.base[row + 3] : 0.0f;
        const float tx = (p[0] + bx) * a.translation_scale, ux = p[1] / a.gradient_scale, uy = p[2] / a.gradient_scale;
        const float ty = (p[3] + by) * a.translation_scale, vx = p[4] / a.gradient_scale, vy = p[5] / a.gradient_scale;
        const float dx = (float)(gx - cx * a.step) * (float)a.stride, dy = (float)(gy - cy * a.step) * (float)a.stride;
        acc[0] += w * (tx + ux * dx + uy * dy);
        acc[1] += w * ux;
        acc[2] += w * uy;
        acc[3] += w * (ty + vx * dx + vy * dy);
        acc[4] += w * vx;
        acc[5] += w * vy;
    }
    float4 *s = reinterpret_cast<float4 *>(a.seeds + (size_t)idx * 8);
    s[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    s[1] = make_float4(acc[4], acc[5], 0.0f, 0.0f);
    a.active[idx] = 1u;
}

// Robust affine field through the lattice translations, on the device (one
// CTA, no host round trip).  Totals t_i = (base_i + pred_i) * scale in pixels
// (columns 0 and 3, FP32); nodes with a non-finite total are outliers.
// Hypotheses: single-node translations, then affine maps through node triples
// (|det| > 1e-9 on rows (1, x, y)); each is scored by the probe nodes within
// the first tolerance, the most supported (lowest index on ties) wins and is
// refitted by least squares on its inliers while the tolerance tightens (sums
// in FP32 within a warp and FP64 across warps, normal equations solved in
// FP64); a refit with fewer than three inliers (or a singular system) stops
// the loop.  base columns 0 and 3 receive the fitted field / scale.  Fewer
// than three finite nodes: base receives the totals.  GB300's FP64 rate is a
// small fraction of its FP32 rate, so FP64 is kept to the 3x3 solves of the
// refits.
constexpr int kConsensusThreads = 256, kConsensusProbes = 256;

__device__ inline bool node_total(const NnConsensusArgs &a, int i, float &u, float &v) {
    if (i < 0 || i >= a.nodes) return false;
    const size_t row = (size_t)i * a.ldp;
    u = (a.base[row] + a.pred[row]) * a.scale;
    v = (a.base[row + 3] + a.pred[row + 3]) * a.scale;
    return isfinite(u) && isfinite(v);
}

// Block sums: FP32 within a warp, FP64 across warps (result in red[0]).
template <int N>
__device__ inline void block_sum(const float (&x)[N], double (*red)[N]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float y[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        y[k] = x[k];
        for (int off = 16; off > 0; off >>= 1) y[k] += __shfl_down_sync(0xffffffffu, y[k], off);
    }
    if (lane == 0)
        for (int k = 0; k < N; ++k) red[warp][k] = (double)y[k];
    __syncthreads();
    if (threadIdx.x < N) {
        double t = 0.0;
        for (int w = 0; w < kConsensusThreads / 32; ++w) t += red[w][threadIdx.x];
        red[0][threadIdx.x] = t;
    }
    __syncthreads();
}

// 3x3 solve by the adjugate; false when |det| <= eps.
template <typename T>
__device__ inline bool solve3(const T m[3][3], const T (&b)[2][3], T eps, T (&c)[6]) {
    const T c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1], c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2],
            c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    const T det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
    if (!(fabs(det) > eps)) return false;
    const T inv[3][3] = {
        {c00, m[0][2] * m[2][1] - m[0][1] * m[2][2], m[0][1] * m[1][2] - m[0][2] * m[1][1]},
        {c01, m[0][0] * m[2][2] - m[0][2] * m[2][0], m[0][2] * m[1][0] - m[0][0] * m[1][2]},
        {c02, m[0][1] * m[2][0] - m[0][0] * m[2][1], m[0][0] * m[1][1] - m[0][1] * m[1][0]}};
    const T rdet = T(1) / det;
#pragma unroll
    for (int o = 0; o < 2; ++o)
#pragma unroll
        for (int r = 0; r < 3; ++r) c[3 * o + r] = (inv[r][0] * b[o][0] + inv[r][1] * b[o][1] + inv[r][2] * b[o][2]) * rdet;
    return true;
}

// Coefficients (u0, ux, uy, v0, vx, vy) of hypothesis h; false if unusable.
__device__ inline bool hypothesis(const NnConsensusArgs &a, int h, float (&c)[6]) {
#pragma unroll
    for (int k = 0; k < 6; ++k) c[k] = 0.0f;
    if (h < a.n_single) return node_total(a, a.single[h], c[0], c[3]);
    const int *t = a.triple + 3 * (h - a.n_single);
    float m[3][3], b[2][3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        if (!node_total(a, t[r], b[0][r], b[1][r])) return false;
        const float2 p = a.xy[t[r]];
        m[r][0] = 1.0f; m[r][1] = p.x; m[r][2] = p.y;
    }
    return solve3<float>(m, b, 1e-9f, c);
}

__global__ void __launch_bounds__(kConsensusThreads) consensus_kernel(NnConsensusArgs a) {
    __shared__ double red[kConsensusThreads / 32][12];
    __shared__ int best_count[kConsensusThreads / 32], best_index[kConsensusThreads / 32];
    __shared__ float coef[6];
    __shared__ int finite_nodes, winner, stop;
    __shared__ float2 probe_t[kConsensusProbes], probe_xy[kConsensusProbes];
    __shared__ uint8_t probe_ok[kConsensusProbes];
    // finite nodes
    {
        int n = 0;
        for (int i = threadIdx.x; i < a.nodes; i += kConsensusThreads) {
            float u, v;
            n += node_total(a, i, u, v) ? 1 : 0;
        }
        n = __reduce_add_sync(0xffffffffu, n);
        if (threadIdx.x == 0) finite_nodes = 0;
        __syncthreads();
        if ((threadIdx.x & 31) == 0) atomicAdd(&finite_nodes, n);
        __syncthreads();
    }
    if (finite_nodes < 3) {
        for (int i = threadIdx.x; i < a.nodes; i += kConsensusThreads) {
            float u, v;
            node_total(a, i, u, v);
            const size_t row = (size_t)i * a.ldp;
            a.base[row] = u / a.scale;
            a.base[row + 3] = v / a.scale;
        }
        return;
    }
    // probe totals in shared memory (the inlier test is a squared distance
    // against the squared tolerance)
    for (int k = threadIdx.x; k < a.n_probe; k += kConsensusThreads) {
        float u, v;
        const int j = a.probe[k];
        const bool ok = node_total(a, j, u, v);
        probe_t[k] = ok ? make_float2(u, v) : make_float2(0.0f, 0.0f);
        probe_xy[k] = ok ? a.xy[j] : make_float2(0.0f, 0.0f);
        probe_ok[k] = ok ? 1 : 0;
    }
    __syncthreads();
    const float tol2 = a.tol[0] * a.tol[0];
    const int hyps = a.n_single + a.n_triple;
    int my_count = -1, my_index = 0x7fffffff;
    for (int h = threadIdx.x; h < hyps; h += kConsensusThreads) {
        float c[6];
        if (!hypothesis(a, h, c)) continue;
        int count = 0;
        for (int k = 0; k < a.n_probe; ++k) {
            const float2 p = probe_xy[k], t = probe_t[k];
            const float du = c[0] + c[1] * p.x + c[2] * p.y - t.x, dv = c[3] + c[4] * p.x + c[5] * p.y - t.y;
            count += (probe_ok[k] && du * du + dv * dv <= tol2) ? 1 : 0;
        }
        if (count > my_count) { my_count = count; my_index = h; }
    }
    for (int off = 16; off > 0; off >>= 1) {
        const int oc = __shfl_down_sync(0xffffffffu, my_count, off), oi = __shfl_down_sync(0xffffffffu, my_index, off);
        if (oc > my_count || (oc == my_count && oi < my_index)) { my_count = oc; my_index = oi; }
    }
    if ((threadIdx.x & 31) == 0) { best_count[threadIdx.x >> 5] = my_count; best_index[threadIdx.x >> 5] = my_index; }
    __syncthreads();
    if (threadIdx.x == 0) {
        int bc = best_count[0], bi = best_index[0];
        for (int w = 1; w < kConsensusThreads / 32; ++w)
            if (best_count[w] > bc || (best_count[w] == bc && best_index[w] < bi)) { bc = best_count[w]; bi = best_index[w]; }
        winner = bc >= 0 ? bi : -1;
        stop = 0;
        float c[6];
        if (winner < 0 || !hypothesis(a, winner, c))
            for (int k = 0; k < 6; ++k) c[k] = 0.0f;
        for (int k = 0; k < 6; ++k) coef[k] = c[k];
    }
    __syncthreads();
    // refits
    for (int t = 0; t < a.n_tol && winner >= 0; ++t) {
        float x[12] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        const float tol2t = a.tol[t] * a.tol[t];
        const float c0 = coef[0], c1 = coef[1], c2 = coef[2], c3 = coef[3], c4 = coef[4], c5 = coef[5];
        for (int i = threadIdx.x; i < a.nodes; i += kConsensusThreads) {
            float u, v;
            if (!node_total(a, i, u, v)) continue;
            const float2 p = a.xy[i];
            const float du = c0 + c1 * p.x + c2 * p.y - u, dv = c3 + c4 * p.x + c5 * p.y - v;
            if (!(du * du + dv * dv <= tol2t)) continue;
            x[0] += 1.0f; x[1] += p.x; x[2] += p.y; x[3] += p.x * p.x; x[4] += p.x * p.y; x[5] += p.y * p.y;
            x[6] += u; x[7] += p.x * u; x[8] += p.y * u; x[9] += v; x[10] += p.x * v; x[11] += p.y * v;
        }
        block_sum<12>(x, red);
        if (threadIdx.x == 0) {
            const double *r = red[0];
            double c[6];
            const double m[3][3] = {{r[0], r[1], r[2]}, {r[1], r[3], r[4]}, {r[2], r[4], r[5]}};
            const double b[2][3] = {{r[6], r[7], r[8]}, {r[9], r[10], r[11]}};
            const double scale = r[0] * r[3] * r[5] + 1e-300;
            if (r[0] < 3.0 || !solve3<double>(m, b, 1e-12 * scale, c)) {
                stop = 1;
            } else {
                for (int k = 0; k < 6; ++k) coef[k] = (float)c[k];
            }
        }
        __syncthreads();
        if (stop) break;
    }
    // fitted field (winner < 0: no usable hypothesis, totals kept)
    for (int i = threadIdx.x; i < a.nodes; i += kConsensusThreads) {
        float u, v;
        node_total(a, i, u, v);
        if (winner >= 0) {
            const float2 p = a.xy[i];
            u = coef[0] + coef[1] * p.x + coef[2] * p.y;
            v = coef[3] + coef[4] * p.x + coef[5] * p.y;
        }
        const size_t row = (size_t)i * a.ldp;
        a.base[row] = u / a.scale;
        a.base[row + 3] = v / a.scale;
    }
}

// Subsets to reseed: not converged (status 0) or converged below the ZNCC
// threshold (-2), among usable subsets; mask / activity 1 for those, 0 else,
// and their count.
// With `list`, the picked indices are also appended to it (one atomicAdd
// per warp; the order across warps is arbitrary).
__global__ void reseed_select_kernel(const float *state, int row_floats, const uint8_t *usable, int count,
                                     uint8_t *mask, uint32_t *active, unsigned *counter, int *list) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool pick = false;
    if (i < count) {
        const float status = state[(size_t)i * row_floats + 6];
        pick = (status == 0.0f || status == -2.0f) && (!usable || usable[i]);
        mask[i] = pick ? 1 : 0;
        active[i] = pick ? 1u : 0u;
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, pick);
    const unsigned votes = __popc(ballot);
    const int lane = threadIdx.x & 31;
    unsigned base = 0u;
    if (lane == 0 && votes && counter) base = atomicAdd(counter, votes);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (list && pick) list[base + __popc(ballot & ((1u << lane) - 1u))] = i;
}

// dst row i = src row i where mask[i] (rows of row_floats floats).
__global__ void merge_rows_kernel(const float *src, const uint8_t *mask, int count, int row_floats, float *dst) {
    const long long n = (long long)count * row_floats;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        if (mask[k / row_floats]) dst[k] = src[k];
}

// Lattice rows from solved node subsets: node (lx, ly) is grid subset
// (lx step, ly step); where its affine state converged (status >= 1, finite
// parameters) its row of `pred` becomes the solved warp in the network's
// normalised layout, translations relative to `base` (when non-NULL), so that
// lattice_seed_kernel reproduces the solved warp at the node.  Other rows keep
// the network's prediction.
__global__ void node_rows_kernel(const float *state, int grid_w, int grid_h, int step, int lattice_w, int lattice_h,
                                 float *pred, const float *base, int ldp, float translation_scale,
                                 float gradient_scale) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= lattice_w * lattice_h) return;
    const int gx = (node % lattice_w) * step, gy = (node / lattice_w) * step;
    if (gx >= grid_w || gy >= grid_h) return;
    const float4 *st = reinterpret_cast<const float4 *>(state + ((size_t)gy * grid_w + gx) * 8);
    const float4 s0 = st[0], s1 = st[1];
    const bool ok = s1.z >= 1.0f && isfinite(s0.x) && isfinite(s0.y) && isfinite(s0.z) && isfinite(s0.w) &&
                    isfinite(s1.x) && isfinite(s1.y);
    if (!ok) return;
    float *row = pred + (size_t)node * ldp;
    const float bu = base ? base[(size_t)node * ldp] : 0.0f, bv = base ? base[(size_t)node * ldp + 3] : 0.0f;
    row[0] = s0.x / translation_scale - bu;
    row[1] = s0.y * gradient_scale;
    row[2] = s0.z * gradient_scale;
    row[3] = s0.w / translation_scale - bv;
    row[4] = s1.x * gradient_scale;
    row[5] = s1.y * gradient_scale;
}

// Direct 3x3 stride-2 convolution of the 2-channel input layer with 32
// outputs, bias and ReLU, for inference: one output pixel per thread, the 18
// input taps in registers and the weights as constant operands of the FMAs
// (kernel parameters), so the layer reads its input once and writes its BF16
// output once, with no im2col operand and none of the GEMM's K padding.
// FP32 accumulation over k = (ky, kx, ci) in order, bias added after the sum,
// as the GEMM epilogue does.
__global__ void __launch_bounds__(256) conv_c2_direct_kernel(NnConvShape s, const uint32_t *__restrict__ x,
                                                             NnConv1Weights p, uint4 *__restrict__ y) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= s.B * s.OH * s.OW) return;
    const int ox = m % s.OW, t = m / s.OW, oy = t % s.OH, b = t / s.OH;
    float in[18];
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
        const int ky = tap / 3, kx = tap - 3 * ky;
        const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
        const uint32_t v = (iy >= 0 && iy < s.H && ix >= 0 && ix < s.W) ? __ldg(x + ((size_t)b * s.H + iy) * s.W + ix) : 0u;
        in[2 * tap] = __uint_as_float(v << 16);             // channel 0 (low half)
        in[2 * tap + 1] = __uint_as_float(v & 0xffff0000u);  // channel 1 (high half)
    }
    uint4 *row = y + (size_t)m * 4;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint32_t packed[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            float r[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int co = q * 8 + h * 2 + e;
                float acc = 0.0f;
#pragma unroll
                for (int k = 0; k < 18; ++k) acc = fmaf(p.w[co][k], in[k], acc);
                r[e] = fmaxf(acc + p.bias[co], 0.0f);
            }
            const __nv_bfloat162 v2 = __floats2bfloat162_rn(r[0], r[1]);
            packed[h] = *reinterpret_cast<const uint32_t *>(&v2);
        }
        row[q] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
    }
}

unsigned blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

cudaError_t launch_nn_patches(const NnPatchArgs &a, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    patch_kernel<<<a.count, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_nn_im2col(const NnConvShape &sh, const void *x, void *A, cudaStream_t s) {
    const long long n = (long long)sh.B * sh.OH * sh.OW * sh.Kp;
    const bool aligned = (reinterpret_cast<uintptr_t>(x) & 15) == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0;
    if (sh.C % 8 == 0 && sh.Kp % 8 == 0 && aligned && n / 8 < (1ll << 31)) {
        im2col_vec_kernel<<<blocks(n / 8, 256), 256, 0, s>>>(sh, static_cast<const uint4 *>(x), static_cast<uint4 *>(A));
        return cudaGetLastError();
    }
    if (sh.C == 2 && sh.Kp % 8 == 0 && sh.Kp >= 24 && aligned && (long long)sh.B * sh.OH * sh.OW < (1ll << 31)) {
        im2col_c2_kernel<<<blocks((long long)sh.B * sh.OH * sh.OW, 256), 256, 0, s>>>(
            sh, static_cast<const uint32_t *>(x), static_cast<uint4 *>(A));
        return cudaGetLastError();
    }
    im2col_kernel<<<blocks(n, 256), 256, 0, s>>>(sh, static_cast<const __nv_bfloat16 *>(x), static_cast<__nv_bfloat16 *>(A));
    return cudaGetLastError();
}

cudaError_t launch_nn_dgrad_gather(const NnConvShape &sh, const void *dz, void *G, cudaStream_t s) {
    const long long n = (long long)sh.B * sh.H * sh.W * 9 * sh.Cout;
    const bool aligned = (reinterpret_cast<uintptr_t>(dz) & 15) == 0 && (reinterpret_cast<uintptr_t>(G) & 15) == 0;
    if (sh.Cout % 8 == 0 && aligned && n / 8 < (1ll << 31)) {
        dgrad_gather_vec_kernel<<<blocks(n / 8, 256), 256, 0, s>>>(sh, static_cast<const uint4 *>(dz),
                                                                    static_cast<uint4 *>(G));
        return cudaGetLastError();
    }
    dgrad_gather_kernel<<<blocks(n, 256), 256, 0, s>>>(sh, static_cast<const __nv_bfloat16 *>(dz),
                                                      static_cast<__nv_bfloat16 *>(G));
    return cudaGetLastError();
}

cudaError_t launch_nn_transpose(const void *src, int R, int C, int ld_src, void *dst, int Rp, int Cp, cudaStream_t s) {
    dim3 grid((Rp + 31) / 32, (Cp + 31) / 32), block(32, 8);
    transpose_kernel<<<grid, block, 0, s>>>(static_cast<const __nv_bfloat16 *>(src), R, C, ld_src,
                                            static_cast<__nv_bfloat16 *>(dst), Rp, Cp);
    return cudaGetLastError();
}

cudaError_t launch_nn_relu_backward(const float *dy, int ld, const void *y, void *dz, long long rows, int C,
                                    cudaStream_t s) {
    relu_backward_kernel<<<blocks(rows * C, 256), 256, 0, s>>>(dy, ld, static_cast<const __nv_bfloat16 *>(y),
                                                               static_cast<__nv_bfloat16 *>(dz), rows, C);
    return cudaGetLastError();
}

cudaError_t launch_nn_bias_grad(const float *dy, int ld, const void *y, long long rows, int C, float *db,
                                cudaStream_t s) {
    bias_grad_kernel<<<C, 256, 0, s>>>(dy, ld, static_cast<const __nv_bfloat16 *>(y), rows, C, db);
    return cudaGetLastError();
}

cudaError_t launch_nn_relu_bias_backward(const float *dy, int ld, const void *y, long long rows, int C, void *dz,
                                        void *dzt, float *partial, float *db, cudaStream_t s) {
    const bool pow2 = C >= 4 && C <= 256 && (C & (C - 1)) == 0;
    const long long tiles = (rows + 63) / 64;
    if (!pow2 || rows <= 0 || ld < C || ld % 4 || !dy || !dz || !partial || !db || (dzt && rows % 8) ||
        tiles >= (1ll << 31) || ((reinterpret_cast<uintptr_t>(dy) | reinterpret_cast<uintptr_t>(dzt)) & 15) ||
        ((reinterpret_cast<uintptr_t>(y) | reinterpret_cast<uintptr_t>(dz)) & 7))
        return cudaErrorInvalidValue;
    const size_t smem = 256 * sizeof(float4) + (size_t)C * 72 * sizeof(__nv_bfloat16);
    static thread_local int configured_device = -1;
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) return err;
    if (configured_device != device) {
        err = cudaFuncSetAttribute(relu_bias_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(256 * sizeof(float4) + 256 * 72 * sizeof(__nv_bfloat16)));
        if (err != cudaSuccess) return err;
        configured_device = device;
    }
    relu_bias_backward_kernel<<<(unsigned)tiles, 256, smem, s>>>(dy, ld, static_cast<const __nv_bfloat16 *>(y), rows,
                                                                 C, static_cast<__nv_bfloat16 *>(dz),
                                                                 static_cast<__nv_bfloat16 *>(dzt), partial,
                                                                 (int)tiles);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    bias_reduce_kernel<<<C, 256, 0, s>>>(partial, (int)tiles, db);
    return cudaGetLastError();
}

cudaError_t launch_nn_splitk_bias_relu(const float *partial, int splits, long long rows, int N, long long split_stride,
                                      const float *bias, int relu, void *y, cudaStream_t s) {
    if (!partial || !y || splits < 1 || rows <= 0 || N <= 0 || N % 4 || split_stride < rows * N ||
        split_stride % 4 || ((reinterpret_cast<uintptr_t>(partial) & 15) | (reinterpret_cast<uintptr_t>(y) & 7)))
        return cudaErrorInvalidValue;
    const long long n = rows * N / 4;
    splitk_bias_relu_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(partial, splits, rows, N, split_stride, bias,
                                                                        relu, static_cast<__nv_bfloat16 *>(y));
    return cudaGetLastError();
}

cudaError_t launch_nn_im2col_t(const NnConvShape &sh, const void *x, void *At, int Kt, cudaStream_t s) {
    const long long M = (long long)sh.B * sh.OH * sh.OW;
    if (M <= 0 || M % 8 || Kt <= 0 || Kt % 64 || M >= (1ll << 31) || (long long)Kt * M >= (1ll << 40) ||
        ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(At)) & 15))
        return cudaErrorInvalidValue;
    // Only the 64-row tiles that hold rows k < 9 C are written; the rows
    // beyond stay as the caller keeps them (zero).
    const int live = std::min(Kt, (9 * sh.C + 63) / 64 * 64);
    dim3 grid((unsigned)((M + 63) / 64), (unsigned)(live / 64));
    im2col_t_kernel<<<grid, 256, 0, s>>>(sh, static_cast<const __nv_bfloat16 *>(x), static_cast<__nv_bfloat16 *>(At),
                                         Kt);
    return cudaGetLastError();
}

cudaError_t launch_nn_splitk_reduce(const float *partial, int splits, int Kp_rows, int N, int Kp, float *out,
                                    cudaStream_t s) {
    splitk_reduce_kernel<<<blocks((long long)N * Kp, 256), 256, 0, s>>>(partial, splits, Kp_rows, N, Kp, out);
    return cudaGetLastError();
}

cudaError_t launch_nn_adam_many(const NnAdamMany &a, cudaStream_t s) {
    if (a.n < 1 || a.n > kMaxAdamTensors) return cudaErrorInvalidValue;
    const long long total = a.offset[a.n];
    if (total <= 0) return cudaSuccess;
    adam_many_kernel<<<blocks(total, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_nn_adam(const NnAdamArgs &a, cudaStream_t s) {
    adam_kernel<<<blocks(a.count, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_nn_pack_weights(const float *w, int Cout, int Cin, int Kp, void *wb, void *wt, int Kt,
                                   cudaStream_t s) {
    pack_weights_kernel<<<blocks((long long)Cout * Kp, 256), 256, 0, s>>>(
        w, Cout, Cin, Kp, static_cast<__nv_bfloat16 *>(wb), static_cast<__nv_bfloat16 *>(wt), Kt);
    return cudaGetLastError();
}

cudaError_t launch_nn_regression_loss(const float *pred, int ldp, const float *target, int outputs, int B, void *grad,
                                      float *grad_f32, int ldg, float *loss, cudaStream_t s) {
    regression_loss_kernel<<<1, 1024, 0, s>>>(pred, ldp, target, outputs, B, static_cast<__nv_bfloat16 *>(grad),
                                             grad_f32, ldg, loss);
    return cudaGetLastError();
}

cudaError_t launch_nn_lattice_seeds(const NnLatticeArgs &a, cudaStream_t s) {
    const long long n = (long long)a.grid_w * a.grid_h;
    if (n <= 0) return cudaSuccess;
    lattice_seed_kernel<<<blocks(n, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_nn_consensus(const NnConsensusArgs &a, cudaStream_t s) {
    if (a.nodes <= 0) return cudaSuccess;
    consensus_kernel<<<1, kConsensusThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_nn_reseed_select(const float *state, int row_floats, const uint8_t *usable, int count,
                                    uint8_t *mask, uint32_t *active, unsigned *counter, int *list, cudaStream_t s) {
    if (list && !counter) return cudaErrorInvalidValue;
    if (counter) {
        const cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) return e;
    }
    if (count <= 0) return cudaSuccess;
    reseed_select_kernel<<<blocks(count, 256), 256, 0, s>>>(state, row_floats, usable, count, mask, active, counter,
                                                            list);
    return cudaGetLastError();
}

cudaError_t launch_nn_merge_rows(const float *src, const uint8_t *mask, int count, int row_floats, float *dst,
                                 cudaStream_t s) {
    const long long n = (long long)count * row_floats;
    if (n <= 0) return cudaSuccess;
    const unsigned g = blocks(n, 256);
    merge_rows_kernel<<<g < 152u * 16u ? g : 152u * 16u, 256, 0, s>>>(src, mask, count, row_floats, dst);
    return cudaGetLastError();
}

cudaError_t launch_nn_node_rows(const float *state, int grid_w, int grid_h, int step, int lattice_w, int lattice_h,
                                float *pred, const float *base, int ldp, float translation_scale, float gradient_scale,
                                cudaStream_t s) {
    const long long n = (long long)lattice_w * lattice_h;
    if (n <= 0) return cudaSuccess;
    node_rows_kernel<<<blocks(n, 256), 256, 0, s>>>(state, grid_w, grid_h, step, lattice_w, lattice_h, pred, base, ldp,
                                                   translation_scale, gradient_scale);
    return cudaGetLastError();
}

cudaError_t launch_nn_conv_c2_direct(const NnConvShape &sh, const void *x, const NnConv1Weights &w, void *y,
                                     cudaStream_t s) {
    const long long rows = (long long)sh.B * sh.OH * sh.OW;
    if (rows <= 0) return cudaSuccess;
    conv_c2_direct_kernel<<<blocks(rows, 256), 256, 0, s>>>(sh, static_cast<const uint32_t *>(x), w,
                                                            static_cast<uint4 *>(y));
    return cudaGetLastError();
}

}  // namespace gbdic
