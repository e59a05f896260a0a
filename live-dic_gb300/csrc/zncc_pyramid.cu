// Final ZNCC (reference: shaders/affine_zncc.wgsl:57-99) and the pyramid /
// temporal kernels (reference: shaders/full_pyramid.wgsl).
#include "gbdic_common.cuh"
#include "gbdic_kernels.h"

namespace gbdic {

namespace {

// ------------------------------------------------------------ final ZNCC
// 64 lanes per subset (two subsets per 128-thread CTA); sums over the valid
// warped pixels of [f, g, f^2, g^2, f g, count], pairwise tree over lanes.
template <int INTERP>
__global__ void __launch_bounds__(128) final_zncc_kernel(ZnccArgs a) {
    __shared__ float red[2][6][64];
    const int sub = threadIdx.x >> 6, lane = threadIdx.x & 63;
    const int index = blockIdx.x * 2 + sub;
    const bool exists = index < a.count;
    const int sidx = exists ? index : 0;
    const float4 *st = reinterpret_cast<const float4 *>(a.state + (size_t)sidx * 8);
    const float4 p = st[0], q = st[1];
    const bool active = exists && q.z == 1.0f;
    float s[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (active) {
        const int S = a.S;
        const int gx = sidx % a.grid_w, gy = sidx / a.grid_w;
        const float half = ((float)S - 1.0f) * 0.5f;
        for (int k = lane; k < S * S; k += 64) {
            const int col = k % S, row = k / S;
            const int px = gx * a.stride + col, py = gy * a.stride + row;
            const float lx = (float)col - half, ly = (float)row - half;
            const float tx = (float)px + (p.x + fmaf(p.y, lx, p.z * ly));
            const float ty = (float)py + (p.w + fmaf(q.x, lx, q.y * ly));
            if (tx >= 2.0f && ty >= 2.0f && tx <= (float)(a.W - 3) && ty <= (float)(a.H - 3)) {
                const float g = sample_target<INTERP, true>(a.coef, a.img, a.W, a.H, tx, ty);
                const float f = a.plane[(size_t)py * a.W + px].x;
                s[0] = s[0] + f;
                s[1] = s[1] + g;
                s[2] = fmaf(f, f, s[2]);
                s[3] = fmaf(g, g, s[3]);
                s[4] = fmaf(f, g, s[4]);
                s[5] = s[5] + 1.0f;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) red[sub][k][lane] = s[k];
    __syncthreads();
    if (lane < 32) {
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            float v = red[sub][k][lane] + red[sub][k][lane + 32];
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_down_sync(kFullMask, v, off);
            s[k] = v;
        }
    }
    if (!exists || lane != 0) return;
    if (!active) {
        a.out[index] = -2.0f;
        return;
    }
    const float n = s[5], nn = fmaxf(n, 1.0f);
    const float vf = s[2] - s[0] * s[0] / nn;
    const float vg = s[3] - s[1] * s[1] / nn;
    if (n == (float)(a.S * a.S) && vf > 1e-9f && vg > 1e-9f) {
        const float r = (s[4] - s[0] * s[1] / n) / sqrtf(vf * vg);
        a.out[index] = fminf(fmaxf(r, -1.0f), 1.0f);
    } else {
        a.out[index] = -2.0f;
    }
}

// ------------------------------------------------------------ reduction
// full_pyramid.wgsl:218-249: exact integer 5x5 [1 4 6 4 1]^2 sum over the
// reflected source, truncating division by 256; 16x16 outputs per CTA
// from a 36x36 byte footprint staged in shared memory.
// Separable form of the exact integer 5x5 reduction: the [1 4 6 4 1] sum of
// every footprint row at the even columns, then the same sum down the rows.
// Integer sums are exact in any order, so the output equals the 5x5 form.
// One CTA: 64 x 16 outputs from a (2*16 + 3) x (2*64 + 3) byte footprint.
constexpr int kRX = 64, kRY = 16;
constexpr int kFX = 2 * kRX + 3, kFY = 2 * kRY + 3;

__global__ void __launch_bounds__(256) reduce_half_kernel(const uint8_t *__restrict__ src, int W, int H,
                                                          uint8_t *__restrict__ dst) {
    __shared__ uint8_t tile[kFY * kFX];
    __shared__ unsigned rows[kFY * kRX];
    const int W2 = W / 2, H2 = H / 2;
    const int fx0 = 2 * (int)blockIdx.x * kRX - 2, fy0 = 2 * (int)blockIdx.y * kRY - 2;
    const int tid = threadIdx.x;
    const bool interior = fx0 >= 0 && fy0 >= 0 && fx0 + kFX <= W && fy0 + kFY <= H;
    for (int i = tid; i < kFY * kFX; i += 256) {
        const int r = i / kFX, c = i - r * kFX;
        const int sx = interior ? fx0 + c : mirror_clamp(fx0 + c, W);
        const int sy = interior ? fy0 + r : mirror_clamp(fy0 + r, H);
        tile[i] = __ldg(src + (size_t)sy * W + sx);
    }
    __syncthreads();
    for (int i = tid; i < kFY * kRX; i += 256) {
        const int r = i / kRX, c = i - r * kRX;
        const uint8_t *t = tile + r * kFX + 2 * c;
        rows[i] = (unsigned)t[0] + 4u * t[1] + 6u * t[2] + 4u * t[3] + (unsigned)t[4];
    }
    __syncthreads();
    for (int i = tid; i < kRY * kRX; i += 256) {
        const int y = i / kRX, c = i - y * kRX;
        const unsigned *v = rows + 2 * y * kRX + c;
        const unsigned acc = v[0] + 4u * v[kRX] + 6u * v[2 * kRX] + 4u * v[3 * kRX] + v[4 * kRX];
        const int X = (int)blockIdx.x * kRX + c, Y = (int)blockIdx.y * kRY + y;
        if (X < W2 && Y < H2) dst[(size_t)Y * W2 + X] = (uint8_t)(acc / 256u);
    }
}

// ------------------------------------------------------------ seed transfer
// full_pyramid.wgsl:251-308
__device__ void accumulate_seed(const SeedArgs &a, int sidx, float weight, float spx, float spy,
                                float dpx, float dpy, float tscale, float *acc, float &wsum) {
    const int ss = state_stride(a.model);
    const float *s = a.source + (size_t)sidx * ss;
    const float status = s[status_slot(a.model)];
    if (status < -0.5f) return;
    const float dx = dpx - spx, dy = dpy - spy;
    float tu = fmaf(s[2], dy, fmaf(s[1], dx, s[0]));
    float tv = fmaf(s[5], dy, fmaf(s[4], dx, s[3]));
    float ux = s[1], uy = s[2], vx = s[4], vy = s[5];
    if (a.model == kModelQuadratic) {
        tu = tu + fmaf(s[8], 0.5f * dy * dy, fmaf(s[7], dx * dy, s[6] * (0.5f * dx * dx)));
        tv = tv + fmaf(s[11], 0.5f * dy * dy, fmaf(s[10], dx * dy, s[9] * (0.5f * dx * dx)));
        ux = ux + fmaf(s[7], dy, s[6] * dx);
        uy = uy + fmaf(s[8], dy, s[7] * dx);
        vx = vx + fmaf(s[10], dy, s[9] * dx);
        vy = vy + fmaf(s[11], dy, s[10] * dx);
    }
    acc[0] = fmaf(weight * tu, tscale, acc[0]);
    acc[1] = fmaf(weight, ux, acc[1]);
    acc[2] = fmaf(weight, uy, acc[2]);
    acc[3] = fmaf(weight * tv, tscale, acc[3]);
    acc[4] = fmaf(weight, vx, acc[4]);
    acc[5] = fmaf(weight, vy, acc[5]);
    if (a.model == kModelQuadratic) {
        const float cs = 1.0f / tscale;
        for (int k = 6; k < 12; ++k) acc[k] = fmaf(weight * s[k], cs, acc[k]);
    }
    wsum = wsum + weight;
}

// full_pyramid.wgsl:310-395: bilinear blend of the permitted source corners
// at the destination centre (normalised); returns the weight sum.  `lx`,
// `ly` receive the lower source corner.
__device__ float interpolate_seed(const SeedArgs &a, int i, unsigned perm, float (&acc)[12], int &lx, int &ly) {
    for (int k = 0; k < 12; ++k) acc[k] = 0.0f;
    float wsum = 0.0f;
    const int dxg = i % a.dst_grid_w, dyg = i / a.dst_grid_w;
    const float soff = (1.0f - a.src_scale) * 0.5f, doff = (1.0f - a.dst_scale) * 0.5f;
    const float dcx = fmaf(a.subset_stride, (float)dxg, 0.5f * a.subset_size);
    const float dcy = fmaf(a.subset_stride, (float)dyg, 0.5f * a.subset_size);
    const float scx = fmaf(a.dst_scale, dcx, doff - soff) / a.src_scale;
    const float scy = fmaf(a.dst_scale, dcy, doff - soff) / a.src_scale;
    const float gxf = (scx - 0.5f * a.subset_size) / a.subset_stride;
    const float gyf = (scy - 0.5f * a.subset_size) / a.subset_stride;
    const int maxx = a.src_grid_w - 2 > 0 ? a.src_grid_w - 2 : 0;
    const int maxy = a.src_grid_h - 2 > 0 ? a.src_grid_h - 2 : 0;
    lx = clampi((int)floorf(gxf), 0, maxx);
    ly = clampi((int)floorf(gyf), 0, maxy);
    const float fx = fminf(fmaxf(gxf - (float)lx, 0.0f), 1.0f);
    const float fy = fminf(fmaxf(gyf - (float)ly, 0.0f), 1.0f);
    const float tscale = a.src_scale / a.dst_scale;
    for (int corner = 0; corner < 4; ++corner) {
        if ((perm & (1u << corner)) == 0u) continue;
        const int ox = corner & 1, oy = corner >> 1;
        const int sx = lx + ox, sy = ly + oy;
        if (sx >= a.src_grid_w || sy >= a.src_grid_h) continue;
        const float wx = ox ? fx : 1.0f - fx, wy = oy ? fy : 1.0f - fy;
        const float spx = fmaf(a.subset_stride, (float)sx, 0.5f * a.subset_size);
        const float spy = fmaf(a.subset_stride, (float)sy, 0.5f * a.subset_size);
        accumulate_seed(a, sy * a.src_grid_w + sx, wx * wy, spx, spy, scx, scy, tscale, acc, wsum);
    }
    const unsigned fallback = perm >> 5;
    if (wsum == 0.0f && fallback != 0u) {
        const int sidx = (int)fallback - 1;
        const float st = a.source[(size_t)sidx * state_stride(a.model) + status_slot(a.model)];
        if (st >= 0.5f) {
            const int sx = sidx % a.src_grid_w, sy = sidx / a.src_grid_w;
            const float spx = fmaf(a.subset_stride, (float)sx, 0.5f * a.subset_size);
            const float spy = fmaf(a.subset_stride, (float)sy, 0.5f * a.subset_size);
            accumulate_seed(a, sidx, 1.0f, spx, spy, scx, scy, tscale, acc, wsum);
        }
    }
    if (wsum > 0.0f)
        for (int k = 0; k < 12; ++k) acc[k] = acc[k] / wsum;
    return wsum;
}

// full_pyramid.wgsl:397-450 (transfer_seed, transfer_seed_roi and, with a
// projection counter, project_temporal_seed).
__global__ void transfer_seed_kernel(SeedArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool projected = false;
    if (i < a.dst_count) {
        const unsigned perm = a.links ? a.links[i] : 31u;
        float acc[12];
        int lx, ly;
        const float wsum = interpolate_seed(a, i, perm, acc, lx, ly);
        float4 *d = reinterpret_cast<float4 *>(a.seed + (size_t)i * state_stride(a.model));
        d[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        if (a.model == kModelQuadratic) {
            d[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
            d[2] = make_float4(acc[8], acc[9], acc[10], acc[11]);
            d[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            d[1] = make_float4(acc[4], acc[5], 0.0f, 0.0f);
        }
        projected = wsum > 0.0f && (perm & 16u) != 0u;
        float *status = a.seed + (size_t)i * state_stride(a.model) + status_slot(a.model);
        if (a.track) *status = wsum >= 0.99999f ? 0.0f : -1.0f;
        if (a.mark_missing && wsum == 0.0f) *status = -1.0f;
        if (a.track && a.projected && !projected) *status = -1.0f;
        a.active[i] = (perm >> 4) & 1u;
    }
    if (a.projected) {
        const int count = __syncthreads_count(projected);
        if (threadIdx.x == 0 && count > 0) atomicAdd(a.projected, (unsigned)count);
    }
}

// full_pyramid.wgsl:452-506.  Runs after the ordinary coarse-to-fine
// transfer into `seed` (with availability markers); `source` is the coarse
// accepted history, `history` the fine one.
__global__ void refine_temporal_seed_kernel(SeedArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.dst_count) return;
    if (a.active[i] == 0u) return;
    const unsigned age = a.history_ages[i];
    if (age == 0xffffffffu || age > a.max_age) return;
    const int ss = state_stride(a.model);
    float *seed = a.seed + (size_t)i * ss;
    if (seed[status_slot(a.model)] < -0.5f) return;
    const unsigned perm = a.links ? a.links[i] : 31u;
    float predicted[12];
    int lx, ly;
    // The lower corner is the one interpolate_seed uses; every permitted
    // corner's coarse history must date from the fine history's frame.
    const float wsum = interpolate_seed(a, i, perm, predicted, lx, ly);
    for (int corner = 0; corner < 4; ++corner) {
        if ((perm & (1u << corner)) == 0u) continue;
        const int sx = lx + (corner & 1), sy = ly + (corner >> 1);
        if (sx >= a.src_grid_w || sy >= a.src_grid_h) continue;
        if (a.source_ages[sy * a.src_grid_w + sx] != age) return;
    }
    if (wsum < 0.99999f) return;
    const float *h = a.history + (size_t)i * ss;
    // a = (tu, ux, uy, tv), b.xy = (vx, vy); quadratic: b.zw and c are the
    // curvature terms.  Markers and iteration slots keep the transfer's.
    const int n = a.model == kModelQuadratic ? 12 : 6;
    for (int k = 0; k < n; ++k) seed[k] = h[k] + (seed[k] - predicted[k]);
}

// ------------------------------------------------------------ temporal
// full_pyramid.wgsl:83-122 velocity prediction into `prediction`.
__global__ void temporal_predict_kernel(TemporalArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool predicted = false;
    if (i < a.count) {
        const int ss = state_stride(a.model), sat = status_slot(a.model);
        const int svec = a.model == kModelQuadratic ? 12 : 4;
        const float *c = a.history + (size_t)i * ss, *p = a.prev_history + (size_t)i * ss;
        float *o = a.prediction + (size_t)i * ss;
        predicted = a.ages[i] == 0u && a.prev_ages[i] == 0u && c[sat] >= 0.5f && p[sat] >= 0.5f;
        for (int k = 0; k < ss; ++k) o[k] = predicted ? fmaf(2.0f, c[k], -p[k]) : c[k];
        for (int k = 0; k < 4; ++k) o[svec + k] = c[svec + k];
        if (a.model != kModelQuadratic && predicted) {
            o[4] = fmaf(2.0f, c[4], -p[4]);
            o[5] = fmaf(2.0f, c[5], -p[5]);
        }
    }
    const int count = __syncthreads_count(predicted);
    if (threadIdx.x == 0 && count > 0) atomicAdd(a.counters + 2, (unsigned)count);
}

// full_pyramid.wgsl:126-148
__global__ void temporal_save_previous_kernel(TemporalArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    const int ss = state_stride(a.model), sat = status_slot(a.model);
    const float rs = a.raw[(size_t)i * ss + sat], fs = a.output[(size_t)i * ss + sat];
    if ((rs == 1.0f || rs == 2.0f) && (fs == 1.0f || fs == 2.0f)) {
        for (int k = 0; k < ss; ++k) a.prev_history[(size_t)i * ss + k] = a.history[(size_t)i * ss + k];
        a.prev_ages[i] = a.ages[i];
    } else if (a.prev_ages[i] != 0xffffffffu) {
        const unsigned age = a.prev_ages[i];
        a.prev_ages[i] = (age < 0xfffffffdu ? age : 0xfffffffdu) + 1u;
    }
}

// full_pyramid.wgsl:508-575
__global__ void temporal_merge_kernel(TemporalArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool accepted = false, expired = false;
    if (i < a.count) {
        const int ss = state_stride(a.model), sat = status_slot(a.model);
        const float rs = a.raw[(size_t)i * ss + sat], fs = a.output[(size_t)i * ss + sat];
        const bool raw_ok = rs == 1.0f || rs == 2.0f, fin_ok = fs == 1.0f || fs == 2.0f;
        if (fin_ok && (a.use_filtered || raw_ok)) {
            const float *src = a.use_filtered ? a.output : a.raw;
            for (int k = 0; k < ss; ++k) a.history[(size_t)i * ss + k] = src[(size_t)i * ss + k];
            a.ages[i] = 0u;
            accepted = true;
        } else if (a.ages[i] != 0xffffffffu) {
            const unsigned age = (a.ages[i] < 0xfffffffdu ? a.ages[i] : 0xfffffffdu) + 1u;
            a.ages[i] = age;
            if (age > a.max_age) {
                a.history[(size_t)i * ss + sat] = -1.0f;
                expired = age == a.max_age + 1u;
            }
        }
    }
    const int na = __syncthreads_count(accepted);
    const int ne = __syncthreads_count(expired);
    if (threadIdx.x == 0 && a.counters) {
        if (na > 0) atomicAdd(a.counters + 1, (unsigned)na);
        if (ne > 0 && a.report_expiry) atomicAdd(a.counters + 3, (unsigned)ne);
    }
}

}  // namespace

cudaError_t launch_final_zncc(const ZnccArgs &a, cudaStream_t stream) {
    if (a.count <= 0) return cudaSuccess;
    const int grid = (a.count + 1) / 2;
    switch (a.interp) {
    case kInterpLinear: final_zncc_kernel<kInterpLinear><<<grid, 128, 0, stream>>>(a); break;
    case kInterpKeys: final_zncc_kernel<kInterpKeys><<<grid, 128, 0, stream>>>(a); break;
    default: final_zncc_kernel<kInterpBspline><<<grid, 128, 0, stream>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_reduce_half(const uint8_t *src, int W, int H, uint8_t *dst, cudaStream_t stream) {
    const int W2 = W / 2, H2 = H / 2;
    if (W2 <= 0 || H2 <= 0) return cudaSuccess;
    reduce_half_kernel<<<dim3((W2 + kRX - 1) / kRX, (H2 + kRY - 1) / kRY), 256, 0, stream>>>(src, W, H, dst);
    return cudaGetLastError();
}

cudaError_t launch_transfer_seed(const SeedArgs &a, cudaStream_t stream) {
    if (a.dst_count <= 0) return cudaSuccess;
    transfer_seed_kernel<<<(a.dst_count + 255) / 256, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_refine_temporal_seed(const SeedArgs &a, cudaStream_t stream) {
    if (a.dst_count <= 0) return cudaSuccess;
    refine_temporal_seed_kernel<<<(a.dst_count + 255) / 256, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_temporal_predict(const TemporalArgs &a, cudaStream_t stream) {
    temporal_predict_kernel<<<(a.count + 255) / 256, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_temporal_save_previous(const TemporalArgs &a, cudaStream_t stream) {
    temporal_save_previous_kernel<<<(a.count + 255) / 256, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_temporal_merge(const TemporalArgs &a, cudaStream_t stream) {
    temporal_merge_kernel<<<(a.count + 255) / 256, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

namespace {

// Every subset seeded with the translation (shift[0], shift[1]) * inv_scale
// (zero gradients), active where ROI-selected.
__global__ void uniform_seed_kernel(float *seed, uint32_t *active, const uint8_t *selected, int count, int ss,
                                    const float *shift, float inv_scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float *s = seed + (size_t)i * ss;
    for (int k = 0; k < ss; ++k) s[k] = 0.0f;
    s[0] = shift[0] * inv_scale;
    s[3] = shift[1] * inv_scale;
    active[i] = selected ? (selected[i] ? 1u : 0u) : 1u;
}

}  // namespace

cudaError_t launch_uniform_seed(float *seed, uint32_t *active, const uint8_t *selected, int count, int model,
                                const float *shift, float inv_scale, cudaStream_t stream) {
    if (count <= 0) return cudaSuccess;
    uniform_seed_kernel<<<(count + 255) / 256, 256, 0, stream>>>(seed, active, selected, count, state_stride(model),
                                                                shift, inv_scale);
    return cudaGetLastError();
}

}  // namespace gbdic
