// Spatial seed propagation (reference: shaders/spatial_seed.wgsl).
//
// affine_frontier_kernel (spatial_seed.wgsl:268-309): every permitted subset
// that is not yet accepted takes the component-wise median of the
// first-order transports of its accepted 3x3 neighbours (t + grad . delta,
// delta = the neighbour-to-subset centre offset) as an affine seed.
//
// spatial_choose_kernel (spatial_seed.wgsl:65-190): one 64-thread CTA per
// subset scores up to 11 translation hypotheses (own, prior, the 8
// neighbours' translations, optionally their median) by ZNCC of the
// reference window against the bilinearly sampled target (every
// sample_step-th pixel), lane-strided partial sums and the pairwise tree of
// the reference, and keeps the best if it beats the own hypothesis by
// min_gain and moves it by more than min_displacement.
//
// Both read one immutable snapshot of states (8 floats per subset) and a
// permission word per subset (3x3 neighbour bits; bit 4 = the subset itself
// is ROI-selected and numerically admissible).
#include "gbdic_common.cuh"
#include "gbdic_kernels.h"

namespace gbdic {
namespace {

// Insertion sort then the mean of the two middle order statistics
// (spatial_seed.wgsl:40-52), including its odd-count form 0.5 (v + v).
__device__ float median_insertion(float *v, int n) {
    for (int i = 1; i < n; ++i) {
        const float value = v[i];
        int j = i;
        while (j > 0 && !(v[j - 1] <= value)) {
            v[j] = v[j - 1];
            --j;
        }
        v[j] = value;
    }
    return 0.5f * (v[(n - 1) / 2] + v[n / 2]);
}

__global__ void affine_frontier_kernel(FrontierArgs a) {
    const int index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= a.count) return;
    const uint32_t perm = a.permissions[index];
    if ((perm & 16u) == 0u) return;
    const float4 *snap = reinterpret_cast<const float4 *>(a.snapshot);
    if (snap[2 * index + 1].z >= 0.5f) return;
    const int gx = index % a.grid_w, gy = index / a.grid_w, gh = a.count / a.grid_w;
    float t0[9], g0[9], g1[9], t1[9], g2[9], g3[9];
    int count = 0;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            if (dx == 0 && dy == 0) continue;
            const int x = gx + dx, y = gy + dy;
            const int bit = (dy + 1) * 3 + dx + 1;
            if (x < 0 || y < 0 || x >= a.grid_w || y >= gh || (perm & (1u << bit)) == 0u) continue;
            const int nb = y * a.grid_w + x;
            const float4 p = snap[2 * nb], q = snap[2 * nb + 1];
            if ((a.permissions[nb] & 16u) == 0u || q.z != 1.0f) continue;
            const float ddx = (float)(-dx) * (float)a.stride, ddy = (float)(-dy) * (float)a.stride;
            t0[count] = p.x + (p.y * ddx + p.z * ddy);
            t1[count] = p.w + (q.x * ddx + q.y * ddy);
            g0[count] = p.y; g1[count] = p.z;
            g2[count] = q.x; g3[count] = q.y;
            ++count;
        }
    if (count == 0) return;
    float4 *seed = reinterpret_cast<float4 *>(a.seeds);
    const float m0 = median_insertion(t0, count), m1 = median_insertion(g0, count);
    const float m2 = median_insertion(g1, count), m3 = median_insertion(t1, count);
    const float m4 = median_insertion(g2, count), m5 = median_insertion(g3, count);
    seed[2 * index] = make_float4(m0, m1, m2, m3);
    seed[2 * index + 1] = make_float4(m4, m5, 0.0f, 0.0f);
    a.active[index] = 1u;
}

__device__ __forceinline__ float unorm(uint8_t b) { return (float)b / 255.0f; }

// 255 * bilinear(target / 255) - 128 at `x, y` (mix(a, b, t) = a (1 - t) + b t).
__device__ __forceinline__ float linear_sample(const uint8_t *img, int W, float x, float y) {
    const float fx = floorf(x), fy = floorf(y);
    const int ix = (int)fx, iy = (int)fy;
    const float tx = x - fx, ty = y - fy;
    const uint8_t *r0 = img + (size_t)iy * W + ix, *r1 = r0 + W;
    const float a = unorm(r0[0]), b = unorm(r0[1]), c = unorm(r1[0]), e = unorm(r1[1]);
    const float top = a * (1.0f - tx) + b * tx;
    const float bottom = c * (1.0f - tx) + e * tx;
    return 255.0f * (top * (1.0f - ty) + bottom * ty) - 128.0f;
}

__global__ void __launch_bounds__(64) spatial_choose_kernel(ChooseArgs a) {
    const int index = blockIdx.x;
    const int lane = threadIdx.x;
    if (index >= a.count) return;
    const uint32_t perm = a.permissions[index];
    if ((perm & 16u) == 0u) return;
    const float4 *snap = reinterpret_cast<const float4 *>(a.snapshot);
    if (a.failed_only && snap[2 * index + 1].z >= 0.5f) return;
    __shared__ float4 cand[11];
    __shared__ float4 sums[64];
    __shared__ float sum_g2[64];
    __shared__ float4 best;  // dx, dy, rho, own rho
    const int gx = index % a.grid_w, gy = index / a.grid_w, gh = a.count / a.grid_w;
    const float ownx = snap[2 * index].x, owny = snap[2 * index].w;
    if (lane == 0) {
        for (int k = 0; k < 11; ++k) cand[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        cand[0] = make_float4(ownx, owny, 1.0f, 0.0f);
        const float4 pr = a.prior ? reinterpret_cast<const float4 *>(a.prior)[2 * index] : make_float4(0, 0, 0, 0);
        cand[1] = make_float4(pr.x, pr.w, 1.0f, 0.0f);
        float us[9], vs[9];
        int n = 0, slot = 2;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int bit = (dy + 1) * 3 + dx + 1;
                const int x = gx + dx, y = gy + dy;
                const bool inside = x >= 0 && y >= 0 && x < a.grid_w && y < gh;
                if (inside && (perm & (1u << bit)) != 0u) {
                    const int nb = y * a.grid_w + x;
                    if ((a.permissions[nb] & 16u) != 0u) {
                        const float px = snap[2 * nb].x, py = snap[2 * nb].w;
                        if ((dx != 0 || dy != 0) && a.candidate_mode != 1) cand[slot] = make_float4(px, py, 1.0f, 0.0f);
                        if (snap[2 * nb + 1].z >= 0.5f) {
                            us[n] = px;
                            vs[n] = py;
                            ++n;
                        }
                    }
                }
                if (dx != 0 || dy != 0) ++slot;
            }
        if (a.candidate_mode != 0 && n > 0)
            cand[10] = make_float4(median_insertion(us, n), median_insertion(vs, n), 1.0f, 0.0f);
        best = make_float4(ownx, owny, -2.0f, -2.0f);
    }
    __syncthreads();
    const float ox = (float)(gx * a.stride), oy = (float)(gy * a.stride);
    const int side = (a.S + a.sample_step - 1) / a.sample_step;
    const int total = side * side;
    const float ftotal = (float)total;
    const float xmax = (float)(a.W - 3), ymax = (float)(a.H - 3);
    for (int k = 0; k < 11; ++k) {
        const float4 c = cand[k];
        const float minx = ox + c.x, miny = oy + c.y;
        const float maxx = minx + (float)(a.S - 1), maxy = miny + (float)(a.S - 1);
        if (c.z == 0.0f || !(fabsf(c.x) <= 1e12f && fabsf(c.y) <= 1e12f) || minx < 2.0f || miny < 2.0f ||
            maxx > xmax || maxy > ymax)
            continue;
        float4 s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float g2 = 0.0f;
        for (int pixel = lane; pixel < total; pixel += 64) {
            const float offx = (float)(pixel % side) * (float)a.sample_step;
            const float offy = (float)(pixel / side) * (float)a.sample_step;
            const int rx = (int)(ox + offx), ry = (int)(oy + offy);
            const float f = 255.0f * unorm(a.ref[(size_t)ry * a.W + rx]) - 128.0f;
            const float g = linear_sample(a.tgt, a.W, (ox + offx) + c.x, (oy + offy) + c.y);
            s.x = s.x + f;
            s.y = s.y + g;
            s.z = s.z + f * g;
            s.w = s.w + f * f;
            g2 = g2 + g * g;
        }
        sums[lane] = s;
        sum_g2[lane] = g2;
        __syncthreads();
        for (int off = 32; off > 0; off >>= 1) {
            if (lane < off) {
                const float4 o = sums[lane + off];
                float4 m = sums[lane];
                m.x = m.x + o.x; m.y = m.y + o.y; m.z = m.z + o.z; m.w = m.w + o.w;
                sums[lane] = m;
                sum_g2[lane] = sum_g2[lane] + sum_g2[lane + off];
            }
            __syncthreads();
        }
        if (lane == 0) {
            const float4 t = sums[0];
            const float vf = fmaxf(0.0f, t.w - t.x * t.x / ftotal);
            const float vg = fmaxf(0.0f, sum_g2[0] - t.y * t.y / ftotal);
            float rho = -2.0f;
            if (vf > 1e-9f && vg > 1e-9f) rho = (t.z - t.x * t.y / ftotal) / sqrtf(vf * vg);
            float4 b = best;
            if (k == 0) b.w = rho;
            if (rho > b.z) b = make_float4(c.x, c.y, rho, b.w);
            best = b;
        }
        __syncthreads();
    }
    if (lane == 0) {
        const float4 b = best;
        const float ddx = b.x - ownx, ddy = b.y - owny;
        const bool improved = b.z > b.w + a.min_gain && sqrtf(ddx * ddx + ddy * ddy) > a.min_displacement;
        reinterpret_cast<float4 *>(a.scores)[index] = make_float4(b.w, b.z, improved ? 1.0f : 0.0f, 0.0f);
        if (improved) {
            float4 *seed = reinterpret_cast<float4 *>(a.seeds);
            seed[2 * index] = make_float4(b.x, 0.0f, 0.0f, b.y);
            seed[2 * index + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            a.active[index] = 1u;
        }
    }
}

}  // namespace

cudaError_t launch_affine_frontier(const FrontierArgs &a, cudaStream_t stream) {
    if (a.count <= 0) return cudaSuccess;
    affine_frontier_kernel<<<(a.count + 127) / 128, 128, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_spatial_choose(const ChooseArgs &a, cudaStream_t stream) {
    if (a.count <= 0) return cudaSuccess;
    if (a.sample_step < 1 || a.S < 1) return cudaErrorInvalidValue;
    spatial_choose_kernel<<<a.count, 64, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace gbdic
