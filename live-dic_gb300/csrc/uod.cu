// Displacement outlier detection and median repair (reference:
// shaders/icgn.wgsl:1087-1605).  One thread per subset reads its own state
// and its 3x3 (or up to 9x9) neighbours and writes the filtered state.
// Neighbour warps are Taylor-recentred to the subset centre before their
// medians are taken; medians are order statistics, so any exact selection
// algorithm gives the same values (a bubble network for <= 9 values, Hoare
// quickselect for up to 81).
#include "gbdic_common.cuh"
#include "gbdic_kernels.h"

namespace gbdic {

namespace {

__device__ float median_small(float *v, int count) {
    for (int phase = 0; phase < 9; ++phase)
        for (int i = 0; i < 8; ++i)
            if (i + 1 < count && v[i] > v[i + 1]) {
                float s = v[i];
                v[i] = v[i + 1];
                v[i + 1] = s;
            }
    if (count % 2 == 1) return v[count / 2];
    return 0.5f * (v[count / 2 - 1] + v[count / 2]);
}

__device__ float select_rank(float *v, int count, int rank) {
    int low = 0, high = count - 1;
    for (int guard = 0; guard < 4096; ++guard) {
        if (low >= high) return v[rank];
        const float pivot = v[low + (high - low) / 2];
        int left = low, right = high;
        for (;;) {
            while (left <= high && v[left] < pivot) ++left;
            while (right >= low && v[right] > pivot) --right;
            if (left > right) break;
            float s = v[left];
            v[left] = v[right];
            v[right] = s;
            ++left;
            --right;
        }
        if (rank <= right) high = right;
        else if (rank >= left) low = left;
        else return v[rank];
    }
    return v[rank];
}

__device__ float median_large(float *v, int count) {
    if (count % 2 == 1) return select_rank(v, count, count / 2);
    const float lo = select_rank(v, count, count / 2 - 1);
    const float hi = select_rank(v, count, count / 2);
    return 0.5f * (lo + hi);
}

// Taylor recentring of component `comp` of state s at offset (ox, oy).
__device__ float recentered(int model, const float *s, int comp, float ox, float oy) {
    if (model == kModelQuadratic) {
        switch (comp) {
        case 0: return fmaf(s[8], 0.5f * oy * oy, fmaf(s[7], ox * oy, fmaf(s[6], 0.5f * ox * ox, fmaf(s[2], oy, fmaf(s[1], ox, s[0])))));
        case 1: return fmaf(s[7], oy, fmaf(s[6], ox, s[1]));
        case 2: return fmaf(s[8], oy, fmaf(s[7], ox, s[2]));
        case 3: return fmaf(s[11], 0.5f * oy * oy, fmaf(s[10], ox * oy, fmaf(s[9], 0.5f * ox * ox, fmaf(s[5], oy, fmaf(s[4], ox, s[3])))));
        case 4: return fmaf(s[10], oy, fmaf(s[9], ox, s[4]));
        case 5: return fmaf(s[11], oy, fmaf(s[10], ox, s[5]));
        default: return s[comp];
        }
    }
    if (comp == 0) return fmaf(s[2], oy, fmaf(s[1], ox, s[0]));
    if (comp == 3) return fmaf(s[5], oy, fmaf(s[4], ox, s[3]));
    return s[comp];
}

__device__ __constant__ int kOrder[12] = {0, 3, 1, 2, 4, 5, 6, 7, 8, 9, 10, 11};

__device__ bool allowed(const UodArgs &a, int index, int dx, int dy, bool wide) {
    if (!a.roi_enabled) return true;
    const float *perm = a.links + (size_t)index * 4;
    unsigned bit, word;
    if (wide) {
        bit = (unsigned)((dy + 4) * 9 + dx + 4);
        word = (unsigned)perm[bit / 24];
    } else {
        bit = (unsigned)((dy + 1) * 3 + dx + 1);
        word = (unsigned)perm[0];
    }
    return (word & (1u << (bit % 24))) != 0u;
}

__device__ void load_state(const float *src, int ss, float *dst) {
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    for (int k = 0; k < ss / 4; ++k) {
        float4 v = s4[k];
        dst[4 * k] = v.x; dst[4 * k + 1] = v.y; dst[4 * k + 2] = v.z; dst[4 * k + 3] = v.w;
    }
}

__device__ void store_state(float *dst, int ss, const float *src) {
    float4 *d4 = reinterpret_cast<float4 *>(dst);
    for (int k = 0; k < ss / 4; ++k) d4[k] = make_float4(src[4 * k], src[4 * k + 1], src[4 * k + 2], src[4 * k + 3]);
}

// icgn.wgsl:1192-1323
__device__ void median_motion(const UodArgs &a, int index) {
    const int ss = state_stride(a.model);
    const int sat = status_slot(a.model);
    float own[16];
    load_state(a.state + (size_t)index * ss, ss, own);
    float out[16];
    for (int k = 0; k < ss; ++k) out[k] = own[k];
    const float own_status = own[sat];
    const float ref_status = a.meta[(size_t)index * meta_stride(a.model) + 1];
    if (!((own_status >= 0.5f && !a.scope_all) || (ref_status < 0.5f && ref_status != -4.0f))) {
        const int px = index % a.grid_w, py = index / a.grid_w;
        const int radius = a.median_size / 2;
        const int active = a.model == kModelTranslation ? 2 : (a.model == kModelQuadratic ? 12 : 6);
        float filtered[12];
        for (int k = 0; k < 12; ++k) filtered[k] = own[k];
        bool complete = true;
        float values[81];
        float nbr[16];
        for (int ai = 0; ai < active && complete; ++ai) {
            const int comp = kOrder[ai];
            int count = 0;
            if (own_status >= 0.5f) values[count++] = recentered(a.model, own, comp, 0.0f, 0.0f);
            for (int dy = -radius; dy <= radius; ++dy)
                for (int dx = -radius; dx <= radius; ++dx) {
                    if (dx == 0 && dy == 0) continue;
                    const int nx = px + dx, ny = py + dy;
                    if (nx < 0 || ny < 0 || nx >= a.grid_w || ny >= a.grid_h) continue;
                    if (!allowed(a, index, dx, dy, a.median_size > 3)) continue;
                    const float *ns = a.state + ((size_t)ny * a.grid_w + nx) * ss;
                    if (ns[sat] < 0.5f) continue;
                    load_state(ns, ss, nbr);
                    values[count++] = recentered(a.model, nbr, comp, -(float)a.subset_stride * (float)dx,
                                                 -(float)a.subset_stride * (float)dy);
                }
            const int minimum = (a.roi_enabled && a.median_size == 3 && own_status < 0.5f) ? 3 : 4;
            if (count < minimum) {
                complete = false;
                break;
            }
            filtered[comp] = median_large(values, count);
        }
        if (complete) {
            for (int k = 0; k < 12 && k < ss; ++k) out[k] = filtered[k];
            if (a.model == kModelQuadratic) {
                out[12] = (a.seed_mode && own_status < 0.5f) ? 0.0f : own[12];
                out[13] = own[13]; out[14] = own[14]; out[15] = own[15];
            } else {
                out[6] = (a.seed_mode && own_status < 0.5f) ? 0.0f : own[6];
                out[7] = own[7];
            }
        }
    }
    store_state(a.out + (size_t)index * ss, ss, out);
}

__global__ void uod_kernel(UodArgs a) {
    const int index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= a.count) return;
    if (a.policy == 3) {
        median_motion(a, index);
        return;
    }
    const int ss = state_stride(a.model);
    const int sat = status_slot(a.model);
    float own[16];
    load_state(a.state + (size_t)index * ss, ss, own);
    float out[16];
    for (int k = 0; k < ss; ++k) out[k] = own[k];
    if (own[sat] >= 0.5f) {
        const int px = index % a.grid_w, py = index / a.grid_w;
        const int ncomp = parameter_count(a.model);
        float nb[9][12];
        float nbr[16];
        int count = 0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                if (dx == 0 && dy == 0) continue;
                const int nx = px + dx, ny = py + dy;
                if (nx < 0 || ny < 0 || nx >= a.grid_w || ny >= a.grid_h) continue;
                if (a.model != kModelQuadratic && !allowed(a, index, dx, dy, false)) continue;
                const float *ns = a.state + ((size_t)ny * a.grid_w + nx) * ss;
                if (ns[sat] < 0.5f) continue;
                load_state(ns, ss, nbr);
                const float ox = -(float)a.subset_stride * (float)dx, oy = -(float)a.subset_stride * (float)dy;
                for (int k = 0; k < ncomp; ++k) nb[count][k] = recentered(a.model, nbr, k, ox, oy);
                ++count;
            }
        if (count >= 4) {
            float filtered[12], medians[12], values[9];
            for (int k = 0; k < 12; ++k) filtered[k] = medians[k] = (k < ncomp) ? own[k] : 0.0f;
            const int model_components = a.model == kModelTranslation ? 2 : ncomp;
            const int median_count = a.policy == 1 ? model_components : 2;
            for (int ai = 0; ai < median_count; ++ai) {
                const int comp = kOrder[ai];
                for (int i = 0; i < count; ++i) values[i] = nb[i][comp];
                medians[comp] = median_small(values, count);
            }
            bool flagged = false;
            for (int ai = 0; ai < 2; ++ai) {
                const int comp = kOrder[ai];
                for (int i = 0; i < count; ++i) values[i] = fabsf(nb[i][comp] - medians[comp]);
                const float spread = median_small(values, count);
                const float score = fabsf(filtered[comp] - medians[comp]) / (spread + 0.1f);
                if (score > 2.0f) flagged = true;
            }
            if (flagged) {
                if (a.policy == 1)
                    for (int ai = 0; ai < model_components; ++ai) filtered[kOrder[ai]] = medians[kOrder[ai]];
                for (int k = 0; k < ncomp; ++k) out[k] = filtered[k];
                if (a.model == kModelQuadratic) {
                    out[12] = 2.0f; out[13] = own[13]; out[14] = 0.0f; out[15] = 0.0f;
                } else {
                    out[6] = 2.0f; out[7] = own[7];
                }
            }
        }
    }
    store_state(a.out + (size_t)index * ss, ss, out);
}

// Stable sort of 8 values (odd-even transposition, swap only when strictly
// greater): the same arrangement as a bubble sort of the compacted values,
// with the +inf padding of missing neighbours at the end.
__device__ __forceinline__ void sort8(float (&v)[8]) {
#pragma unroll
    for (int round = 0; round < 8; ++round) {
#pragma unroll
        for (int i = round & 1; i + 1 < 8; i += 2) {
            const float lo = v[i], hi = v[i + 1];
            const bool swap = lo > hi;
            v[i] = swap ? hi : lo;
            v[i + 1] = swap ? lo : hi;
        }
    }
}

// median_small() of the first `count` (4..8) sorted values.
__device__ __forceinline__ float median_sorted8(const float (&v)[8], int count) {
    switch (count) {
    case 4: return 0.5f * (v[1] + v[2]);
    case 5: return v[2];
    case 6: return 0.5f * (v[2] + v[3]);
    case 7: return v[3];
    default: return 0.5f * (v[3] + v[4]);
    }
}

// 3x3 UOD (replace / flag) of translation and affine states with every
// neighbour in registers: the neighbour slots keep the scan order of the
// generic kernel, missing ones read +inf, and the order statistics come
// from sort8, so the result equals uod_kernel's bit for bit.
template <int MODEL>
__global__ void __launch_bounds__(128) uod3_kernel(UodArgs a) {
    constexpr int ss = state_stride(MODEL), sat = status_slot(MODEL), nc = parameter_count(MODEL);
    const int index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= a.count) return;
    float own[ss];
    load_state(a.state + (size_t)index * ss, ss, own);
    float out[ss];
#pragma unroll
    for (int k = 0; k < ss; ++k) out[k] = own[k];
    if (own[sat] >= 0.5f) {
        const int px = index % a.grid_w, py = index / a.grid_w;
        const float kInf = __int_as_float(0x7f800000);
        float nb[8][nc];
        bool valid[8];
        int count = 0;
#pragma unroll
        for (int slot = 0; slot < 8; ++slot) {
            const int cell = slot < 4 ? slot : slot + 1;  // 3x3 scan order without the centre
            const int dx = cell % 3 - 1, dy = cell / 3 - 1;
            const int nx = px + dx, ny = py + dy;
            bool ok = nx >= 0 && ny >= 0 && nx < a.grid_w && ny < a.grid_h && allowed(a, index, dx, dy, false);
            float nbr[ss];
            if (ok) {
                load_state(a.state + ((size_t)ny * a.grid_w + nx) * ss, ss, nbr);
                ok = nbr[sat] >= 0.5f;
            }
            valid[slot] = ok;
            count += ok ? 1 : 0;
            const float ox = -(float)a.subset_stride * (float)dx, oy = -(float)a.subset_stride * (float)dy;
#pragma unroll
            for (int k = 0; k < nc; ++k) nb[slot][k] = ok ? recentered(MODEL, nbr, k, ox, oy) : kInf;
        }
        if (count >= 4) {
            float filtered[nc], medians[nc];
#pragma unroll
            for (int k = 0; k < nc; ++k) filtered[k] = medians[k] = own[k];
            constexpr int model_components = MODEL == kModelTranslation ? 2 : nc;
            const int median_count = a.policy == 1 ? model_components : 2;
#pragma unroll
            for (int ai = 0; ai < model_components; ++ai) {
                if (ai >= median_count) break;
                const int comp = ai == 0 ? 0 : (ai == 1 ? 3 : (ai == 2 ? 1 : (ai == 3 ? 2 : ai)));
                float v[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) v[i] = nb[i][comp];
                sort8(v);
                medians[comp] = median_sorted8(v, count);
            }
            bool flagged = false;
#pragma unroll
            for (int ai = 0; ai < 2; ++ai) {
                const int comp = ai == 0 ? 0 : 3;
                float v[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) v[i] = valid[i] ? fabsf(nb[i][comp] - medians[comp]) : kInf;
                sort8(v);
                const float spread = median_sorted8(v, count);
                const float score = fabsf(filtered[comp] - medians[comp]) / (spread + 0.1f);
                if (score > 2.0f) flagged = true;
            }
            if (flagged) {
                if (a.policy == 1) {
#pragma unroll
                    for (int k = 0; k < model_components; ++k) {
                        const int comp = k == 0 ? 0 : (k == 1 ? 3 : (k == 2 ? 1 : (k == 3 ? 2 : k)));
                        filtered[comp] = medians[comp];
                    }
                }
#pragma unroll
                for (int k = 0; k < nc; ++k) out[k] = filtered[k];
                out[6] = 2.0f;
                out[7] = own[7];
            }
        }
    }
    store_state(a.out + (size_t)index * ss, ss, out);
}

}  // namespace

cudaError_t launch_uod(const UodArgs &a, cudaStream_t stream) {
    if (a.count <= 0) return cudaSuccess;
    const int grid = (a.count + 127) / 128;
    if (a.policy != 3 && a.model == kModelAffine) uod3_kernel<kModelAffine><<<grid, 128, 0, stream>>>(a);
    else if (a.policy != 3 && a.model == kModelTranslation) uod3_kernel<kModelTranslation><<<grid, 128, 0, stream>>>(a);
    else uod_kernel<<<grid, 128, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace gbdic
