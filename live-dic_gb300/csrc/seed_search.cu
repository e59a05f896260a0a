// Integer-pixel ZNCC seed search (the reference's nearest component is the
// 11-candidate translation scorer `choose`, shaders/spatial_seed.wgsl:65-190;
// an exhaustive search is new here).
//
// One CTA (4 warps) per subset.  The subset's reference bytes (S x S) and the
// target tile covering every candidate shift ((S + 2R)^2 bytes) are staged in
// shared memory.  Warp w scans candidates w, w+4, ... of the (2R+1)^2 integer
// shifts in row-major (dy, dx) order; for each, the lanes accumulate the five
// correlation sums sum f, sum g, sum f^2, sum g^2, sum f g over lane-strided
// pixels and combine them with warp shuffles.  The sums are exact integers
// (8-bit inputs), so the result does not depend on the reduction order; ZNCC
// is evaluated in binary64 from the exact sums,
//   (n Sfg - Sf Sg) / sqrt((n Sff - Sf^2) (n Sgg - Sg^2)),
// and the best candidate (lowest index on ties) becomes a translation seed.
// Candidates whose window leaves the image are skipped.  In centred mode the
// shifts are taken around the rounded translation already in the seed (the
// reseeding of a failed learned proposal), and a subset mask can restrict the
// search to chosen subsets.
#include "gbdic_common.cuh"
#include "gbdic_kernels.h"

namespace gbdic {

namespace {

__global__ void __launch_bounds__(128) zncc_search_kernel(SearchArgs a) {
    extern __shared__ uint8_t smem[];
    const int idx = blockIdx.x;
    if (idx >= a.count) return;
    const int ss = state_stride(a.model), sat = status_slot(a.model);
    float *seed = a.seed + (size_t)idx * ss;
    if (a.only_missing && seed[sat] != -1.0f) return;  // block-uniform
    if (a.subset_mask != nullptr && a.subset_mask[idx] == 0) return;
    const bool selected = a.selected == nullptr || a.selected[idx] != 0;
    const int S = a.S, R = a.radius, T = S + 2 * R, side = 2 * R + 1, C = side * side;
    // Centred mode: candidates around the rounded current translation seed.
    int cx0 = 0, cy0 = 0;
    if (a.centered) {
        const float sx = seed[0], sy = seed[3];
        cx0 = (fabsf(sx) <= (float)a.W) ? (int)rintf(sx) : 0;
        cy0 = (fabsf(sy) <= (float)a.H) ? (int)rintf(sy) : 0;
    }
    const int px0 = (idx % a.grid_w) * a.stride + cx0, py0 = (idx / a.grid_w) * a.stride + cy0;
    const int rx0 = (idx % a.grid_w) * a.stride, ry0 = (idx / a.grid_w) * a.stride;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    __shared__ double s_best[4];
    __shared__ int s_cand[4];
    if (!selected) {
        if (!a.only_missing && tid == 0) {
            for (int k = 0; k < ss; ++k) seed[k] = 0.0f;
            a.active[idx] = 0u;
            if (a.score) a.score[idx] = -2.0f;
        }
        return;
    }
    uint8_t *ref = smem;
    uint8_t *tile = smem + S * S;
    for (int i = tid; i < S * S; i += blockDim.x) {
        const int col = i % S, row = i / S;
        ref[i] = a.ref[(size_t)(ry0 + row) * a.W + rx0 + col];
    }
    for (int i = tid; i < T * T; i += blockDim.x) {
        const int col = i % T, row = i / T;
        const int x = clampi(px0 - R + col, 0, a.W - 1), y = clampi(py0 - R + row, 0, a.H - 1);
        tile[i] = a.tgt[(size_t)y * a.W + x];
    }
    __syncthreads();
    // reference sums (exact)
    long long sf = 0, sff = 0;
    for (int p = lane; p < S * S; p += 32) {
        const int f = ref[p];
        sf += f;
        sff += f * f;
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        sf += __shfl_xor_sync(kFullMask, sf, off);
        sff += __shfl_xor_sync(kFullMask, sff, off);
    }
    const long long n = (long long)S * S;
    const long long vf = n * sff - sf * sf;
    double best = -3.0;
    int best_cand = -1;
    for (int cand = warp; cand < C; cand += 4) {
        const int dy = cand / side - R, dx = cand % side - R;
        if (px0 + dx < 0 || py0 + dy < 0 || px0 + dx + S - 1 > a.W - 1 || py0 + dy + S - 1 > a.H - 1) continue;
        int sg = 0, sgg = 0, sfg = 0;
        for (int p = lane; p < S * S; p += 32) {
            const int col = p % S, row = p / S;
            const int g = tile[(row + R + dy) * T + col + R + dx];
            const int f = ref[p];
            sg += g;
            sgg += g * g;
            sfg += f * g;
        }
        long long lg = sg, lgg = sgg, lfg = sfg;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            lg += __shfl_xor_sync(kFullMask, lg, off);
            lgg += __shfl_xor_sync(kFullMask, lgg, off);
            lfg += __shfl_xor_sync(kFullMask, lfg, off);
        }
        const long long vg = n * lgg - lg * lg;
        double score = -2.0;
        if (vf > 0 && vg > 0) score = (double)(n * lfg - sf * lg) / sqrt((double)vf * (double)vg);
        if (score > best) {
            best = score;
            best_cand = cand;
        }
    }
    if (lane == 0) {
        s_best[warp] = best;
        s_cand[warp] = best_cand;
    }
    __syncthreads();
    if (tid == 0) {
        double b = -3.0;
        int c = -1;
        for (int w = 0; w < 4; ++w) {
            if (s_cand[w] < 0) continue;
            if (s_best[w] > b || (s_best[w] == b && s_cand[w] < c)) {
                b = s_best[w];
                c = s_cand[w];
            }
        }
        for (int k = 0; k < ss; ++k) seed[k] = 0.0f;
        if (c >= 0 && b > -1.5) {
            seed[0] = (float)(cx0 + c % side - R);
            seed[3] = (float)(cy0 + c / side - R);
        }
        a.active[idx] = 1u;
        if (a.score) a.score[idx] = (float)b;
        if (a.searched) atomicAdd(a.searched, 1u);
    }
}

}  // namespace

size_t zncc_search_smem(int S, int radius) {
    const size_t T = (size_t)S + 2 * (size_t)radius;
    return (size_t)S * S + T * T;
}

cudaError_t launch_zncc_search(const SearchArgs &a, cudaStream_t stream) {
    if (a.count <= 0) return cudaSuccess;
    const size_t smem = zncc_search_smem(a.S, a.radius);
    if (smem > 48 * 1024) return cudaErrorInvalidValue;
    zncc_search_kernel<<<a.count, 128, smem, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace gbdic
