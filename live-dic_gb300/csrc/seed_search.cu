// Integer-pixel ZNCC seed search (the reference's nearest component is the
// 11-candidate translation scorer `choose`, shaders/spatial_seed.wgsl:65-190;
// an exhaustive search is new here).
//
// One CTA (128 threads) per subset.  The subset's reference bytes (S x S) and
// the target tile covering every candidate shift ((S + 2R)^2 bytes) are
// staged in shared memory, 4 bytes per word.  Thread t scores candidates t,
// t+128, ... of the (2R+1)^2 integer shifts in row-major (dy, dx) order: the
// five correlation sums sum f, sum g, sum f^2, sum g^2, sum f g come from
// 4-pixel DP4A dot products of packed bytes.  The sums are exact integers
// (8-bit inputs), so the result does not depend on the summation order; ZNCC
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

// Shared layout: the subset's reference rows packed 4 bytes per word and
// zero-padded to RW = ceil(S / 4) words; the target tile (T = S + 2R rows)
// with rows of TW = ceil(T / 4) + 1 words (one spare word so that an
// unaligned 4-byte window never reads past its row).
__host__ __device__ inline int ref_words(int S) { return (S + 3) / 4; }
__host__ __device__ inline int tile_words(int S, int R) { return (S + 2 * R + 3) / 4 + 1; }

// The search of subset idx by the whole CTA (every return is CTA-uniform).
__device__ void search_one(const SearchArgs &a, int idx, uint32_t *smem_words, double *s_best, int *s_cand) {
    if (idx < 0 || idx >= a.count) return;
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
    const int tid = threadIdx.x;
    if (!selected) {
        if (!a.only_missing && tid == 0) {
            for (int k = 0; k < ss; ++k) seed[k] = 0.0f;
            a.active[idx] = 0u;
            if (a.score) a.score[idx] = -2.0f;
        }
        return;
    }
    const int RW = ref_words(S), TW = tile_words(S, R);
    uint32_t *ref = smem_words;               // S x RW
    uint32_t *tile = smem_words + S * RW;     // T x TW
    for (int i = tid; i < S * RW; i += blockDim.x) {
        const int row = i / RW, w = i - row * RW;
        uint32_t v = 0u;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int col = 4 * w + b;
            if (col < S) v |= (uint32_t)a.ref[(size_t)(ry0 + row) * a.W + rx0 + col] << (8 * b);
        }
        ref[i] = v;
    }
    for (int i = tid; i < T * TW; i += blockDim.x) {
        const int row = i / TW, w = i - row * TW;
        const int y = clampi(py0 - R + row, 0, a.H - 1);
        uint32_t v = 0u;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int col = 4 * w + b;
            if (col < T) v |= (uint32_t)a.tgt[(size_t)y * a.W + clampi(px0 - R + col, 0, a.W - 1)] << (8 * b);
        }
        tile[i] = v;
    }
    __syncthreads();
    // Reference sums (exact): sum f and sum f^2 over the packed words.
    unsigned sf = 0u, sff = 0u;  // unsigned bytes: the u32 DP4A form
    for (int i = 0; i < S * RW; ++i) {
        const uint32_t f4 = ref[i];
        sf = __dp4a(f4, 0x01010101u, sf);
        sff = __dp4a(f4, f4, sff);
    }
    const long long n = (long long)S * S;
    const long long vf = n * (long long)sff - (long long)sf * (long long)sf;
    // Byte mask of the last word of a window row (columns beyond S).
    const int tail = S - 4 * (RW - 1);
    const uint32_t last_mask = tail >= 4 ? 0xffffffffu : (0xffffffffu >> (8 * (4 - tail)));
    // One candidate per thread: candidates tid, tid + 128, ... in row-major
    // (dy, dx) order; the window's 4-byte groups are funnel-shifted out of
    // the tile words and summed with DP4A (exact 32-bit integer sums).
    double best = -3.0;
    int best_cand = -1;
    for (int cand = tid; cand < C; cand += blockDim.x) {
        const int dy = cand / side - R, dx = cand % side - R;
        if (px0 + dx < 0 || py0 + dy < 0 || px0 + dx + S - 1 > a.W - 1 || py0 + dy + S - 1 > a.H - 1) continue;
        const int c0 = R + dx, shift = 8 * (c0 & 3), w0 = c0 >> 2;
        unsigned sg = 0u, sgg = 0u, sfg = 0u;
        for (int row = 0; row < S; ++row) {
            const uint32_t *trow = tile + (row + R + dy) * TW + w0;
            const uint32_t *frow = ref + row * RW;
            for (int w = 0; w < RW; ++w) {
                uint32_t g4 = __funnelshift_r(trow[w], trow[w + 1], shift);
                if (w == RW - 1) g4 &= last_mask;
                const uint32_t f4 = frow[w];
                sg = __dp4a(g4, 0x01010101u, sg);
                sgg = __dp4a(g4, g4, sgg);
                sfg = __dp4a(f4, g4, sfg);
            }
        }
        const long long vg = n * (long long)sgg - (long long)sg * (long long)sg;
        double score = -2.0;
        if (vf > 0 && vg > 0)
            score = (double)(n * (long long)sfg - (long long)sf * (long long)sg) / sqrt((double)vf * (double)vg);
        if (score > best) {
            best = score;
            best_cand = cand;
        }
    }
    s_best[tid] = best;
    s_cand[tid] = best_cand;
    __syncthreads();
    if (tid == 0) {
        double b = -3.0;
        int c = -1;
        for (int t = 0; t < (int)blockDim.x; ++t) {
            if (s_cand[t] < 0) continue;
            if (s_best[t] > b || (s_best[t] == b && s_cand[t] < c)) {
                b = s_best[t];
                c = s_cand[t];
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

// One CTA per subset, or (list mode) a fixed grid striding over the first
// *list_count entries of subset_list.
__global__ void __launch_bounds__(128) zncc_search_kernel(SearchArgs a) {
    extern __shared__ uint32_t smem_words[];
    __shared__ double s_best[128];
    __shared__ int s_cand[128];
    if (a.subset_list == nullptr) {
        search_one(a, blockIdx.x, smem_words, s_best, s_cand);
        return;
    }
    const int live = min(a.count, (int)*a.list_count);
    for (int i = blockIdx.x; i < live; i += gridDim.x) {
        search_one(a, a.subset_list[i], smem_words, s_best, s_cand);
        __syncthreads();  // the tiles and the candidate table are reused
    }
}

}  // namespace

size_t zncc_search_smem(int S, int radius) {
    const size_t T = (size_t)S + 2 * (size_t)radius;
    return ((size_t)S * ref_words(S) + T * tile_words(S, radius)) * sizeof(uint32_t);
}

cudaError_t launch_zncc_search(const SearchArgs &a, cudaStream_t stream) {
    if (a.count <= 0) return cudaSuccess;
    const size_t smem = zncc_search_smem(a.S, a.radius);
    if (smem > 48 * 1024) return cudaErrorInvalidValue;
    if (a.subset_list != nullptr && a.list_count == nullptr) return cudaErrorInvalidValue;
    const int grid = a.subset_list != nullptr ? (a.count < 1024 ? a.count : 1024) : a.count;
    zncc_search_kernel<<<grid, 128, smem, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace gbdic
