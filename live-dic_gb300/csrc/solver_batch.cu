// One persistent IC-GN launch over many registration jobs of uneven image
// size, subset size and shape function (B-spline interpolation, uniform
// weighting).  Every job keeps the single-frame solver's arithmetic: a
// work item is one subset of one job and is solved by the same solve_group
// body as icgn_kernel, so a job's states are bit-identical to a solo launch
// with the same lanes per subset.
//
// Two queue layouts.  Per class (GBDIC_BATCH_PERSISTENT): affine and
// translation jobs share one launch and quadratic jobs get their own, as
// independent graph branches.  Single (GBDIC_BATCH_SINGLE): one persistent
// launch over every job of the step, the shape function dispatched per job;
// the quadratic body's 96-register budget (five CTAs per SM) is the affine
// one's, so mixing the classes costs the light one no occupancy.
//
// Work queue: the jobs' subsets are laid end to end in queue order, each
// job's range padded to a whole number of scheduling units (a warp, or a
// 128-thread block when a subset spans more than one warp) so that every
// unit works on a single job and takes the same branch and barriers.  A
// unit claims its next items with one atomicAdd on the queue head; units
// that drew cheap subsets simply come back sooner, which rebalances the
// uneven iteration counts.
#include "gbdic_kernels.h"
#include "solver_impl.cuh"

namespace gbdic {
namespace {

template <int LANES, bool QUAD>
__global__ void __launch_bounds__(128, QUAD ? GBDIC_QUAD_MIN_BLOCKS : GBDIC_SOLVER_MIN_BLOCKS) icgn_batch_kernel(BatchSolveArgs b) {
    constexpr bool kBlock = LANES > 32;
    constexpr int kUnitThreads = kBlock ? 128 : 32;
    constexpr int kGroups = kUnitThreads / LANES;
    constexpr int kMaxSums = SumCount<QUAD ? kModelQuadratic : kModelAffine>::value;
    __shared__ float red_smem[kBlock ? 128 * kMaxSums : 1];
    __shared__ int first[kMaxBatchJobs + 1];
    __shared__ int unit_base;
    const int tid = threadIdx.x;
    const int glane = tid % LANES;
    const int group_in_unit = (tid % kUnitThreads) / LANES;
    const int lane_in_warp = tid & 31;
    float *red = red_smem + (kBlock ? group_in_unit * LANES * kMaxSums : 0);
    for (int i = tid; i <= b.jobs; i += blockDim.x) first[i] = b.first[i];
    __syncthreads();
    const int total = first[b.jobs];
    for (;;) {
        int base;
        if (kBlock) {
            if (tid == 0) unit_base = (int)atomicAdd(b.work_counter, (unsigned)kGroups);
            __syncthreads();
            base = unit_base;
            __syncthreads();
        } else {
            int v = 0;
            if (lane_in_warp == 0) v = (int)atomicAdd(b.work_counter, (unsigned)kGroups);
            base = __shfl_sync(kFullMask, v, 0);
        }
        if (base >= total) break;
        int lo = 0, hi = b.jobs - 1;  // last job whose range starts at or before base
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (first[mid] <= base) lo = mid;
            else hi = mid - 1;
        }
        const SolveArgs a = b.args[lo];
        const int idx = base - first[lo] + group_in_unit;
        if (QUAD)
            solve_group<kModelQuadratic, kInterpBspline, LANES, false>(a, idx, glane, lane_in_warp, red);
        else if (b.models[lo] == kModelTranslation)
            solve_group<kModelTranslation, kInterpBspline, LANES, false>(a, idx, glane, lane_in_warp, red);
        else
            solve_group<kModelAffine, kInterpBspline, LANES, false>(a, idx, glane, lane_in_warp, red);
    }
}

// Every class in one queue: the per-job shape function picks the body.
template <int LANES>
__global__ void __launch_bounds__(128, GBDIC_QUAD_MIN_BLOCKS) icgn_batch_any_kernel(BatchSolveArgs b) {
    constexpr bool kBlock = LANES > 32;
    constexpr int kUnitThreads = kBlock ? 128 : 32;
    constexpr int kGroups = kUnitThreads / LANES;
    constexpr int kMaxSums = SumCount<kModelQuadratic>::value;
    __shared__ float red_smem[kBlock ? 128 * kMaxSums : 1];
    __shared__ int first[kMaxBatchJobs + 1];
    __shared__ int unit_base;
    const int tid = threadIdx.x;
    const int glane = tid % LANES;
    const int group_in_unit = (tid % kUnitThreads) / LANES;
    const int lane_in_warp = tid & 31;
    float *red = red_smem + (kBlock ? group_in_unit * LANES * kMaxSums : 0);
    for (int i = tid; i <= b.jobs; i += blockDim.x) first[i] = b.first[i];
    __syncthreads();
    const int total = first[b.jobs];
    for (;;) {
        int base;
        if (kBlock) {
            if (tid == 0) unit_base = (int)atomicAdd(b.work_counter, (unsigned)kGroups);
            __syncthreads();
            base = unit_base;
            __syncthreads();
        } else {
            int v = 0;
            if (lane_in_warp == 0) v = (int)atomicAdd(b.work_counter, (unsigned)kGroups);
            base = __shfl_sync(kFullMask, v, 0);
        }
        if (base >= total) break;
        int lo = 0, hi = b.jobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (first[mid] <= base) lo = mid;
            else hi = mid - 1;
        }
        const SolveArgs a = b.args[lo];
        const int idx = base - first[lo] + group_in_unit;
        const int model = b.models[lo];
        if (model == kModelQuadratic)
            solve_group<kModelQuadratic, kInterpBspline, LANES, false>(a, idx, glane, lane_in_warp, red);
        else if (model == kModelTranslation)
            solve_group<kModelTranslation, kInterpBspline, LANES, false>(a, idx, glane, lane_in_warp, red);
        else
            solve_group<kModelAffine, kInterpBspline, LANES, false>(a, idx, glane, lane_in_warp, red);
    }
}

template <bool QUAD>
int occupancy(int lanes) {
    int blocks = 0;
    cudaError_t err = cudaErrorInvalidValue;
    if (lanes == 16) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_batch_kernel<16, QUAD>, 128, 0);
    if (lanes == 32) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_batch_kernel<32, QUAD>, 128, 0);
    if (lanes == 64) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_batch_kernel<64, QUAD>, 128, 0);
    if (lanes == 128) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_batch_kernel<128, QUAD>, 128, 0);
    return err == cudaSuccess ? blocks : 0;
}

template <bool QUAD>
cudaError_t launch(const BatchSolveArgs &b, int lanes, int grid, cudaStream_t stream) {
    switch (lanes) {
    case 16: icgn_batch_kernel<16, QUAD><<<grid, 128, 0, stream>>>(b); break;
    case 32: icgn_batch_kernel<32, QUAD><<<grid, 128, 0, stream>>>(b); break;
    case 64: icgn_batch_kernel<64, QUAD><<<grid, 128, 0, stream>>>(b); break;
    case 128: icgn_batch_kernel<128, QUAD><<<grid, 128, 0, stream>>>(b); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace

int batch_units(int lanes) { return lanes > 32 ? 128 / lanes : 32 / lanes; }

int icgn_batch_occupancy(int lanes, bool quadratic) {
    return quadratic ? occupancy<true>(lanes) : occupancy<false>(lanes);
}

int icgn_batch_any_occupancy(int lanes) {
    int blocks = 0;
    cudaError_t err = cudaErrorInvalidValue;
    if (lanes == 16) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_batch_any_kernel<16>, 128, 0);
    if (lanes == 32) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_batch_any_kernel<32>, 128, 0);
    if (lanes == 64) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_batch_any_kernel<64>, 128, 0);
    if (lanes == 128) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, icgn_batch_any_kernel<128>, 128, 0);
    return err == cudaSuccess ? blocks : 0;
}

cudaError_t launch_icgn_batch_any(const BatchSolveArgs &b, int lanes, int grid, cudaStream_t stream) {
    if (b.jobs <= 0 || b.jobs > kMaxBatchJobs || grid <= 0) return cudaErrorInvalidValue;
    switch (lanes) {
    case 16: icgn_batch_any_kernel<16><<<grid, 128, 0, stream>>>(b); break;
    case 32: icgn_batch_any_kernel<32><<<grid, 128, 0, stream>>>(b); break;
    case 64: icgn_batch_any_kernel<64><<<grid, 128, 0, stream>>>(b); break;
    case 128: icgn_batch_any_kernel<128><<<grid, 128, 0, stream>>>(b); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_icgn_batch(const BatchSolveArgs &b, int lanes, bool quadratic, int grid, cudaStream_t stream) {
    if (b.jobs <= 0 || b.jobs > kMaxBatchJobs || grid <= 0) return cudaErrorInvalidValue;
    return quadratic ? launch<true>(b, lanes, grid, stream) : launch<false>(b, lanes, grid, stream);
}

}  // namespace gbdic
