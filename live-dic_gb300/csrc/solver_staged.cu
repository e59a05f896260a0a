// IC-GN solver with TMA-staged coefficient tiles (the "staged" solver modes;
// reference operations: shaders/icgn.wgsl:230-319 sample_cubic and 712-780
// the pixel loop, with the iteration of 595-1017 as in solver_impl.cuh).
//
// The exact solver's pixel loop (pixel p on lane p mod LANES, packed FP32
// pairs, the reference's summation order) with one change of memory path:
// every warp owns a TW x TH float tile of the B-spline coefficient plane in
// shared memory, loaded by one cp.async.bulk.tensor.2d per (re)load from a
// tensor map over the plane and completed on the warp's mbarrier.  The tile
// is placed over the union of the tap footprints of the warp's two subsets
// (16 lanes per subset; neighbouring subsets overlap by all but one stride)
// and is reloaded only when a footprint leaves it.  The TMA x coordinate is
// kept a multiple of 4 floats (16 bytes).  Footprints that do not fit fall
// back to the global loads of the exact loop for that iteration, and every
// wait is bounded (an expired wait switches the warp to global loads).  The
// samples are the same coefficients combined by the same operations, so the
// results are bit-identical to the exact solver's.
//
// Tile shapes ("tile shape" axis of the autotuner): compact 56 x 44
// (9,856 bytes per warp, two S <= 31 subsets at stride <= 8 with a few
// pixels of slack) and wide 72 x 56 (16,128 bytes; S up to 41 or larger
// strides).  Four warps per CTA; the plane's row pitch must be a multiple of
// 16 bytes (W % 4 == 0) for the tensor map.
#include <cuda.h>

#include "gbdic_kernels.h"
#include "solver_impl.cuh"

namespace gbdic {
namespace {

constexpr int kStageWarps = 4;

template <int TW, int TH>
constexpr size_t stage_smem_bytes() {
    return (size_t)kStageWarps * TW * TH * sizeof(float) + 128;  // + alignment slack
}

template <int MODEL, int LANES, bool GAUSS, int TW, int TH>
__global__ void __launch_bounds__(128, GBDIC_SOLVER_MIN_BLOCKS)
    icgn_staged_kernel(const __grid_constant__ CUtensorMap map, SolveArgs a) {
    static_assert(LANES == 16 || LANES == 32, "staged tiles serve warp-sized groups");
    static_assert((TW * 4) % 16 == 0 && (TW * TH * 4) % 128 == 0, "TMA box and tile alignment");
    constexpr int kGroups = 32 / LANES;
    extern __shared__ uint8_t stage_raw[];
    __shared__ uint64_t bars[kStageWarps];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float *tiles = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(stage_raw) + 127) & ~uintptr_t(127));
    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
            static_cast<uint32_t>(__cvta_generic_to_shared(&bars[warp]))));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    const StageTile st{&map, tiles + (size_t)warp * TW * TH, &bars[warp]};
    StageState ss{0, 0, 0u, false, false, false};
    const int glane = tid % LANES;
    const int group_in_warp = lane / LANES;
    const long long unit = (long long)blockIdx.x * kStageWarps + warp;
    for (;;) {
        int base;
        if (a.persistent) {
            int v = 0;
            if (lane == 0) v = (int)atomicAdd(a.work_counter, (unsigned)kGroups);
            base = __shfl_sync(kFullMask, v, 0);
        } else {
            base = unit * kGroups < (long long)a.count ? (int)(unit * kGroups) : a.count;
        }
        if (base >= a.count) break;
        solve_group<MODEL, kInterpBspline, LANES, GAUSS, false, TW, TH>(a, base + group_in_warp, glane, lane, nullptr,
                                                                          &st, &ss);
        if (!a.persistent) break;
    }
    // A load whose wait expired may still land: wait for it (bounded) so
    // that no copy writes into the CTA's shared memory after it exits.
    if (ss.pending && lane == 0) stage_wait(&bars[warp], ss.phase);
    __syncwarp();
}

typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// W x H FP32 plane (row pitch W floats), box TW x TH, zero fill outside.
template <int TW, int TH>
bool plane_map(CUtensorMap *map, const float *plane, int W, int H) {
    EncodeTiled fn = encode_fn();
    if (!fn || W % 4 != 0) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
    const cuuint64_t strides[1] = {(cuuint64_t)W * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)TW, (cuuint32_t)TH};
    const cuuint32_t estride[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(plane), dims, strides, box, estride,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int MODEL, int LANES, bool GAUSS, int TW, int TH>
cudaError_t launch_shape(const SolveArgs &a, int grid, cudaStream_t stream, int *occupancy_only) {
    auto kernel = icgn_staged_kernel<MODEL, LANES, GAUSS, TW, TH>;
    constexpr size_t smem = stage_smem_bytes<TW, TH>();
    static thread_local int configured_device = -1;
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) return err;
    if (configured_device != device) {
        err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        configured_device = device;
    }
    if (occupancy_only) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occupancy_only, kernel, 128, smem);
    CUtensorMap map;
    if (!plane_map<TW, TH>(&map, a.coef, a.W, a.H)) return cudaErrorInvalidValue;
    kernel<<<grid, 128, smem, stream>>>(map, a);
    return cudaGetLastError();
}

template <int MODEL, int LANES, bool GAUSS>
cudaError_t launch_tile(const SolveArgs &a, int tile, int grid, cudaStream_t stream, int *occupancy_only) {
    if (tile == 1) return launch_shape<MODEL, LANES, GAUSS, 56, 44>(a, grid, stream, occupancy_only);
    if (tile == 2) return launch_shape<MODEL, LANES, GAUSS, 72, 56>(a, grid, stream, occupancy_only);
    return cudaErrorInvalidValue;
}

template <int MODEL>
cudaError_t launch_model(const SolveArgs &a, int lanes, bool gauss, int tile, int grid, cudaStream_t stream,
                         int *occupancy_only) {
    if (lanes == 16)
        return gauss ? launch_tile<MODEL, 16, true>(a, tile, grid, stream, occupancy_only)
                     : launch_tile<MODEL, 16, false>(a, tile, grid, stream, occupancy_only);
    if (lanes == 32)
        return gauss ? launch_tile<MODEL, 32, true>(a, tile, grid, stream, occupancy_only)
                     : launch_tile<MODEL, 32, false>(a, tile, grid, stream, occupancy_only);
    return cudaErrorInvalidValue;
}

}  // namespace

bool icgn_staged_supported(int model, int interp, int lanes, int W) {
    return (model == kModelAffine || model == kModelTranslation) && interp == kInterpBspline &&
           (lanes == 16 || lanes == 32) && W % 4 == 0;
}

cudaError_t launch_icgn_staged(const SolveArgs &a, int model, int lanes, bool gauss, int tile, int grid,
                               cudaStream_t stream, int *occupancy_only) {
    if (model == kModelAffine) return launch_model<kModelAffine>(a, lanes, gauss, tile, grid, stream, occupancy_only);
    if (model == kModelTranslation)
        return launch_model<kModelTranslation>(a, lanes, gauss, tile, grid, stream, occupancy_only);
    return cudaErrorInvalidValue;
}

int icgn_staged_occupancy(int model, int lanes, bool gauss, int tile) {
    SolveArgs unused{};
    int blocks = 0;
    if (launch_icgn_staged(unused, model, lanes, gauss, tile, 0, nullptr, &blocks) != cudaSuccess) return 0;
    return blocks;
}

}  // namespace gbdic
