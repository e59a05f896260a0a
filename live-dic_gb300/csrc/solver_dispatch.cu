// Launch geometry and dispatch of the IC-GN solver variants.
#include "gbdic_kernels.h"

namespace gbdic {

int icgn_grid(int count, int lanes) {
    if (count <= 0) return 0;
    if (lanes > 32) {
        const int groups = 128 / lanes;  // subsets per block
        return (count + groups - 1) / groups;
    }
    const int per_warp = 32 / lanes;
    const int units = (count + per_warp - 1) / per_warp;  // warps
    return (units + 3) / 4;                                // 4 warps per block
}

namespace {

// Every subset's row as the seeded solver writes it for a disabled subset
// (solver_impl.cuh solve_group: the seed's warp, status `rejected`, zero
// iterations; preserve_disabled off).  List-mode solves write this first so
// that the rows they do not list equal the full-grid solve's.
template <int MODEL>
__global__ void disabled_rows_kernel(SolveArgs a, int total) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const float4 *s = reinterpret_cast<const float4 *>(a.seed + (size_t)idx * state_stride(MODEL));
    const float4 s0 = __ldg(s), s1 = __ldg(s + 1);
    const bool translation = MODEL == kModelTranslation;
    const float mvalid = __ldg(a.meta + (size_t)idx * meta_stride(MODEL) + 1);
    const bool valid = __ldg(a.active + idx) != 0u && mvalid >= 0.5f;
    const float rejected = a.roi_enabled ? fminf(-1.0f, mvalid) : -1.0f;
    const float status = valid ? 0.0f : rejected;
    float4 *o = reinterpret_cast<float4 *>(a.state + (size_t)idx * state_stride(MODEL));
    o[0] = make_float4(s0.x, translation ? 0.0f : s0.y, translation ? 0.0f : s0.z, s0.w);
    if (MODEL == kModelQuadratic) {
        const float4 s2 = __ldg(s + 2);
        o[1] = make_float4(s1.x, s1.y, s1.z, s1.w);
        o[2] = s2;
        o[3] = make_float4(status, 0.0f, 0.0f, 0.0f);
    } else {
        o[1] = make_float4(translation ? 0.0f : s1.x, translation ? 0.0f : s1.y, status, 0.0f);
    }
}

cudaError_t dispatch(const SolveArgs &a, int model, int interp, int lanes, bool gauss, int grid,
                     cudaStream_t stream, int *occupancy_only) {
    switch (model) {
    case kModelAffine:
        return launch_icgn_model<kModelAffine>(a, interp, lanes, gauss, grid, stream, occupancy_only);
    case kModelTranslation:
        return launch_icgn_model<kModelTranslation>(a, interp, lanes, gauss, grid, stream, occupancy_only);
    case kModelQuadratic:
        return launch_icgn_model<kModelQuadratic>(a, interp, lanes, gauss, grid, stream, occupancy_only);
    default:
        return cudaErrorInvalidValue;
    }
}
}  // namespace

int icgn_occupancy(int model, int interp, int lanes, bool gauss) {
    SolveArgs unused{};
    int blocks = 0;
    if (dispatch(unused, model, interp, lanes, gauss, 0, nullptr, &blocks) != cudaSuccess) return 0;
    return blocks;
}

int icgn_fast_occupancy(int model, int lanes, bool gauss) {
    SolveArgs unused{};
    int blocks = 0;
    if (launch_icgn_fast(unused, model, lanes, gauss, 0, nullptr, &blocks) != cudaSuccess) return 0;
    return blocks;
}

cudaError_t launch_disabled_rows(const SolveArgs &a, int model, int total, cudaStream_t stream) {
    if (total <= 0) return cudaSuccess;
    const int grid = (total + 255) / 256;
    switch (model) {
    case kModelAffine: disabled_rows_kernel<kModelAffine><<<grid, 256, 0, stream>>>(a, total); break;
    case kModelTranslation: disabled_rows_kernel<kModelTranslation><<<grid, 256, 0, stream>>>(a, total); break;
    case kModelQuadratic: disabled_rows_kernel<kModelQuadratic><<<grid, 256, 0, stream>>>(a, total); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_icgn(const SolveArgs &a, int model, int interp, int lanes, bool gauss,
                        int persistent_grid, cudaStream_t stream) {
    if (a.count <= 0) return cudaSuccess;
    const int grid = a.persistent ? persistent_grid : icgn_grid(a.count, lanes);
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    if (a.fast_segments > 0 && icgn_fast_supported(model, interp, lanes))
        return launch_icgn_fast(a, model, lanes, gauss, grid, stream, nullptr);
    if (a.staged_tile > 0 && icgn_staged_supported(model, interp, lanes, a.W))
        return launch_icgn_staged(a, model, lanes, gauss, a.staged_tile, grid, stream, nullptr);
    return dispatch(a, model, interp, lanes, gauss, grid, stream, nullptr);
}

}  // namespace gbdic
