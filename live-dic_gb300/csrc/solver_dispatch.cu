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
