// IC-GN over partial-support ROI windows (reference: solve_partial /
// solve_partial_seeded / retry_partial_seeded, shaders/icgn.wgsl:1042-1085):
// the solve_group body of the complete-window solver with the window's
// support bits, support box and partial metadata (validity -4, partial mean
// and weight sum).  One grid launch over the partial windows, after the
// complete-window launch of the same frame.
#include "gbdic_kernels.h"
#include "solver_impl.cuh"

namespace gbdic {
namespace {

template <int MODEL, int INTERP, int LANES, bool GAUSS>
cudaError_t go(const SolveArgs &a, cudaStream_t s) {
    icgn_kernel<MODEL, INTERP, LANES, GAUSS, true><<<icgn_grid(a.count, LANES), 128, 0, s>>>(a);
    return cudaGetLastError();
}

template <int MODEL, int INTERP, bool GAUSS>
cudaError_t by_lanes(const SolveArgs &a, int lanes, cudaStream_t s) {
    switch (lanes) {
    case 16: return go<MODEL, INTERP, 16, GAUSS>(a, s);
    case 32: return go<MODEL, INTERP, 32, GAUSS>(a, s);
    case 64: return go<MODEL, INTERP, 64, GAUSS>(a, s);
    case 128: return go<MODEL, INTERP, 128, GAUSS>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int MODEL, bool GAUSS>
cudaError_t by_interp(const SolveArgs &a, int interp, int lanes, cudaStream_t s) {
    switch (interp) {
    case kInterpBspline: return by_lanes<MODEL, kInterpBspline, GAUSS>(a, lanes, s);
    case kInterpLinear: return by_lanes<MODEL, kInterpLinear, GAUSS>(a, lanes, s);
    case kInterpKeys: return by_lanes<MODEL, kInterpKeys, GAUSS>(a, lanes, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int MODEL>
cudaError_t by_weight(const SolveArgs &a, int interp, int lanes, bool gauss, cudaStream_t s) {
    return gauss ? by_interp<MODEL, true>(a, interp, lanes, s) : by_interp<MODEL, false>(a, interp, lanes, s);
}

}  // namespace

cudaError_t launch_icgn_partial(const SolveArgs &args, int model, int interp, int lanes, bool gauss,
                                cudaStream_t stream) {
    if (args.count <= 0) return cudaSuccess;
    if (!args.partial_index || !args.support || !args.support_box || args.support_words <= 0)
        return cudaErrorInvalidValue;
    SolveArgs a = args;
    a.persistent = 0;
    switch (model) {
    case kModelAffine: return by_weight<kModelAffine>(a, interp, lanes, gauss, stream);
    case kModelTranslation: return by_weight<kModelTranslation>(a, interp, lanes, gauss, stream);
    default: return cudaErrorInvalidValue;  // the ROI supports translation and affine windows only
    }
}

}  // namespace gbdic
