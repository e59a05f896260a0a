// gbdic_register_noalloc: one registration that allocates no memory.
//
// Some callers cannot call cudaMalloc at all: code that runs while a CUDA
// stream is being captured into a graph (an allocation would invalidate the
// capture), real-time loops whose latency budget forbids allocator calls, and
// plug-ins that live inside a host framework which owns every device
// allocation.  They hand over device buffers for the inputs (target bytes,
// prepared reference arrays) and the output state; the only scratch the path
// needs, the B-spline coefficient plane written by the FIR prefilter and read
// by the IC-GN solver, lives in the file-scope array below.
//
// The array is a fixed 8 MiB (2,097,152 float32 coefficients, e.g. one
// 1920x1080 frame) and every GPU that loads the library keeps it until the
// process exits.  Larger frames are rejected with GBDIC_EINVAL.  All calls
// share the one array and it keeps the last call's contents; the prefilter
// rewrites every coefficient of the frame before the solver reads any, so
// nothing has to be cleared.  Calls whose work overlaps on the GPU (two
// streams, or two threads) race on the array and must be serialised by the
// caller.
//
// The first call on a device, with that device current, resolves the
// array's device address with cudaGetSymbolAddress and uploads the FIR taps
// to constant memory; that first call should come before any stream capture.
// The cached address and taps belong to the device's context: after a
// cudaDeviceReset they are stale, so the entry point must not be used on a
// device that has been reset.
//
// Only complete windows are solved.  Partial-support windows (metadata
// validity -4) keep the status the solver gives invalid windows (-4 with
// roi_enabled, else -1) and zero parameters, and the stagnation stop is off
// (divergence_patience 0).
#include <cstring>
#include <mutex>
#include <string>

#include "engine.h"

namespace {

constexpr size_t kNoAllocMaxPixels = 2097152;  // 8 MiB of float32 coefficients

static __device__ __align__(256) float g_noalloc_coefficients[kNoAllocMaxPixels];

constexpr int kMaxDevices = 64;
struct DeviceScratch {
    bool ready = false;
    float *coefficients = nullptr;  // device address of g_noalloc_coefficients
};
DeviceScratch g_scratch[kMaxDevices];
std::mutex g_scratch_mutex;

// Once per device, with that device current: the array's device address
// (the host-side symbol is only a stand-in) and the FIR taps.
int scratch_for_current_device(float **coefficients, std::string &error) {
    int device = -1;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess || device < 0 || device >= kMaxDevices) {
        error = std::string("no usable current CUDA device: ") + cudaGetErrorString(err);
        return GBDIC_ECUDA;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    DeviceScratch &s = g_scratch[device];
    if (!s.ready) {
        void *address = nullptr;
        err = cudaGetSymbolAddress(&address, g_noalloc_coefficients);
        if (err != cudaSuccess || address == nullptr) {
            error = std::string("cudaGetSymbolAddress of the scratch array failed: ") + cudaGetErrorString(err);
            return GBDIC_ECUDA;
        }
        float taps[25];
        gbdic::fir_taps(taps);
        err = gbdic::set_fir_taps(taps);
        if (err != cudaSuccess) {
            error = std::string("FIR taps upload failed: ") + cudaGetErrorString(err);
            return GBDIC_ECUDA;
        }
        s.coefficients = static_cast<float *>(address);
        s.ready = true;
    }
    *coefficients = s.coefficients;
    return GBDIC_OK;
}

int fail_with(int code, const std::string &message) {
    gbdic::set_thread_error(message);
    return code;
}

}  // namespace

extern "C" int gbdic_register_noalloc(const gbdic_noalloc_frame *f, float *device_state, void *stream) {
    if (f == nullptr || device_state == nullptr) return fail_with(GBDIC_EINVAL, "frame description and state are required");
    if (!f->frame || !f->plane || !f->metadata || !f->inverse)
        return fail_with(GBDIC_EINVAL, "frame, plane, metadata and inverse device pointers are required");
    if (f->motion_model < 0 || f->motion_model > 2) return fail_with(GBDIC_EINVAL, "invalid motion_model");
    if (f->interpolation < 0 || f->interpolation > 2) return fail_with(GBDIC_EINVAL, "invalid interpolation");
    if (f->threads_per_subset != 16 && f->threads_per_subset != 32 && f->threads_per_subset != 64 &&
        f->threads_per_subset != 128)
        return fail_with(GBDIC_EINVAL, "threads_per_subset must be 16, 32, 64, or 128");
    if (f->subset_size < 4 || f->subset_stride < 1 || f->subset_stride > f->subset_size)
        return fail_with(GBDIC_EINVAL, "invalid subset_size / subset_stride");
    const gbdic_solver_cfg &c = f->cfg;
    if (c.iterations < 1 || c.iterations > 30 || !(c.tolerance > 0.0f) || !(c.zncc_min >= 0.0f && c.zncc_min <= 1.0f))
        return fail_with(GBDIC_EINVAL, "invalid solver configuration");
    int gw = 0, gh = 0;
    gbdic::grid_of(f->width, f->height, f->subset_size, f->subset_stride, gw, gh);
    if (f->width < 16 || f->height < 16 || gw < 1 || gh < 1) return fail_with(GBDIC_EINVAL, "invalid frame dimensions");
    const size_t pixels = (size_t)f->width * (size_t)f->height;
    if (pixels > kNoAllocMaxPixels)
        return fail_with(GBDIC_EINVAL, "frame of " + std::to_string(pixels) + " pixels exceeds the " +
                                           std::to_string(kNoAllocMaxPixels) +
                                           "-pixel scratch of gbdic_register_noalloc");
    float *coefficients = nullptr;
    std::string error;
    const int rc = scratch_for_current_device(&coefficients, error);
    if (rc != GBDIC_OK) return fail_with(rc, error);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (f->interpolation == gbdic::kInterpBspline) {
        cudaError_t err = gbdic::launch_fir_prefilter(f->frame, f->width, f->height, f->width, coefficients, s);
        if (err != cudaSuccess) return fail_with(GBDIC_ECUDA, std::string("prefilter launch: ") + cudaGetErrorString(err));
    }
    gbdic::SolveArgs a{};
    a.coef = coefficients;
    a.img = f->frame;
    a.plane = reinterpret_cast<const float4 *>(f->plane);
    a.meta = f->metadata;
    a.inv = f->inverse;
    a.weights = f->weights;
    a.state = device_state;
    a.W = f->width; a.H = f->height; a.grid_w = gw; a.count = gw * gh;
    a.S = f->subset_size; a.stride = f->subset_stride;
    a.iterations = c.iterations; a.tolerance = c.tolerance; a.zncc_min = c.zncc_min;
    a.roi_enabled = f->roi_enabled ? 1 : 0;
    a.use_mean = f->subset_stride != f->subset_size;
    a.div_min = 4;
    cudaError_t err = gbdic::launch_icgn(a, f->motion_model, f->interpolation, f->threads_per_subset,
                                         f->weights != nullptr, 0, s);
    if (err != cudaSuccess) return fail_with(GBDIC_ECUDA, std::string("solver launch: ") + cudaGetErrorString(err));
    return GBDIC_OK;
}
