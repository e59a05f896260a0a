// Host runtime of the gbdic library (see engine.h).
//
// Each level (image scale) keeps its prepared reference resident in HBM
// (reference plane, metadata, inverse Hessians) and, per pipeline slot, its
// own target, coefficient plane and solver states, so that several frames can
// be in flight.  Frames are staged through pinned host buffers.
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <thread>

#include "engine.h"

namespace gbdic {

cudaError_t set_gauss_taps(const float *taps7);

namespace {

// Runtime taps of the target FIR: float32 values of the central 25 taps of
// the Gaussian(sigma 1) * inverse cubic B-spline filter
// (wgpu_backend.py:_fir_weights, 527-541), offsets -12..12.
const uint32_t kFirBits[25] = {
    0x318eddc4u, 0x3333f91eu, 0xb41a28f9u, 0x35101d98u, 0xb6067631u, 0x36fae8afu, 0xb7ea19e9u,
    0x38da6b5eu, 0xb9cbc9bfu, 0x3abe2309u, 0x3cad8b0cu, 0x3e738da4u, 0x3ef59511u, 0x3e738da4u,
    0x3cad8b0cu, 0x3abe2309u, 0xb9cbc9bfu, 0x38da6b5eu, 0xb7ea19e9u, 0x36fae8afu, 0xb6067631u,
    0x35101d98u, 0xb41a28f9u, 0x3333f91eu, 0x318eddc4u};

}  // namespace

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void fail(int code, const std::string &message) { throw Failure{code, message}; }

// Bounded host wait on an event (GBDIC_ETIMEOUT after `timeout_ms`).
void wait_event(cudaEvent_t ev, double timeout_ms) {
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t err = cudaEventQuery(ev);
        if (err == cudaSuccess) return;
        if (err != cudaErrorNotReady) check_cuda(err, "device execution");
        if (ms_since(t0) > timeout_ms) fail(GBDIC_ETIMEOUT, "device work did not complete within the wait limit");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

void validate_options(const gbdic_options &o) {
    if (o.motion_model < 0 || o.motion_model > 2) fail(GBDIC_EINVAL, "motion_model must be 'affine', 'translation', or 'quadratic'");
    if (o.interpolation < 0 || o.interpolation > 2) fail(GBDIC_EINVAL, "interpolation must be 'bspline', 'linear', or 'cubic'");
    if (o.subset_size < 4 || o.subset_size > 46340) fail(GBDIC_EINVAL, "subset_size must be an integer from 4 to 46340");
    if (o.subset_stride < 1 || o.subset_stride > o.subset_size) fail(GBDIC_EINVAL, "subset_stride must be between 1 and subset_size");
    if (o.spatial_weighting < 0 || o.spatial_weighting > 1) fail(GBDIC_EINVAL, "spatial_weighting must be 'uniform' or 'gaussian'");
    if (o.spatial_weighting == 1 && !(std::isfinite(o.gaussian_sigma) && o.gaussian_sigma > 0.0f))
        fail(GBDIC_EINVAL, "gaussian_sigma must be finite and greater than zero");
    if (o.outlier_policy < 0 || o.outlier_policy > 3) fail(GBDIC_EINVAL, "outlier_policy must be 'replace', 'flag', 'disabled', or 'median'");
    if (o.median_filter_size != 3 && o.median_filter_size != 5 && o.median_filter_size != 7 && o.median_filter_size != 9)
        fail(GBDIC_EINVAL, "median_filter_size must be one of 3, 5, 7, or 9 subsets");
    if (o.median_filter_scope < 0 || o.median_filter_scope > 1) fail(GBDIC_EINVAL, "median_filter_scope must be 'rejected' or 'all'");
    if (o.threads_per_subset != 16 && o.threads_per_subset != 32 && o.threads_per_subset != 64 && o.threads_per_subset != 128)
        fail(GBDIC_EINVAL, "threads_per_subset must be 16, 32, 64, or 128");
    if (o.divergence_patience < 0 || o.divergence_patience > 30) fail(GBDIC_EINVAL, "divergence_patience must be an integer from 0 to 30");
    if (o.divergence_min_iterations < 1 || o.divergence_min_iterations > 30)
        fail(GBDIC_EINVAL, "divergence_min_iterations must be an integer from 1 to 30");
    if (o.pipeline_slots < 1 || o.pipeline_slots > 64) fail(GBDIC_EINVAL, "pipeline_depth must be a positive integer");
    if (o.solver_mode < GBDIC_SOLVER_EXACT || o.solver_mode > GBDIC_SOLVER_STAGED_WIDE)
        fail(GBDIC_EINVAL, "solver_mode must be 'exact', 'fast', 'staged' or 'staged-wide'");
}

void validate_cfg(const gbdic_solver_cfg *c) {
    if (!c) fail(GBDIC_EINVAL, "solver configuration is required");
    if (c->iterations < 1 || c->iterations > 30) fail(GBDIC_EINVAL, "iterations must be between 1 and 30");
    if (!(std::isfinite(c->tolerance) && c->tolerance > 0.0f)) fail(GBDIC_EINVAL, "tolerance must be a finite positive number");
    if (!(std::isfinite(c->zncc_min) && c->zncc_min >= 0.0f && c->zncc_min <= 1.0f)) fail(GBDIC_EINVAL, "zncc_min must be between 0 and 1");
}

void grid_of(int W, int H, int S, int st, int &gw, int &gh) {
    if (W < S || H < S) { gw = gh = 0; return; }
    gw = 1 + (W - S) / st;
    gh = 1 + (H - S) / st;
}

void fir_taps(float out[25]) { std::memcpy(out, kFirBits, sizeof kFirBits); }

void check_cuda(cudaError_t err, const char *what) {
    if (err != cudaSuccess) throw Failure{GBDIC_ECUDA, std::string(what) + ": " + cudaGetErrorString(err)};
}

void DeviceBuffer::ensure(size_t bytes) {
    if (ptr_ != nullptr && bytes <= bytes_) return;
    reset();
    if (bytes == 0) return;
    check_cuda(cudaMalloc(&ptr_, bytes), "cudaMalloc");
    bytes_ = bytes;
}

void DeviceBuffer::reset() {
    if (ptr_ != nullptr) cudaFree(ptr_);
    ptr_ = nullptr;
    bytes_ = 0;
}

void HostBuffer::ensure(size_t bytes) {
    if (ptr_ != nullptr && bytes <= bytes_) return;
    reset();
    if (bytes == 0) return;
    check_cuda(cudaMallocHost(&ptr_, bytes), "cudaMallocHost");
    bytes_ = bytes;
}

void HostBuffer::reset() {
    if (ptr_ != nullptr) cudaFreeHost(ptr_);
    ptr_ = nullptr;
    bytes_ = 0;
}

Runtime::Runtime(const gbdic_options &options) {
    validate_options(options);
    opt_.o = options;
    opt_.lanes = options.threads_per_subset;
    device_ = options.device;
    int count = 0;
    check_cuda(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
    if (device_ < 0 || device_ >= count) fail(GBDIC_EINVAL, "CUDA device ordinal out of range");
    check_cuda(cudaSetDevice(device_), "cudaSetDevice");
    check_cuda(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_), "attribute");
    check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    float taps[25];
    std::memcpy(taps, kFirBits, sizeof taps);
    check_cuda(set_fir_taps(taps), "FIR taps");
    double g[7], gs = 0.0;
    for (int k = 0; k < 7; ++k) { g[k] = std::exp(-0.5 * (k - 3) * (k - 3)); gs += g[k]; }
    float gf[7];
    for (int k = 0; k < 7; ++k) gf[k] = (float)(g[k] / gs);
    check_cuda(set_gauss_taps(gf), "Gaussian taps");
    const int S = options.subset_size;
    opt_.weights.resize((size_t)S * S);
    double wsum = 0.0;
    const double half = 0.5 * (S - 1), sigma = options.gaussian_sigma;
    for (int r = 0; r < S; ++r)
        for (int c = 0; c < S; ++c) {
            double w = 1.0;
            if (options.spatial_weighting == 1) {
                const double x = c - half, y = r - half;
                w = std::exp(-0.5 * (x * x + y * y) / (sigma * sigma));
            }
            opt_.weights[(size_t)r * S + c] = (float)w;
            wsum += w;
        }
    opt_.weight_sum = (float)wsum;
    weights_.ensure(opt_.weights.size() * sizeof(float));
    check_cuda(cudaMemcpy(weights_.get(), opt_.weights.data(), opt_.weights.size() * sizeof(float),
                          cudaMemcpyHostToDevice), "weights upload");
    // exp(-(x^2 + y^2) / 2 sigma^2) = exp(-x^2 / 2 sigma^2) exp(-y^2 / 2 sigma^2)
    std::vector<float> axis((size_t)S, 1.0f);
    if (options.spatial_weighting == 1)
        for (int k = 0; k < S; ++k) axis[k] = (float)std::exp(-0.5 * (k - half) * (k - half) / (sigma * sigma));
    axis_weights_.ensure(axis.size() * sizeof(float));
    check_cuda(cudaMemcpy(axis_weights_.get(), axis.data(), axis.size() * sizeof(float), cudaMemcpyHostToDevice),
               "axis weights upload");
    if (options.persistent) persistent_grid(opt_.lanes);
}

Runtime::~Runtime() {
    if (stream_ != nullptr) {
        cudaSetDevice(device_);
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
    for (auto ev : profile_begin_) cudaEventDestroy(ev);
    for (auto ev : profile_end_) cudaEventDestroy(ev);
}

bool Runtime::fast_active() const {
    return opt_.o.solver_mode == GBDIC_SOLVER_FAST &&
           icgn_fast_supported(opt_.o.motion_model, opt_.o.interpolation, opt_.lanes);
}

void Runtime::set_mode(int mode) {
    if (mode < GBDIC_SOLVER_EXACT || mode > GBDIC_SOLVER_STAGED_WIDE)
        fail(GBDIC_EINVAL, "solver_mode must be 'exact', 'fast', 'staged' or 'staged-wide'");
    opt_.o.solver_mode = mode;
    if (opt_.o.persistent) persistent_grid(opt_.lanes);
}

void Runtime::set_variant(int lanes, bool persistent) {
    if (lanes != 16 && lanes != 32 && lanes != 64 && lanes != 128)
        fail(GBDIC_EINVAL, "threads_per_subset must be 16, 32, 64, or 128");
    opt_.lanes = lanes;
    opt_.o.threads_per_subset = lanes;
    opt_.o.persistent = persistent ? 1 : 0;
    if (persistent) persistent_grid(lanes);
}

int Runtime::persistent_grid(int lanes) {
    // Queried once per lane count outside any stream capture, then cached.
    const bool fast = opt_.o.solver_mode == GBDIC_SOLVER_FAST &&
                      icgn_fast_supported(opt_.o.motion_model, opt_.o.interpolation, lanes);
    // Staged tiles: occupancy of the widest-level variant (the engine's
    // levels differ in width only by factors of two).
    const int tile = (opt_.o.solver_mode == GBDIC_SOLVER_STAGED || opt_.o.solver_mode == GBDIC_SOLVER_STAGED_WIDE) &&
                             icgn_staged_supported(opt_.o.motion_model, opt_.o.interpolation, lanes, 4)
                         ? opt_.o.solver_mode - GBDIC_SOLVER_STAGED + 1
                         : 0;
    const int variant = fast ? 1 : (tile ? 1 + tile : 0);
    if (lanes != persistent_lanes_ || variant != persistent_variant_ || persistent_grid_ <= 0) {
        const bool gauss = opt_.o.spatial_weighting == 1;
        const int per_sm = fast   ? icgn_fast_occupancy(opt_.o.motion_model, lanes, gauss)
                           : tile ? icgn_staged_occupancy(opt_.o.motion_model, lanes, gauss, tile)
                                  : icgn_occupancy(opt_.o.motion_model, opt_.o.interpolation, lanes, gauss);
        persistent_grid_ = std::max(1, per_sm) * sm_count_;
        persistent_lanes_ = lanes;
        persistent_variant_ = variant;
    }
    return persistent_grid_;
}

void Runtime::configure_level(Level &level, int W, int H, int slots) {
    if (level.W == W && level.H == H && !level.slots.empty()) {
        // Same geometry (a reference rebuilt for every pair): keep the slot
        // allocations, clear their states as fresh slots would be.
        const size_t ss = (size_t)level.count * state_stride(opt_.o.motion_model) * sizeof(float);
        for (auto &sl : level.slots) {
            check_cuda(cudaMemsetAsync(sl->state.get(), 0, ss, stream_), "clear state");
            check_cuda(cudaMemsetAsync(sl->filtered.get(), 0, ss, stream_), "clear state");
        }
        ensure_slots(level, slots);
        return;
    }
    level.W = W;
    level.H = H;
    grid_of(W, H, opt_.o.subset_size, opt_.o.subset_stride, level.gw, level.gh);
    level.count = level.gw * level.gh;
    level.slots.clear();
    ensure_slots(level, slots);
}

void Runtime::ensure_slots(Level &level, int slots) {
    const size_t px = (size_t)level.W * level.H;
    const size_t ss = (size_t)level.count * state_stride(opt_.o.motion_model) * sizeof(float);
    while ((int)level.slots.size() < slots) {
        auto s = std::make_unique<LevelSlot>();
        s->frame.ensure(px);
        if (opt_.o.interpolation == kInterpBspline) s->coef.ensure(px * sizeof(float));
        s->state.ensure(ss);
        s->filtered.ensure(ss);
        s->seed.ensure(ss);
        s->active.ensure((size_t)level.count * sizeof(uint32_t));
        s->counter.ensure(sizeof(unsigned));
        check_cuda(cudaMemsetAsync(s->state.get(), 0, ss, stream_), "clear state");
        check_cuda(cudaMemsetAsync(s->filtered.get(), 0, ss, stream_), "clear state");
        level.slots.push_back(std::move(s));
    }
}

double Runtime::prepare_reference(Level &level, const uint8_t *device_image, const uint8_t *roi_selected,
                                  const float *roi_links) {
    const int model = opt_.o.motion_model, n = parameter_count(model);
    const size_t px = (size_t)level.W * level.H;
    level.plane.ensure(px * sizeof(float4));
    level.meta.ensure((size_t)level.count * meta_stride(model) * sizeof(float));
    level.inv.ensure((size_t)level.count * n * n * sizeof(float));
    level.intensity.ensure(px * sizeof(float));
    level.spline.ensure(px * sizeof(float));
    level.scratch.ensure(px * sizeof(float));
    level.valid.ensure(sizeof(unsigned));
    level.admissible.ensure((size_t)level.count);
    level.ref_image.ensure(px);
    check_cuda(cudaMemcpyAsync(level.ref_image.get(), device_image, px, cudaMemcpyDeviceToDevice, stream_),
               "reference bytes");
    level.partial_count = 0;
    level.roi = roi_selected != nullptr;
    if (roi_selected) {
        level.selected.ensure(level.count);
        check_cuda(cudaMemcpyAsync(level.selected.get(), roi_selected, level.count, cudaMemcpyHostToDevice, stream_), "ROI upload");
    }
    if (roi_links) {
        level.links.ensure((size_t)level.count * 4 * sizeof(float));
        check_cuda(cudaMemcpyAsync(level.links.get(), roi_links, (size_t)level.count * 4 * sizeof(float),
                                   cudaMemcpyHostToDevice, stream_), "ROI links upload");
    } else {
        level.links.reset();
    }
    check_cuda(cudaMemsetAsync(level.valid.get(), 0, sizeof(unsigned), stream_), "clear counter");
    PrepArgs a{};
    a.img = device_image;
    a.W = level.W; a.H = level.H; a.pitch = level.W;
    a.S = opt_.o.subset_size; a.stride = opt_.o.subset_stride;
    a.grid_w = level.gw; a.grid_h = level.gh; a.count = level.count;
    a.model = model; a.interp = opt_.o.interpolation; a.gaussian_weighting = opt_.o.spatial_weighting;
    a.weights = weights_.as<float>();
    a.axis_weights = axis_weights_.as<float>();
    a.weight_sum = opt_.weight_sum;
    a.selected = roi_selected ? level.selected.as<uint8_t>() : nullptr;
    a.intensity = level.intensity.as<float>();
    a.spline = level.spline.as<float>();
    a.scratch = level.scratch.as<float>();
    a.plane = level.plane.as<float4>();
    a.meta = level.meta.as<float>();
    a.inv = level.inv.as<float>();
    a.valid_count = level.valid.as<unsigned>();
    a.admissible = level.admissible.as<uint8_t>();
    a.moments = nullptr;
    if (quadratic_row_prep_supported(model, opt_.o.spatial_weighting, a.S, a.stride, a.grid_h)) {
        level.moments.ensure(quadratic_row_prep_moment_floats(level.count) * sizeof(float));
        a.moments = level.moments.as<float>();
    }
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    cudaEventRecord(e0, stream_);
    check_cuda(launch_reference_prep(a, stream_), "reference preparation launch");
    cudaEventRecord(e1, stream_);
    unsigned valid = 0;
    check_cuda(cudaMemcpyAsync(&valid, level.valid.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, stream_), "readback");
    wait_event(e1, kWaitMs);
    check_cuda(cudaStreamSynchronize(stream_), "reference preparation");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    level.valid_count = (int)valid;
    return ms;
}

void Runtime::upload_reference_arrays(Level &level, const float *plane, const float *meta, const float *inverse,
                                      const float *links) {
    const int model = opt_.o.motion_model, n = parameter_count(model);
    const size_t px = (size_t)level.W * level.H;
    level.plane.ensure(px * sizeof(float4));
    level.meta.ensure((size_t)level.count * meta_stride(model) * sizeof(float));
    level.inv.ensure((size_t)level.count * n * n * sizeof(float));
    level.partial_count = 0;
    check_cuda(cudaMemcpy(level.plane.get(), plane, px * sizeof(float4), cudaMemcpyHostToDevice), "plane upload");
    check_cuda(cudaMemcpy(level.meta.get(), meta, (size_t)level.count * meta_stride(model) * sizeof(float),
                          cudaMemcpyHostToDevice), "metadata upload");
    check_cuda(cudaMemcpy(level.inv.get(), inverse, (size_t)level.count * n * n * sizeof(float),
                          cudaMemcpyHostToDevice), "inverse upload");
    level.roi = links != nullptr;
    if (links) {
        level.links.ensure((size_t)level.count * 4 * sizeof(float));
        check_cuda(cudaMemcpy(level.links.get(), links, (size_t)level.count * 4 * sizeof(float),
                              cudaMemcpyHostToDevice), "links upload");
    } else {
        level.links.reset();
    }
    int valid = 0;
    std::vector<float> m((size_t)level.count * meta_stride(model));
    std::memcpy(m.data(), meta, m.size() * sizeof(float));
    std::vector<uint8_t> adm((size_t)level.count);
    for (int i = 0; i < level.count; ++i) {
        const float flag = m[(size_t)i * meta_stride(model) + 1];
        valid += flag > 0.5f;
        adm[(size_t)i] = (flag > 0.5f || flag == -4.0f) ? 1 : 0;
    }
    level.valid_count = valid;
    level.admissible.ensure((size_t)level.count);
    check_cuda(cudaMemcpy(level.admissible.get(), adm.data(), adm.size(), cudaMemcpyHostToDevice), "admissibility upload");
}

void Runtime::set_partial_support(Level &level, int count, const int32_t *indices, const uint32_t *words,
                                  int words_per_window, const float *boxes, const float *metadata_rows,
                                  const float *inverse_rows) {
    const auto &o = opt_.o;
    if (o.motion_model == GBDIC_MODEL_QUADRATIC) fail(GBDIC_EINVAL, "partial ROI windows support translation and affine models");
    if (count < 0 || (count > 0 && (!indices || !words || !boxes || !metadata_rows || !inverse_rows)))
        fail(GBDIC_EINVAL, "partial support tables are incomplete");
    if (count > 0 && words_per_window != (o.subset_size * o.subset_size + 31) / 32)
        fail(GBDIC_EINVAL, "words_per_window must be ceil(subset_size^2 / 32)");
    for (int k = 0; k < count; ++k)
        if (indices[k] < 0 || indices[k] >= level.count) fail(GBDIC_EINVAL, "partial window index out of range");
    check_cuda(cudaStreamSynchronize(stream_), "pending work");
    const int ms = gbdic::meta_stride(o.motion_model), n = gbdic::parameter_count(o.motion_model);
    std::vector<float> meta((size_t)level.count * ms), inv((size_t)level.count * n * n);
    std::vector<uint8_t> adm((size_t)level.count);
    check_cuda(cudaMemcpy(meta.data(), level.meta.get(), meta.size() * sizeof(float), cudaMemcpyDeviceToHost), "metadata");
    check_cuda(cudaMemcpy(inv.data(), level.inv.get(), inv.size() * sizeof(float), cudaMemcpyDeviceToHost), "inverse");
    check_cuda(cudaMemcpy(adm.data(), level.admissible.get(), adm.size(), cudaMemcpyDeviceToHost), "admissibility");
    for (int k = 0; k < count; ++k) {
        const size_t i = (size_t)indices[k];
        std::memcpy(&meta[i * ms], metadata_rows + (size_t)k * ms, ms * sizeof(float));
        std::memcpy(&inv[i * n * n], inverse_rows + (size_t)k * n * n, (size_t)n * n * sizeof(float));
        adm[i] = meta[i * ms + 1] == -4.0f ? 1 : 0;
    }
    check_cuda(cudaMemcpy(level.meta.get(), meta.data(), meta.size() * sizeof(float), cudaMemcpyHostToDevice), "metadata");
    check_cuda(cudaMemcpy(level.inv.get(), inv.data(), inv.size() * sizeof(float), cudaMemcpyHostToDevice), "inverse");
    check_cuda(cudaMemcpy(level.admissible.get(), adm.data(), adm.size(), cudaMemcpyHostToDevice), "admissibility");
    level.partial_count = count;
    level.support_words = words_per_window;
    if (count > 0) {
        level.partial_index.ensure((size_t)count * sizeof(int32_t));
        level.partial_words.ensure((size_t)count * words_per_window * sizeof(uint32_t));
        level.partial_boxes.ensure((size_t)count * 4 * sizeof(float));
        check_cuda(cudaMemcpy(level.partial_index.get(), indices, (size_t)count * sizeof(int32_t), cudaMemcpyHostToDevice),
                   "partial indices");
        check_cuda(cudaMemcpy(level.partial_words.get(), words, (size_t)count * words_per_window * sizeof(uint32_t),
                              cudaMemcpyHostToDevice), "support words");
        check_cuda(cudaMemcpy(level.partial_boxes.get(), boxes, (size_t)count * 4 * sizeof(float), cudaMemcpyHostToDevice),
                   "support boxes");
    }
    int valid = 0;
    for (int i = 0; i < level.count; ++i) valid += meta[(size_t)i * ms + 1] > 0.5f;
    level.valid_count = valid;
}

void Runtime::enqueue_prefilter(Level &level, LevelSlot &slot, const uint8_t *frame, cudaStream_t s) {
    if (opt_.o.interpolation != kInterpBspline) return;
    check_cuda(launch_fir_prefilter(frame ? frame : slot.frame.as<uint8_t>(), level.W, level.H, level.W,
                                    slot.coef.as<float>(), s),
               "prefilter launch");
}

SolveArgs Runtime::solve_args(Level &level, LevelSlot &slot, const gbdic_solver_cfg &cfg, bool seeded, bool preserve,
                              const uint8_t *frame, float *state) const {
    SolveArgs a{};
    a.coef = slot.coef.as<float>();
    a.img = frame ? frame : slot.frame.as<uint8_t>();
    a.plane = level.plane.as<float4>();
    a.meta = level.meta.as<float>();
    a.inv = level.inv.as<float>();
    a.weights = opt_.o.spatial_weighting == 1 ? weights_.as<float>() : nullptr;
    a.seed = seeded ? slot.seed.as<float>() : nullptr;
    a.active = seeded ? slot.active.as<uint32_t>() : nullptr;
    a.state = state ? state : slot.state.as<float>();
    a.work_counter = slot.counter.as<unsigned>();
    a.W = level.W; a.H = level.H; a.grid_w = level.gw; a.count = level.count;
    a.S = opt_.o.subset_size; a.stride = opt_.o.subset_stride;
    a.iterations = cfg.iterations; a.tolerance = cfg.tolerance; a.zncc_min = cfg.zncc_min;
    a.weight_sum = opt_.weight_sum;
    a.roi_enabled = level.roi ? 1 : 0;
    a.preserve_disabled = preserve ? 1 : 0;
    a.use_mean = opt_.o.subset_stride != opt_.o.subset_size;
    a.div_patience = level.divergence ? opt_.o.divergence_patience : 0;
    a.div_min = opt_.o.divergence_min_iterations;
    a.persistent = opt_.o.persistent;
    a.fast_segments = fast_active() ? icgn_fast_segments(opt_.o.subset_size, opt_.lanes) : 0;
    a.staged_tile = opt_.o.solver_mode == GBDIC_SOLVER_STAGED        ? 1
                    : opt_.o.solver_mode == GBDIC_SOLVER_STAGED_WIDE ? 2
                                                                     : 0;
    return a;
}

void Runtime::enqueue_solve(Level &level, LevelSlot &slot, const gbdic_solver_cfg &cfg, bool seeded, bool preserve,
                            const uint8_t *frame, float *state, cudaStream_t s) {
    SolveArgs a = solve_args(level, slot, cfg, seeded, preserve, frame, state);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    check_cuda(cudaStreamIsCapturing(s, &capture), "capture query");
    const bool timed = profiling_ && capture == cudaStreamCaptureStatusNone &&
                       profile_used_ < (int)profile_begin_.size();
    if (profiling_) a.iteration_total = profile_iterations_.as<unsigned long long>();
    int grid = 0;
    if (a.persistent) {
        grid = persistent_grid(opt_.lanes);
        check_cuda(cudaMemsetAsync(slot.counter.get(), 0, sizeof(unsigned), s), "queue reset");
    }
    if (timed) check_cuda(cudaEventRecord(profile_begin_[profile_used_], s), "profile event");
    check_cuda(launch_icgn(a, opt_.o.motion_model, opt_.o.interpolation, opt_.lanes, opt_.o.spatial_weighting == 1,
                           grid, s), "solver launch");
    if (level.partial_count > 0) {
        // Partial-support windows after the complete ones (their validity -4
        // makes the complete-window launch skip them).
        SolveArgs b = a;
        b.count = level.partial_count;
        b.partial_index = level.partial_index.as<int>();
        b.support = level.partial_words.as<uint32_t>();
        b.support_box = level.partial_boxes.as<float4>();
        b.support_words = level.support_words;
        check_cuda(launch_icgn_partial(b, opt_.o.motion_model, opt_.o.interpolation, opt_.lanes,
                                       opt_.o.spatial_weighting == 1, s), "partial solver launch");
    }
    if (timed) check_cuda(cudaEventRecord(profile_end_[profile_used_++], s), "profile event");
    if (profiling_) ++profile_launches_;
}

void Runtime::set_profiling(bool enable) {
    if (enable && profile_begin_.empty()) {
        profile_begin_.resize(4096);
        profile_end_.resize(4096);
        for (size_t i = 0; i < profile_begin_.size(); ++i) {
            check_cuda(cudaEventCreate(&profile_begin_[i]), "event");
            check_cuda(cudaEventCreate(&profile_end_[i]), "event");
        }
        profile_iterations_.ensure(sizeof(unsigned long long));
    }
    profiling_ = enable;
    profile_reset();
}

void Runtime::profile_reset() {
    profile_used_ = 0;
    profile_launches_ = 0;
    if (profile_iterations_.get())
        check_cuda(cudaMemset(profile_iterations_.get(), 0, sizeof(unsigned long long)), "profile reset");
}

void Runtime::profile_read(double &solver_ms, long long &launches, long long &timed, unsigned long long &iterations) {
    solver_ms = 0.0;
    for (int i = 0; i < profile_used_; ++i) {
        check_cuda(cudaEventSynchronize(profile_end_[i]), "profile sync");
        float ms = 0.0f;
        check_cuda(cudaEventElapsedTime(&ms, profile_begin_[i], profile_end_[i]), "profile elapsed");
        solver_ms += ms;
    }
    launches = profile_launches_;
    timed = profile_used_;
    iterations = 0;
    if (profile_iterations_.get())
        check_cuda(cudaMemcpy(&iterations, profile_iterations_.get(), sizeof(iterations), cudaMemcpyDeviceToHost),
                   "profile readback");
}

void Runtime::enqueue_solve_list(Level &level, LevelSlot &slot, const gbdic_solver_cfg &cfg, const int *list,
                                 int length, const unsigned *list_count, int lanes, const uint8_t *frame, float *state,
                                 cudaStream_t s) {
    if (level.partial_count > 0) fail(GBDIC_EINVAL, "listed solves need a reference without partial-support windows");
    if (lanes == 0) lanes = opt_.lanes;
    if (lanes != 16 && lanes != 32 && lanes != 64 && lanes != 128)
        fail(GBDIC_EINVAL, "threads_per_subset must be 16, 32, 64, or 128");
    SolveArgs a = solve_args(level, slot, cfg, true, false, frame, state);
    a.fast_segments = 0;
    a.staged_tile = 0;
    const int model = opt_.o.motion_model, interp = opt_.o.interpolation;
    check_cuda(launch_disabled_rows(a, model, level.count, s), "disabled rows");
    if (length <= 0) return;
    a.subset_list = list;
    a.list_count = list_count;
    a.count = length;
    int grid = 0;
    const bool gauss = opt_.o.spatial_weighting == 1;
    if (list_count != nullptr) {
        // a device-side length: a persistent grid over the list
        a.persistent = 1;
        const int per_sm = icgn_occupancy(model, interp, lanes, gauss);
        grid = std::max(1, per_sm) * sm_count_;
        check_cuda(cudaMemsetAsync(slot.counter.get(), 0, sizeof(unsigned), s), "queue reset");
    } else {
        a.persistent = 0;
    }
    check_cuda(launch_icgn(a, model, interp, lanes, gauss, grid, s), "listed solver launch");
}

void Runtime::enqueue_uod(Level &level, LevelSlot &slot, bool seed_mode, float *out, cudaStream_t s) {
    if (opt_.o.outlier_policy == GBDIC_OUTLIER_DISABLED) return;
    UodArgs u{};
    u.state = slot.state.as<float>();
    u.out = out ? out : slot.filtered.as<float>();
    u.meta = level.meta.as<float>();
    u.links = level.links.get() ? level.links.as<float>() : nullptr;
    u.grid_w = level.gw; u.grid_h = level.gh; u.count = level.count;
    u.subset_stride = opt_.o.subset_stride;
    u.model = opt_.o.motion_model;
    u.policy = opt_.o.outlier_policy;
    u.median_size = opt_.o.outlier_policy == GBDIC_OUTLIER_MEDIAN ? opt_.o.median_filter_size : 3;
    u.scope_all = opt_.o.median_filter_scope;
    u.seed_mode = seed_mode ? 1 : 0;
    u.roi_enabled = (level.roi && u.links != nullptr) ? 1 : 0;
    check_cuda(launch_uod(u, s), "UOD launch");
}

const float *Runtime::output_state(LevelSlot &slot) const {
    return opt_.o.outlier_policy == GBDIC_OUTLIER_DISABLED ? slot.state.as<float>() : slot.filtered.as<float>();
}

void Runtime::upload_frame(Level &level, LevelSlot &slot, const uint8_t *frame, int64_t row_stride,
                           HostBuffer &staging, cudaStream_t s) {
    const size_t W = (size_t)level.W, H = (size_t)level.H;
    staging.ensure(W * H);
    uint8_t *dst = staging.as<uint8_t>();
    host_copy_rows(dst, frame, W, H, row_stride);
    check_cuda(cudaMemcpyAsync(slot.frame.get(), dst, W * H, cudaMemcpyHostToDevice, s), "frame upload");
}

namespace {

// Fixed pool of copy workers.  run() executes part 0 on the caller and parts
// 1..n-1 on the workers and returns when all are done; calls are
// serialised.  A process forked after the pool started gets a new pool.
class CopyPool {
  public:
    static CopyPool &get() {
        static std::mutex guard;
        static CopyPool *pool = nullptr;
        std::lock_guard<std::mutex> lock(guard);
        if (pool == nullptr || pool->pid_ != getpid()) pool = new CopyPool();  // a forked child abandons the old one
        return *pool;
    }
    int width() const { return (int)workers_.size() + 1; }
    void run(int parts, const std::function<void(int)> &fn) {
        std::lock_guard<std::mutex> serial(run_mutex_);
        parts = std::min(parts, width());
        {
            std::lock_guard<std::mutex> lock(m_);
            job_ = &fn;
            parts_ = parts;
            next_ = 1;
            pending_ = parts - 1;
            ++generation_;
        }
        cv_.notify_all();
        fn(0);
        std::unique_lock<std::mutex> lock(m_);
        done_.wait(lock, [&] { return pending_ == 0; });
        job_ = nullptr;
    }

  private:
    CopyPool() : pid_(getpid()) {
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const int extra = (int)std::min(3u, hw > 1 ? hw - 1 : 0u);
        for (int i = 0; i < extra; ++i) {
            std::thread t([this] { loop(); });
            t.detach();
            workers_.push_back(0);
        }
    }
    void loop() {
        unsigned long long seen = 0;
        for (;;) {
            const std::function<void(int)> *fn = nullptr;
            int part = -1;
            {
                std::unique_lock<std::mutex> lock(m_);
                cv_.wait(lock, [&] { return generation_ != seen && next_ < parts_; });
                part = next_++;
                if (next_ >= parts_) seen = generation_;
                fn = job_;
            }
            (*fn)(part);
            std::lock_guard<std::mutex> lock(m_);
            if (--pending_ == 0) done_.notify_all();
        }
    }
    pid_t pid_;
    std::vector<int> workers_;
    std::mutex run_mutex_, m_;
    std::condition_variable cv_, done_;
    const std::function<void(int)> *job_ = nullptr;
    int parts_ = 0, next_ = 0, pending_ = 0;
    unsigned long long generation_ = 0;
};

constexpr size_t kParallelCopyBytes = 2u << 20;

}  // namespace

void host_copy(void *dst, const void *src, size_t bytes) {
    if (bytes < kParallelCopyBytes) {
        std::memcpy(dst, src, bytes);
        return;
    }
    CopyPool &pool = CopyPool::get();
    const int parts = std::max(1, std::min(pool.width(), (int)(bytes / (1u << 20))));
    const size_t chunk = (bytes + parts - 1) / parts;
    pool.run(parts, [&](int k) {
        const size_t begin = (size_t)k * chunk, end = std::min(bytes, begin + chunk);
        if (begin < end) std::memcpy(static_cast<uint8_t *>(dst) + begin, static_cast<const uint8_t *>(src) + begin,
                                     end - begin);
    });
}

void host_copy_rows(uint8_t *dst, const uint8_t *src, size_t width, size_t height, int64_t stride) {
    if (stride == (int64_t)width) {
        host_copy(dst, src, width * height);
        return;
    }
    if (width * height < kParallelCopyBytes) {
        for (size_t r = 0; r < height; ++r) std::memcpy(dst + r * width, src + (size_t)r * stride, width);
        return;
    }
    CopyPool &pool = CopyPool::get();
    const int parts = pool.width();
    const size_t rows = (height + parts - 1) / parts;
    pool.run(parts, [&](int k) {
        const size_t begin = (size_t)k * rows, end = std::min(height, begin + rows);
        for (size_t r = begin; r < end; ++r) std::memcpy(dst + r * width, src + (size_t)r * stride, width);
    });
}

}  // namespace gbdic

