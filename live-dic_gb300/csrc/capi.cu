// C ABI of the gbdic library (declarations and reference citations in
// include/gbdic.h).  Every entry point converts exceptions into a return
// code plus a message retrievable with gbdic_last_error().
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"

using gbdic::Failure;
using gbdic::check_cuda;
using gbdic::fail;

namespace {

thread_local std::string g_create_error;

struct SlotHost {
    gbdic::HostBuffer in, out;
    cudaEvent_t begin = nullptr, end = nullptr, done = nullptr;
    cudaEvent_t uploaded = nullptr, computed = nullptr;  // stream pipeline ordering
    bool pending = false;
    std::chrono::steady_clock::time_point submitted;
    double upload_ms = 0.0;
    cudaGraphExec_t graph = nullptr;
    void create() {
        check_cuda(cudaEventCreate(&begin), "event");
        check_cuda(cudaEventCreate(&end), "event");
        check_cuda(cudaEventCreateWithFlags(&done, cudaEventDisableTiming), "event");
        check_cuda(cudaEventCreateWithFlags(&uploaded, cudaEventDisableTiming), "event");
        check_cuda(cudaEventCreateWithFlags(&computed, cudaEventDisableTiming), "event");
    }
    void destroy() {
        if (graph) cudaGraphExecDestroy(graph);
        if (begin) cudaEventDestroy(begin);
        if (end) cudaEventDestroy(end);
        if (done) cudaEventDestroy(done);
        if (uploaded) cudaEventDestroy(uploaded);
        if (computed) cudaEventDestroy(computed);
        graph = nullptr;
        begin = end = done = uploaded = computed = nullptr;
    }
};

void fill_timing(gbdic_timing *t, const SlotHost &h, double execute_ms, double readback_ms) {
    if (!t) return;
    float dev = 0.0f;
    cudaEventElapsedTime(&dev, h.begin, h.end);
    t->upload_ms = h.upload_ms;
    t->execute_ms = execute_ms;
    t->readback_ms = readback_ms;
    t->total_ms = gbdic::ms_since(h.submitted);
    t->device_ms = dev;
}

template <typename Handle, typename F>
int guarded(Handle *h, F &&f) {
    if (h == nullptr) {
        g_create_error = "null handle";
        return GBDIC_EINVAL;
    }
    try {
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        f();
        return GBDIC_OK;
    } catch (const Failure &x) {
        h->error = x.message;
        return x.code;
    } catch (const std::exception &x) {
        h->error = x.what();
        return GBDIC_ECUDA;
    }
}

}  // namespace

struct gbdic_engine {
    std::unique_ptr<gbdic::Runtime> rt;
    gbdic::Level level;
    std::vector<SlotHost> host;
    std::vector<gbdic_solver_cfg> slot_cfg;
    bool ready = false;
    std::string error;
    int device = 0;
    // Stream pipeline (submit / retire): uploads and readbacks on their own
    // streams, so a slot's upload overlaps the previous frame's solve and its
    // readback the next one's.
    cudaStream_t upload = nullptr, readback = nullptr;
    ~gbdic_engine() {
        if (rt) {
            cudaSetDevice(device);
            cudaStreamSynchronize(rt->stream());
        }
        for (cudaStream_t st : {upload, readback}) {
            if (st) {
                cudaStreamSynchronize(st);
                cudaStreamDestroy(st);
            }
        }
        for (auto &h : host) h.destroy();
        level.slots.clear();
    }
    void sync_copies() const {
        for (cudaStream_t st : {upload, readback})
            if (st) check_cuda(cudaStreamSynchronize(st), "pending copies");
    }
    void require_ready(const char *what) const {
        if (!ready) fail(GBDIC_ESTATE, std::string("Call set_reference() before ") + what + "().");
    }
    void check_slot(int slot) const {
        if (slot < 0 || slot >= (int)host.size()) fail(GBDIC_EINVAL, "slot index out of range");
    }
};

extern "C" {

int gbdic_abi_version(void) { return GBDIC_ABI_VERSION; }

}  // extern "C"

void gbdic::set_thread_error(const std::string &message) { g_create_error = message; }

extern "C" {

const char *gbdic_last_error(const gbdic_engine *engine) {
    return engine ? engine->error.c_str() : g_create_error.c_str();
}

int gbdic_create(const gbdic_options *options, gbdic_engine **out) {
    if (!options || !out) {
        g_create_error = "options and output handle are required";
        return GBDIC_EINVAL;
    }
    *out = nullptr;
    auto *e = new gbdic_engine();
    try {
        gbdic::validate_options(*options);
        e->device = options->device;
        e->rt = std::make_unique<gbdic::Runtime>(*options);
        e->host = std::vector<SlotHost>(options->pipeline_slots);
        for (auto &h : e->host) h.create();
        check_cuda(cudaStreamCreateWithFlags(&e->upload, cudaStreamNonBlocking), "stream");
        check_cuda(cudaStreamCreateWithFlags(&e->readback, cudaStreamNonBlocking), "stream");
        e->slot_cfg.resize(options->pipeline_slots);
    } catch (const Failure &x) {
        g_create_error = x.message;
        delete e;
        return x.code;
    }
    *out = e;
    return GBDIC_OK;
}

void gbdic_destroy(gbdic_engine *engine) { delete engine; }

namespace {
// set_reference of a host (device = false) or device image.
int set_reference_impl(gbdic_engine *e, const uint8_t *image, bool device, int32_t width, int32_t height,
                       int64_t row_stride, const uint8_t *roi_selected, const float *roi_links, gbdic_ref_info *info) {
    return guarded(e, [&] {
        const auto &o = e->rt->opts().o;
        if (!image) fail(GBDIC_EINVAL, "image is required");
        if (width < 16 || height < 16) fail(GBDIC_EINVAL, "Image dimensions must each be at least 16 pixels.");
        if (row_stride < width) fail(GBDIC_EINVAL, "row_stride must be at least the width");
        int gw, gh;
        gbdic::grid_of(width, height, o.subset_size, o.subset_stride, gw, gh);
        if (gw < 1 || gh < 1)
            fail(GBDIC_EINVAL, "Reference dimensions must each be at least " + std::to_string(o.subset_size) + " pixels.");
        e->sync_copies();
        e->ready = false;
        e->rt->configure_level(e->level, width, height, (int)e->host.size());
        auto &slot = *e->level.slots[0];
        if (device)
            check_cuda(cudaMemcpy2DAsync(slot.frame.get(), (size_t)width, image, (size_t)row_stride, (size_t)width,
                                         (size_t)height, cudaMemcpyDeviceToDevice, e->rt->stream()),
                       "reference copy");
        else
            e->rt->upload_frame(e->level, slot, image, row_stride, e->host[0].in, e->rt->stream());
        const double ms = e->rt->prepare_reference(e->level, slot.frame.as<uint8_t>(), roi_selected, roi_links);
        for (auto &h : e->host) {
            if (h.graph) cudaGraphExecDestroy(h.graph);
            h.graph = nullptr;
            h.pending = false;
        }
        e->ready = true;
        if (info) {
            info->width = width; info->height = height;
            info->grid_width = gw; info->grid_height = gh;
            info->valid_count = e->level.valid_count;
            info->device_ms = ms;
        }
    });
}

}  // namespace

int gbdic_set_reference(gbdic_engine *e, const uint8_t *image, int32_t width, int32_t height, int64_t row_stride,
                        const uint8_t *roi_selected, const float *roi_links, gbdic_ref_info *info) {
    return set_reference_impl(e, image, false, width, height, row_stride, roi_selected, roi_links, info);
}

int gbdic_set_reference_device(gbdic_engine *e, const uint8_t *device_image, int32_t width, int32_t height,
                               int64_t row_stride, const uint8_t *roi_selected, const float *roi_links,
                               gbdic_ref_info *info) {
    return set_reference_impl(e, device_image, true, width, height, row_stride, roi_selected, roi_links, info);
}

int gbdic_set_reference_arrays(gbdic_engine *e, int32_t width, int32_t height, const float *plane,
                               const float *metadata, const float *inverse, const float *roi_links,
                               gbdic_ref_info *info) {
    return guarded(e, [&] {
        const auto &o = e->rt->opts().o;
        if (!plane || !metadata || !inverse) fail(GBDIC_EINVAL, "plane, metadata and inverse are required");
        int gw, gh;
        gbdic::grid_of(width, height, o.subset_size, o.subset_stride, gw, gh);
        if (width < 16 || height < 16 || gw < 1 || gh < 1) fail(GBDIC_EINVAL, "invalid reference dimensions");
        e->sync_copies();
        e->ready = false;
        e->rt->configure_level(e->level, width, height, (int)e->host.size());
        e->rt->upload_reference_arrays(e->level, plane, metadata, inverse, roi_links);
        e->ready = true;
        if (info) {
            info->width = width; info->height = height;
            info->grid_width = gw; info->grid_height = gh;
            info->valid_count = e->level.valid_count;
            info->device_ms = 0.0;
        }
    });
}

namespace {

// Frame stages of the single-scale engine on slot k (after the upload).
void enqueue_frame(gbdic_engine *e, int k, const gbdic_solver_cfg &cfg, bool seeded, bool preserve, bool prefilter) {
    auto &rt = *e->rt;
    auto &lvl = e->level;
    auto &slot = *lvl.slots[k];
    auto &h = e->host[k];
    cudaStream_t s = rt.stream();
    check_cuda(cudaEventRecord(h.begin, s), "event");
    if (prefilter) rt.enqueue_prefilter(lvl, slot, nullptr, s);
    rt.enqueue_solve(lvl, slot, cfg, seeded, preserve, nullptr, nullptr, s);
    rt.enqueue_uod(lvl, slot, false, nullptr, s);
    check_cuda(cudaEventRecord(h.end, s), "event");
}

void readback(gbdic_engine *e, int k, float *out_state, gbdic_timing *timing, std::chrono::steady_clock::time_point t_exec) {
    auto &rt = *e->rt;
    auto &lvl = e->level;
    auto &h = e->host[k];
    const size_t bytes = (size_t)lvl.count * gbdic::state_stride(rt.opts().o.motion_model) * sizeof(float);
    h.out.ensure(bytes);
    check_cuda(cudaMemcpyAsync(h.out.as<float>(), rt.output_state(*lvl.slots[k]), bytes, cudaMemcpyDeviceToHost,
                               rt.stream()), "state readback");
    check_cuda(cudaEventRecord(h.done, rt.stream()), "event");
    gbdic::wait_event(h.done, gbdic::kWaitMs);
    const double exec_ms = gbdic::ms_since(t_exec);
    const auto t_copy = std::chrono::steady_clock::now();
    if (out_state) gbdic::host_copy(out_state, h.out.as<float>(), bytes);
    fill_timing(timing, h, exec_ms, gbdic::ms_since(t_copy));
}

}  // namespace

int gbdic_register(gbdic_engine *e, const uint8_t *frame, int64_t row_stride, const gbdic_solver_cfg *cfg,
                   float *out_state, gbdic_timing *timing) {
    return guarded(e, [&] {
        e->require_ready("register");
        gbdic::validate_cfg(cfg);
        if (!frame) fail(GBDIC_EINVAL, "frame is required");
        if (row_stride < e->level.W) fail(GBDIC_EINVAL, "row_stride must be at least the width");
        auto &h = e->host[0];
        h.submitted = std::chrono::steady_clock::now();
        e->rt->upload_frame(e->level, *e->level.slots[0], frame, row_stride, h.in, e->rt->stream());
        h.upload_ms = gbdic::ms_since(h.submitted);
        const auto t_exec = std::chrono::steady_clock::now();
        enqueue_frame(e, 0, *cfg, false, false, true);
        readback(e, 0, out_state, timing, t_exec);
    });
}

int gbdic_register_seeded(gbdic_engine *e, const uint8_t *frame, int64_t row_stride, const float *seed_state,
                          const uint32_t *active, const gbdic_solver_cfg *cfg, float *out_state,
                          gbdic_timing *timing) {
    return guarded(e, [&] {
        e->require_ready("register_seeded");
        gbdic::validate_cfg(cfg);
        if (!frame || !seed_state || !active) fail(GBDIC_EINVAL, "frame, seed_state and active are required");
        if (row_stride < e->level.W) fail(GBDIC_EINVAL, "row_stride must be at least the width");
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        auto &h = e->host[0];
        const auto s = e->rt->stream();
        h.submitted = std::chrono::steady_clock::now();
        e->rt->upload_frame(lvl, slot, frame, row_stride, h.in, s);
        const size_t sb = (size_t)lvl.count * gbdic::state_stride(e->rt->opts().o.motion_model) * sizeof(float);
        check_cuda(cudaMemcpyAsync(slot.seed.get(), seed_state, sb, cudaMemcpyHostToDevice, s), "seed upload");
        check_cuda(cudaMemcpyAsync(slot.active.get(), active, (size_t)lvl.count * sizeof(uint32_t), cudaMemcpyHostToDevice, s),
                   "activity upload");
        h.upload_ms = gbdic::ms_since(h.submitted);
        const auto t_exec = std::chrono::steady_clock::now();
        enqueue_frame(e, 0, *cfg, true, false, true);
        readback(e, 0, out_state, timing, t_exec);
    });
}

int gbdic_reduce_frame(gbdic_engine *e, const gbdic_engine *finer, int32_t finer_slot) {
    return guarded(e, [&] {
        e->require_ready("reduce_frame");
        if (!finer || !finer->ready) fail(GBDIC_ESTATE, "the finer engine has no prepared reference");
        finer->check_slot(finer_slot);
        if (finer->device != e->device) fail(GBDIC_EINVAL, "both engines must use the same device");
        if (e->level.W != finer->level.W / 2 || e->level.H != finer->level.H / 2)
            fail(GBDIC_EINVAL, "this engine's frame must be half the finer engine's (width // 2, height // 2)");
        cudaStream_t s = e->rt->stream();
        // The finer engine's work on its frame precedes the reduction.
        cudaEvent_t done = nullptr;
        check_cuda(cudaEventCreateWithFlags(&done, cudaEventDisableTiming), "event");
        cudaError_t err = cudaEventRecord(done, finer->rt->stream());
        if (err == cudaSuccess) err = cudaStreamWaitEvent(s, done, 0);
        cudaEventDestroy(done);
        check_cuda(err, "stream order");
        check_cuda(gbdic::launch_reduce_half(finer->level.slots[finer_slot]->frame.as<uint8_t>(), finer->level.W,
                                             finer->level.H, e->level.slots[0]->frame.as<uint8_t>(), s),
                   "reduction launch");
    });
}

int gbdic_register_seeded_resident(gbdic_engine *e, const float *seed_state, const uint32_t *active,
                                   const gbdic_solver_cfg *cfg, float *out_state, gbdic_timing *timing) {
    return guarded(e, [&] {
        e->require_ready("register_seeded");
        gbdic::validate_cfg(cfg);
        if (!seed_state || !active) fail(GBDIC_EINVAL, "seed_state and active are required");
        if (e->host[0].pending) fail(GBDIC_ESTATE, "slot is still in flight; retire it first");
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        auto &h = e->host[0];
        const auto s = e->rt->stream();
        h.submitted = std::chrono::steady_clock::now();
        const size_t sb = (size_t)lvl.count * gbdic::state_stride(e->rt->opts().o.motion_model) * sizeof(float);
        check_cuda(cudaMemcpyAsync(slot.seed.get(), seed_state, sb, cudaMemcpyHostToDevice, s), "seed upload");
        check_cuda(cudaMemcpyAsync(slot.active.get(), active, (size_t)lvl.count * sizeof(uint32_t), cudaMemcpyHostToDevice, s),
                   "activity upload");
        h.upload_ms = gbdic::ms_since(h.submitted);
        const auto t_exec = std::chrono::steady_clock::now();
        enqueue_frame(e, 0, *cfg, true, false, true);
        readback(e, 0, out_state, timing, t_exec);
    });
}

int gbdic_retry_seeded(gbdic_engine *e, int32_t slot_index, const float *seed_state, const uint32_t *active,
                       const gbdic_solver_cfg *cfg, float *out_state, gbdic_timing *timing) {
    return guarded(e, [&] {
        e->require_ready("retry_seeded");
        gbdic::validate_cfg(cfg);
        e->check_slot(slot_index);
        if (!seed_state || !active) fail(GBDIC_EINVAL, "seed_state and active are required");
        if (e->host[slot_index].pending) fail(GBDIC_ESTATE, "slot is still in flight; retire it first");
        auto &lvl = e->level;
        auto &slot = *lvl.slots[slot_index];
        auto &h = e->host[slot_index];
        const auto s = e->rt->stream();
        h.submitted = std::chrono::steady_clock::now();
        const size_t sb = (size_t)lvl.count * gbdic::state_stride(e->rt->opts().o.motion_model) * sizeof(float);
        check_cuda(cudaMemcpyAsync(slot.seed.get(), seed_state, sb, cudaMemcpyHostToDevice, s), "seed upload");
        check_cuda(cudaMemcpyAsync(slot.active.get(), active, (size_t)lvl.count * sizeof(uint32_t), cudaMemcpyHostToDevice, s),
                   "activity upload");
        h.upload_ms = gbdic::ms_since(h.submitted);
        const auto t_exec = std::chrono::steady_clock::now();
        enqueue_frame(e, slot_index, *cfg, true, true, false);
        readback(e, slot_index, out_state, timing, t_exec);
    });
}

int gbdic_final_zncc(gbdic_engine *e, float *out_zncc) {
    return guarded(e, [&] {
        e->require_ready("final_zncc");
        if (!out_zncc) fail(GBDIC_EINVAL, "output is required");
        if (e->rt->opts().o.motion_model != GBDIC_MODEL_AFFINE || e->rt->opts().o.spatial_weighting != 0)
            fail(GBDIC_EINVAL, "include_zncc requires affine motion and uniform full windows");
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        gbdic::DeviceBuffer out;
        out.ensure((size_t)lvl.count * sizeof(float));
        gbdic::ZnccArgs z{};
        z.coef = slot.coef.as<float>();
        z.img = slot.frame.as<uint8_t>();
        z.plane = lvl.plane.as<float4>();
        z.state = e->rt->output_state(slot);
        z.out = out.as<float>();
        z.W = lvl.W; z.H = lvl.H; z.grid_w = lvl.gw; z.count = lvl.count;
        z.S = e->rt->opts().o.subset_size; z.stride = e->rt->opts().o.subset_stride;
        z.interp = e->rt->opts().o.interpolation;
        check_cuda(gbdic::launch_final_zncc(z, e->rt->stream()), "final ZNCC launch");
        check_cuda(cudaMemcpyAsync(out_zncc, out.get(), (size_t)lvl.count * sizeof(float), cudaMemcpyDeviceToHost,
                                   e->rt->stream()), "ZNCC readback");
        check_cuda(cudaStreamSynchronize(e->rt->stream()), "final ZNCC");
    });
}

int gbdic_submit(gbdic_engine *e, int32_t slot_index, const uint8_t *frame, int64_t row_stride,
                 const gbdic_solver_cfg *cfg) {
    return guarded(e, [&] {
        e->require_ready("register_stream");
        gbdic::validate_cfg(cfg);
        e->check_slot(slot_index);
        if (!frame) fail(GBDIC_EINVAL, "frame is required");
        if (row_stride < e->level.W) fail(GBDIC_EINVAL, "row_stride must be at least the width");
        auto &h = e->host[slot_index];
        if (h.pending) fail(GBDIC_ESTATE, "slot is still in flight; retire it first");
        h.submitted = std::chrono::steady_clock::now();
        // upload stream -> the engine's stream -> readback stream; a slot is
        // reused only after its retire waited for its readback
        cudaStream_t s = e->rt->stream();
        e->rt->upload_frame(e->level, *e->level.slots[slot_index], frame, row_stride, h.in, e->upload);
        check_cuda(cudaEventRecord(h.uploaded, e->upload), "event");
        check_cuda(cudaStreamWaitEvent(s, h.uploaded, 0), "upload wait");
        h.upload_ms = gbdic::ms_since(h.submitted);
        enqueue_frame(e, slot_index, *cfg, false, false, true);
        check_cuda(cudaEventRecord(h.computed, s), "event");
        auto &lvl = e->level;
        const size_t bytes = (size_t)lvl.count * gbdic::state_stride(e->rt->opts().o.motion_model) * sizeof(float);
        h.out.ensure(bytes);
        check_cuda(cudaStreamWaitEvent(e->readback, h.computed, 0), "compute wait");
        check_cuda(cudaMemcpyAsync(h.out.as<float>(), e->rt->output_state(*lvl.slots[slot_index]), bytes,
                                   cudaMemcpyDeviceToHost, e->readback), "state readback");
        check_cuda(cudaEventRecord(h.done, e->readback), "event");
        h.pending = true;
    });
}

int gbdic_retire(gbdic_engine *e, int32_t slot_index, float *out_state, gbdic_timing *timing) {
    return guarded(e, [&] {
        e->check_slot(slot_index);
        auto &h = e->host[slot_index];
        if (!h.pending) fail(GBDIC_ESTATE, "slot has no registration in flight");
        const auto t_wait = std::chrono::steady_clock::now();
        h.pending = false;
        gbdic::wait_event(h.done, gbdic::kWaitMs);
        const double wait_ms = gbdic::ms_since(t_wait);
        const auto t_copy = std::chrono::steady_clock::now();
        const size_t bytes = (size_t)e->level.count * gbdic::state_stride(e->rt->opts().o.motion_model) * sizeof(float);
        if (out_state) gbdic::host_copy(out_state, h.out.as<float>(), bytes);
        fill_timing(timing, h, wait_ms, gbdic::ms_since(t_copy));
    });
}

int gbdic_register_device(gbdic_engine *e, const uint8_t *device_frame, const gbdic_solver_cfg *cfg,
                          float *device_state, void *stream) {
    return guarded(e, [&] {
        e->require_ready("register");
        gbdic::validate_cfg(cfg);
        if (!device_frame || !device_state) fail(GBDIC_EINVAL, "device_frame and device_state are required");
        auto &rt = *e->rt;
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        cudaStream_t s = stream ? (cudaStream_t)stream : rt.stream();
        rt.enqueue_prefilter(lvl, slot, device_frame, s);
        const bool disabled = rt.opts().o.outlier_policy == GBDIC_OUTLIER_DISABLED;
        rt.enqueue_solve(lvl, slot, *cfg, false, false, device_frame, disabled ? device_state : nullptr, s);
        if (!disabled) rt.enqueue_uod(lvl, slot, false, device_state, s);
    });
}

int gbdic_field_summary(const float *packed, int64_t count, int32_t stride, int32_t n, float *accepted_tx,
                        float *accepted_ty, float *accepted_iterations, int64_t *accepted, int64_t *replaced) {
    if (!packed || count < 0 || n < 4 || stride < n + 2 || !accepted_tx || !accepted_ty || !accepted_iterations ||
        !accepted || !replaced) {
        gbdic::set_thread_error("field summary arguments are invalid");
        return GBDIC_EINVAL;
    }
    int64_t a = 0, r = 0;
    for (int64_t i = 0; i < count; ++i) {
        const float *s = packed + i * stride;
        const float status = s[n];
        if (status > 0.5f) {
            accepted_tx[a] = s[0];
            accepted_ty[a] = s[3];
            accepted_iterations[a] = s[n + 1];
            ++a;
        }
        r += status > 1.5f ? 1 : 0;
    }
    *accepted = a;
    *replaced = r;
    return GBDIC_OK;
}

int gbdic_set_partial_support(gbdic_engine *e, int32_t count, const int32_t *indices, const uint32_t *words,
                              int32_t words_per_window, const float *boxes, const float *metadata_rows,
                              const float *inverse_rows) {
    return guarded(e, [&] {
        e->require_ready("set_partial_support");
        e->rt->set_partial_support(e->level, count, indices, words, words_per_window, boxes, metadata_rows,
                                   inverse_rows);
        for (auto &h : e->host) {
            if (h.graph) cudaGraphExecDestroy(h.graph);
            h.graph = nullptr;
        }
    });
}

int gbdic_register_seeded_device(gbdic_engine *e, const uint8_t *device_frame, const float *device_seed,
                                 const uint32_t *device_active, const gbdic_solver_cfg *cfg, float *device_state,
                                 void *stream) {
    return guarded(e, [&] {
        e->require_ready("register_seeded");
        gbdic::validate_cfg(cfg);
        if (!device_frame || !device_seed || !device_active || !device_state)
            fail(GBDIC_EINVAL, "device frame, seed, activity and state are required");
        auto &rt = *e->rt;
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        cudaStream_t s = stream ? (cudaStream_t)stream : rt.stream();
        const size_t sb = (size_t)lvl.count * gbdic::state_stride(rt.opts().o.motion_model) * sizeof(float);
        check_cuda(cudaMemcpyAsync(slot.seed.get(), device_seed, sb, cudaMemcpyDeviceToDevice, s), "seed copy");
        check_cuda(cudaMemcpyAsync(slot.active.get(), device_active, (size_t)lvl.count * sizeof(uint32_t),
                                   cudaMemcpyDeviceToDevice, s), "activity copy");
        rt.enqueue_prefilter(lvl, slot, device_frame, s);
        const bool disabled = rt.opts().o.outlier_policy == GBDIC_OUTLIER_DISABLED;
        rt.enqueue_solve(lvl, slot, *cfg, true, false, device_frame, disabled ? device_state : nullptr, s);
        if (!disabled) rt.enqueue_uod(lvl, slot, false, device_state, s);
    });
}

int gbdic_resolve_seeded_device(gbdic_engine *e, const uint8_t *device_frame, const float *device_seed,
                                const uint32_t *device_active, const gbdic_solver_cfg *cfg, float *device_state,
                                void *stream) {
    return guarded(e, [&] {
        e->require_ready("resolve_seeded");
        gbdic::validate_cfg(cfg);
        if (!device_frame || !device_seed || !device_active || !device_state)
            fail(GBDIC_EINVAL, "device frame, seed, activity and state are required");
        auto &rt = *e->rt;
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        cudaStream_t s = stream ? (cudaStream_t)stream : rt.stream();
        const size_t sb = (size_t)lvl.count * gbdic::state_stride(rt.opts().o.motion_model) * sizeof(float);
        check_cuda(cudaMemcpyAsync(slot.seed.get(), device_seed, sb, cudaMemcpyDeviceToDevice, s), "seed copy");
        check_cuda(cudaMemcpyAsync(slot.active.get(), device_active, (size_t)lvl.count * sizeof(uint32_t),
                                   cudaMemcpyDeviceToDevice, s), "activity copy");
        // Same frame as the previous seeded registration: its B-spline
        // coefficients are still in the slot.
        const bool disabled = rt.opts().o.outlier_policy == GBDIC_OUTLIER_DISABLED;
        rt.enqueue_solve(lvl, slot, *cfg, true, false, device_frame, disabled ? device_state : nullptr, s);
        if (!disabled) rt.enqueue_uod(lvl, slot, false, device_state, s);
    });
}

int gbdic_solve_listed_device(gbdic_engine *e, const uint8_t *device_frame, const float *device_seed,
                              const uint32_t *device_active, const int32_t *device_list, int32_t list_length,
                              const uint32_t *device_list_count, int32_t prefilter, int32_t threads_per_subset,
                              const gbdic_solver_cfg *cfg, float *device_state, void *stream) {
    return guarded(e, [&] {
        e->require_ready("solve_listed");
        gbdic::validate_cfg(cfg);
        if (!device_frame || !device_seed || !device_active || !device_state || (!device_list && list_length > 0))
            fail(GBDIC_EINVAL, "device frame, seed, activity, list and state are required");
        auto &rt = *e->rt;
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        if (list_length < 0 || list_length > lvl.count) fail(GBDIC_EINVAL, "list_length must be in [0, subsets]");
        cudaStream_t s = stream ? (cudaStream_t)stream : rt.stream();
        const size_t sb = (size_t)lvl.count * gbdic::state_stride(rt.opts().o.motion_model) * sizeof(float);
        check_cuda(cudaMemcpyAsync(slot.seed.get(), device_seed, sb, cudaMemcpyDeviceToDevice, s), "seed copy");
        check_cuda(cudaMemcpyAsync(slot.active.get(), device_active, (size_t)lvl.count * sizeof(uint32_t),
                                   cudaMemcpyDeviceToDevice, s), "activity copy");
        if (prefilter) rt.enqueue_prefilter(lvl, slot, device_frame, s);
        const bool disabled = rt.opts().o.outlier_policy == GBDIC_OUTLIER_DISABLED;
        rt.enqueue_solve_list(lvl, slot, *cfg, reinterpret_cast<const int *>(device_list), list_length,
                              reinterpret_cast<const unsigned *>(device_list_count), threads_per_subset,
                              device_frame, disabled ? device_state : nullptr, s);
        if (!disabled) rt.enqueue_uod(lvl, slot, false, device_state, s);
    });
}

int gbdic_search_seeds_listed_device(gbdic_engine *e, const uint8_t *device_frame, float *device_seed,
                                     uint32_t *device_active, const int32_t *device_list,
                                     const uint32_t *device_list_count, int32_t radius, int32_t centered,
                                     void *stream) {
    return guarded(e, [&] {
        e->require_ready("seed search");
        auto &lvl = e->level;
        if (!device_frame || !device_seed || !device_active || !device_list || !device_list_count)
            fail(GBDIC_EINVAL, "device frame, seed, activity, list and list count are required");
        if (!lvl.ref_image.get()) fail(GBDIC_ESTATE, "seed search needs a reference prepared by set_reference()");
        const auto &o = e->rt->opts().o;
        if (radius < 1 || gbdic::zncc_search_smem(o.subset_size, radius) > 48 * 1024)
            fail(GBDIC_EINVAL, "radius must be >= 1 and its search tile must fit 48 KB of shared memory");
        gbdic::SearchArgs q{};
        q.ref = lvl.ref_image.as<uint8_t>();
        q.tgt = device_frame;
        q.seed = device_seed;
        q.active = device_active;
        q.selected = lvl.roi && lvl.selected.get() ? lvl.selected.as<uint8_t>() : nullptr;
        q.W = lvl.W; q.H = lvl.H; q.grid_w = lvl.gw; q.count = lvl.count;
        q.S = o.subset_size; q.stride = o.subset_stride; q.radius = radius; q.model = o.motion_model;
        q.centered = centered ? 1 : 0;
        q.subset_list = reinterpret_cast<const int *>(device_list);
        q.list_count = reinterpret_cast<const unsigned *>(device_list_count);
        cudaStream_t s = stream ? (cudaStream_t)stream : e->rt->stream();
        check_cuda(gbdic::launch_zncc_search(q, s), "seed search launch");
    });
}

int gbdic_search_seeds_device(gbdic_engine *e, const uint8_t *device_frame, float *device_seed,
                              uint32_t *device_active, const uint8_t *device_mask, int32_t radius, int32_t centered,
                              void *stream) {
    return guarded(e, [&] {
        e->require_ready("seed search");
        auto &lvl = e->level;
        if (!device_frame || !device_seed || !device_active) fail(GBDIC_EINVAL, "device frame, seed and activity are required");
        if (!lvl.ref_image.get()) fail(GBDIC_ESTATE, "seed search needs a reference prepared by set_reference()");
        const auto &o = e->rt->opts().o;
        if (radius < 1 || gbdic::zncc_search_smem(o.subset_size, radius) > 48 * 1024)
            fail(GBDIC_EINVAL, "radius must be >= 1 and its search tile must fit 48 KB of shared memory");
        gbdic::SearchArgs q{};
        q.ref = lvl.ref_image.as<uint8_t>();
        q.tgt = device_frame;
        q.seed = device_seed;
        q.active = device_active;
        q.selected = lvl.roi && lvl.selected.get() ? lvl.selected.as<uint8_t>() : nullptr;
        q.W = lvl.W; q.H = lvl.H; q.grid_w = lvl.gw; q.count = lvl.count;
        q.S = o.subset_size; q.stride = o.subset_stride; q.radius = radius; q.model = o.motion_model;
        q.centered = centered ? 1 : 0;
        q.subset_mask = device_mask;
        cudaStream_t s = stream ? (cudaStream_t)stream : e->rt->stream();
        check_cuda(gbdic::launch_zncc_search(q, s), "seed search launch");
    });
}

int gbdic_apply_uod(gbdic_engine *e, const float *state_in, int32_t seed_mode, float *state_out) {
    return guarded(e, [&] {
        e->require_ready("apply_uod");
        if (!state_in || !state_out) fail(GBDIC_EINVAL, "state_in and state_out are required");
        auto &rt = *e->rt;
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        const size_t bytes = (size_t)lvl.count * gbdic::state_stride(rt.opts().o.motion_model) * sizeof(float);
        cudaStream_t s = rt.stream();
        check_cuda(cudaMemcpyAsync(slot.state.get(), state_in, bytes, cudaMemcpyHostToDevice, s), "state upload");
        if (rt.opts().o.outlier_policy == GBDIC_OUTLIER_DISABLED) {
            check_cuda(cudaMemcpyAsync(slot.filtered.get(), slot.state.get(), bytes, cudaMemcpyDeviceToDevice, s), "copy");
        } else {
            rt.enqueue_uod(lvl, slot, seed_mode != 0, nullptr, s);
        }
        check_cuda(cudaMemcpyAsync(state_out, slot.filtered.get(), bytes, cudaMemcpyDeviceToHost, s), "state readback");
        check_cuda(cudaStreamSynchronize(s), "UOD");
    });
}

namespace {

// Device copies of a host snapshot / permission table for the spatial seed
// kernels, and the activity readback.
struct SpatialBuffers {
    gbdic::DeviceBuffer snapshot, prior, permissions, seeds, scores, active;
    void load(int count, const float *states, const float *prior_states, const uint32_t *perms, cudaStream_t s) {
        snapshot.ensure((size_t)count * 8 * sizeof(float));
        permissions.ensure((size_t)count * sizeof(uint32_t));
        seeds.ensure((size_t)count * 8 * sizeof(float));
        scores.ensure((size_t)count * 4 * sizeof(float));
        active.ensure((size_t)count * sizeof(uint32_t));
        check_cuda(cudaMemcpyAsync(snapshot.get(), states, (size_t)count * 8 * sizeof(float), cudaMemcpyHostToDevice, s),
                   "snapshot upload");
        check_cuda(cudaMemcpyAsync(permissions.get(), perms, (size_t)count * sizeof(uint32_t), cudaMemcpyHostToDevice, s),
                   "permission upload");
        if (prior_states) {
            prior.ensure((size_t)count * 8 * sizeof(float));
            check_cuda(cudaMemcpyAsync(prior.get(), prior_states, (size_t)count * 8 * sizeof(float),
                                       cudaMemcpyHostToDevice, s), "prior upload");
        }
        check_cuda(cudaMemsetAsync(seeds.get(), 0, (size_t)count * 8 * sizeof(float), s), "clear");
        check_cuda(cudaMemsetAsync(scores.get(), 0, (size_t)count * 4 * sizeof(float), s), "clear");
        check_cuda(cudaMemsetAsync(active.get(), 0, (size_t)count * sizeof(uint32_t), s), "clear");
    }
    void read(int count, float *out_seeds, float *out_scores, uint8_t *out_active, cudaStream_t s) {
        std::vector<uint32_t> act((size_t)count);
        if (out_seeds)
            check_cuda(cudaMemcpyAsync(out_seeds, seeds.get(), (size_t)count * 8 * sizeof(float), cudaMemcpyDeviceToHost, s),
                       "seed readback");
        if (out_scores)
            check_cuda(cudaMemcpyAsync(out_scores, scores.get(), (size_t)count * 4 * sizeof(float), cudaMemcpyDeviceToHost,
                                       s), "score readback");
        check_cuda(cudaMemcpyAsync(act.data(), active.get(), (size_t)count * sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
                   "activity readback");
        check_cuda(cudaStreamSynchronize(s), "spatial seeds");
        if (out_active)
            for (int i = 0; i < count; ++i) out_active[i] = act[(size_t)i] ? 1 : 0;
    }
};

}  // namespace

int gbdic_affine_frontier(gbdic_engine *e, const float *states, const uint32_t *permissions, float *out_seeds,
                          uint8_t *out_active) {
    return guarded(e, [&] {
        e->require_ready("affine_frontier_seeds");
        if (!states || !permissions) fail(GBDIC_EINVAL, "states and permissions are required");
        if (e->rt->opts().o.motion_model != GBDIC_MODEL_AFFINE)
            fail(GBDIC_EINVAL, "affine_frontier_seeds requires motion_model='affine'");
        auto &lvl = e->level;
        cudaStream_t s = e->rt->stream();
        SpatialBuffers b;
        b.load(lvl.count, states, nullptr, permissions, s);
        gbdic::FrontierArgs a{};
        a.snapshot = b.snapshot.as<float>();
        a.permissions = b.permissions.as<uint32_t>();
        a.seeds = b.seeds.as<float>();
        a.active = b.active.as<uint32_t>();
        a.count = lvl.count; a.grid_w = lvl.gw; a.stride = e->rt->opts().o.subset_stride;
        check_cuda(gbdic::launch_affine_frontier(a, s), "affine frontier launch");
        b.read(lvl.count, out_seeds, nullptr, out_active, s);
    });
}

int gbdic_spatial_choose(gbdic_engine *e, const float *states, const float *prior, const uint32_t *permissions,
                         const gbdic_choose_cfg *cfg, float *out_seeds, float *out_scores, uint8_t *out_active) {
    return guarded(e, [&] {
        e->require_ready("spatial seed selection");
        if (!states || !permissions || !cfg) fail(GBDIC_EINVAL, "states, permissions and cfg are required");
        if (cfg->sample_step < 1 || cfg->sample_step > e->rt->opts().o.subset_size)
            fail(GBDIC_EINVAL, "sample_step must be in [1, subset_size]");
        if (cfg->candidate_mode < 0 || cfg->candidate_mode > 2) fail(GBDIC_EINVAL, "candidate_mode must be 0, 1 or 2");
        if (!(cfg->min_gain >= 0.0f) || !(cfg->min_displacement >= 0.0f))
            fail(GBDIC_EINVAL, "min_gain and min_displacement must be non-negative");
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        if (!lvl.ref_image.get())
            fail(GBDIC_ESTATE, "spatial seed selection needs a reference prepared by set_reference()");
        cudaStream_t s = e->rt->stream();
        SpatialBuffers b;
        b.load(lvl.count, states, prior, permissions, s);
        gbdic::ChooseArgs a{};
        a.ref = lvl.ref_image.as<uint8_t>();
        a.tgt = slot.frame.as<uint8_t>();
        a.snapshot = b.snapshot.as<float>();
        a.prior = prior ? b.prior.as<float>() : nullptr;
        a.permissions = b.permissions.as<uint32_t>();
        a.seeds = b.seeds.as<float>();
        a.scores = b.scores.as<float>();
        a.active = b.active.as<uint32_t>();
        a.W = lvl.W; a.H = lvl.H; a.grid_w = lvl.gw; a.count = lvl.count;
        a.S = e->rt->opts().o.subset_size; a.stride = e->rt->opts().o.subset_stride;
        a.sample_step = cfg->sample_step;
        a.min_gain = cfg->min_gain; a.min_displacement = cfg->min_displacement;
        a.failed_only = cfg->failed_only ? 1 : 0; a.candidate_mode = cfg->candidate_mode;
        check_cuda(gbdic::launch_spatial_choose(a, s), "spatial choose launch");
        b.read(lvl.count, out_seeds, out_scores, out_active, s);
    });
}

int gbdic_export(gbdic_engine *e, int32_t what, void *host_out, int64_t bytes) {
    return guarded(e, [&] {
        e->require_ready("export");
        if (!host_out) fail(GBDIC_EINVAL, "output is required");
        auto &lvl = e->level;
        auto &slot = *lvl.slots[0];
        const int model = e->rt->opts().o.motion_model, n = gbdic::parameter_count(model);
        const void *src = nullptr;
        size_t size = 0;
        switch (what) {
        case GBDIC_EXPORT_COEFFICIENTS: src = slot.coef.get(); size = (size_t)lvl.W * lvl.H * sizeof(float); break;
        case GBDIC_EXPORT_PLANE: src = lvl.plane.get(); size = (size_t)lvl.W * lvl.H * sizeof(float4); break;
        case GBDIC_EXPORT_METADATA: src = lvl.meta.get(); size = (size_t)lvl.count * gbdic::meta_stride(model) * sizeof(float); break;
        case GBDIC_EXPORT_INVERSE: src = lvl.inv.get(); size = (size_t)lvl.count * n * n * sizeof(float); break;
        case GBDIC_EXPORT_RAW_STATE: src = slot.state.get(); size = (size_t)lvl.count * gbdic::state_stride(model) * sizeof(float); break;
        case GBDIC_EXPORT_OUTPUT_STATE: src = e->rt->output_state(slot); size = (size_t)lvl.count * gbdic::state_stride(model) * sizeof(float); break;
        case GBDIC_EXPORT_WEIGHTS: src = e->rt->weights().get(); size = e->rt->opts().weights.size() * sizeof(float); break;
        case GBDIC_EXPORT_FRAME: src = slot.frame.get(); size = (size_t)lvl.W * lvl.H; break;
        case GBDIC_EXPORT_ADMISSIBLE: src = lvl.admissible.get(); size = (size_t)lvl.count; break;
        case GBDIC_EXPORT_SEED: src = slot.seed.get(); size = (size_t)lvl.count * gbdic::state_stride(model) * sizeof(float); break;
        case GBDIC_EXPORT_ACTIVE: src = slot.active.get(); size = (size_t)lvl.count * sizeof(uint32_t); break;
        default: fail(GBDIC_EINVAL, "unknown export selector");
        }
        if (src == nullptr) fail(GBDIC_ESTATE, "buffer not available in this configuration");
        if ((size_t)bytes < size) fail(GBDIC_EINVAL, "output buffer too small: need " + std::to_string(size) + " bytes");
        check_cuda(cudaStreamSynchronize(e->rt->stream()), "pending work");
        check_cuda(cudaMemcpy(host_out, src, size, cudaMemcpyDeviceToHost), "export");
    });
}

}  // extern "C"

extern "C" {

int gbdic_set_solver_variant(gbdic_engine *e, int32_t threads_per_subset, int32_t persistent) {
    return guarded(e, [&] {
        check_cuda(cudaStreamSynchronize(e->rt->stream()), "pending work");
        e->rt->set_variant(threads_per_subset, persistent != 0);
        for (auto &h : e->host) {
            if (h.graph) cudaGraphExecDestroy(h.graph);
            h.graph = nullptr;
        }
    });
}

int gbdic_set_solver_mode(gbdic_engine *e, int32_t mode) {
    return guarded(e, [&] {
        check_cuda(cudaStreamSynchronize(e->rt->stream()), "pending work");
        e->rt->set_mode(mode);
        for (auto &h : e->host) {
            if (h.graph) cudaGraphExecDestroy(h.graph);
            h.graph = nullptr;
        }
    });
}

int gbdic_profile(gbdic_engine *e, int32_t enable) {
    return guarded(e, [&] {
        check_cuda(cudaStreamSynchronize(e->rt->stream()), "pending work");
        e->rt->set_profiling(enable != 0);
    });
}

int gbdic_profile_read(gbdic_engine *e, double *solver_ms, int64_t *launches, int64_t *timed_launches,
                       uint64_t *iterations) {
    return guarded(e, [&] {
        double ms = 0.0;
        long long n = 0, t = 0;
        unsigned long long it = 0;
        e->rt->profile_read(ms, n, t, it);
        if (solver_ms) *solver_ms = ms;
        if (launches) *launches = n;
        if (timed_launches) *timed_launches = t;
        if (iterations) *iterations = it;
    });
}

}  // extern "C"
