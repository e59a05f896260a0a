// Full GPU-resident pyramid engine (reference: full_pyramid_backend.py,
// ICGNWGPUFullPyramid, 158-1926).  Per frame, inside one CUDA graph per
// slot: upload the finest target, reduce it level by level, solve the
// coarsest level (zero seed, or seeded from the temporal history), then for
// each finer level transfer the coarse field, prefilter, solve seeded and
// apply UOD; finally merge the finest field into the temporal history and
// read back the finest state and four counters.
#include <cstring>
#include <string>

#include "engine.h"

using gbdic::Failure;
using gbdic::check_cuda;
using gbdic::fail;

namespace {

struct PyramidSlot {
    gbdic::HostBuffer in, out, counters_host;
    gbdic::DeviceBuffer counters;  // 4 x u32
    gbdic::HostBuffer shift_host;  // global translation seed (dx, dy), read at graph launch
    gbdic::DeviceBuffer shift_dev;
    cudaEvent_t begin = nullptr, end = nullptr;
    cudaEvent_t uploaded = nullptr, computed = nullptr;  // copy-stream ordering
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // whole pyramid, finest level alone
    bool pending = false;
    std::chrono::steady_clock::time_point submitted;
    double upload_ms = 0.0;
    void create() {
        check_cuda(cudaEventCreate(&begin), "event");
        check_cuda(cudaEventCreate(&end), "event");
        check_cuda(cudaEventCreateWithFlags(&uploaded, cudaEventDisableTiming), "event");
        check_cuda(cudaEventCreateWithFlags(&computed, cudaEventDisableTiming), "event");
        counters.ensure(4 * sizeof(uint32_t));
        counters_host.ensure(4 * sizeof(uint32_t));
        shift_host.ensure(2 * sizeof(float));
        shift_dev.ensure(2 * sizeof(float));
        shift_host.as<float>()[0] = shift_host.as<float>()[1] = 0.0f;
    }
    void drop_graphs() {
        for (auto &g : graph) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
    }
    void destroy() {
        drop_graphs();
        if (begin) cudaEventDestroy(begin);
        if (end) cudaEventDestroy(end);
        if (uploaded) cudaEventDestroy(uploaded);
        if (computed) cudaEventDestroy(computed);
        begin = end = uploaded = computed = nullptr;
    }
};

thread_local std::string g_pyramid_error;

}  // namespace

struct gbdic_pyramid {
    std::unique_ptr<gbdic::Runtime> rt;
    gbdic_pyramid_options po{};
    std::vector<std::unique_ptr<gbdic::Level>> levels;  // 0 = finest
    std::vector<std::unique_ptr<gbdic::DeviceBuffer>> seed_links;
    std::vector<bool> has_seed_links;
    gbdic::DeviceBuffer temporal_links;
    bool has_temporal_links = false;
    gbdic::DeviceBuffer history, ages, prev_history, prev_ages, prediction;
    gbdic::DeviceBuffer coarse_history, coarse_ages;  // temporal fine correction
    gbdic::DeviceBuffer fine_links;                   // adaptive: projection onto the finest grid
    int active_levels = 0;                            // levels the next frames run
    // Side stream and events of the prefilter branch: the finer levels'
    // B-spline prefilters run beside the reductions and coarse solves.
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, reduced_ev[4] = {}, filtered_ev[4] = {};
    // Host-frame pipeline: uploads and readbacks on their own streams, so a
    // slot's upload overlaps the previous frame's solve and its readback the
    // next one's.
    cudaStream_t upload = nullptr, readback = nullptr;
    std::vector<PyramidSlot> slots;
    bool ready = false;
    std::string error;
    int device = 0;

    ~gbdic_pyramid() {
        if (rt) {
            cudaSetDevice(device);
            cudaStreamSynchronize(rt->stream());
        }
        if (side) {
            cudaStreamSynchronize(side);
            cudaStreamDestroy(side);
        }
        for (cudaStream_t st : {upload, readback}) {
            if (st) {
                cudaStreamSynchronize(st);
                cudaStreamDestroy(st);
            }
        }
        if (fork_ev) cudaEventDestroy(fork_ev);
        for (auto &e : reduced_ev)
            if (e) cudaEventDestroy(e);
        for (auto &e : filtered_ev)
            if (e) cudaEventDestroy(e);
        for (auto &s : slots) s.destroy();
        levels.clear();
    }
    int L() const { return (int)levels.size(); }
    bool temporal() const { return po.initialization == 1; }
    // ZNCC integer seed search at the coarsest level: initialization 2;
    // temporal initialization with a search radius (subsets without
    // history); or Fourier initialization with a search radius (shifts
    // centred on the global translation, the residual of a non-rigid field).
    bool search() const { return po.seed_search_radius > 0 && po.initialization >= 1 && po.initialization <= 3; }
    bool velocity() const { return po.temporal_prediction == 1; }
    bool fine_correction() const { return po.temporal_fine_correction != 0; }
    // Global translation seed of the coarsest level (Fourier initialization).
    bool global() const { return po.initialization == 3; }
    gbdic_solver_cfg cfg_of(int level) const {
        const int schedule = L() - 1 - level;  // options are coarsest first
        return gbdic_solver_cfg{po.iterations[schedule], po.tolerance[schedule], po.zncc_min};
    }
    size_t state_bytes(int level) const {
        return (size_t)levels[level]->count * gbdic::state_stride(po.base.motion_model) * sizeof(float);
    }
};

namespace {

template <typename F>
int pguarded(gbdic_pyramid *p, F &&f) {
    if (p == nullptr) {
        g_pyramid_error = "null handle";
        return GBDIC_EINVAL;
    }
    try {
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        f();
        return GBDIC_OK;
    } catch (const Failure &x) {
        p->error = x.message;
        return x.code;
    } catch (const std::exception &x) {
        p->error = x.what();
        return GBDIC_ECUDA;
    }
}

void reset_temporal(gbdic_pyramid *p, cudaStream_t s) {
    if (!p->temporal()) return;
    const int count = p->levels[0]->count;
    const int model = p->po.base.motion_model, ss = gbdic::state_stride(model);
    std::vector<float> state((size_t)count * ss, 0.0f);
    for (int i = 0; i < count; ++i) state[(size_t)i * ss + gbdic::parameter_count(model)] = -1.0f;
    check_cuda(cudaMemcpy(p->history.get(), state.data(), state.size() * sizeof(float), cudaMemcpyHostToDevice), "history");
    check_cuda(cudaMemset(p->ages.get(), 0xff, (size_t)count * sizeof(uint32_t)), "ages");
    if (p->velocity()) {
        check_cuda(cudaMemcpy(p->prev_history.get(), state.data(), state.size() * sizeof(float), cudaMemcpyHostToDevice),
                   "history");
        check_cuda(cudaMemset(p->prev_ages.get(), 0xff, (size_t)count * sizeof(uint32_t)), "ages");
    }
    if (p->fine_correction()) {
        const int cc = p->levels.back()->count;
        std::vector<float> coarse((size_t)cc * ss, 0.0f);
        for (int i = 0; i < cc; ++i) coarse[(size_t)i * ss + gbdic::parameter_count(model)] = -1.0f;
        check_cuda(cudaMemcpy(p->coarse_history.get(), coarse.data(), coarse.size() * sizeof(float),
                              cudaMemcpyHostToDevice), "history");
        check_cuda(cudaMemset(p->coarse_ages.get(), 0xff, (size_t)cc * sizeof(uint32_t)), "ages");
    }
    p->active_levels = p->L();
    (void)s;
}

// Everything a frame does after its finest target is resident at `frame0`.
// `L` = levels this frame runs (the whole pyramid, or 1 under the adaptive
// policy: full_pyramid_backend.py:1447-1481).
void enqueue_pyramid(gbdic_pyramid *p, int k, const uint8_t *frame0, float *out_state, cudaStream_t s) {
    auto &rt = *p->rt;
    const int L = p->active_levels;
    const int model = p->po.base.motion_model;
    const bool median = p->po.base.outlier_policy == GBDIC_OUTLIER_MEDIAN;
    auto &ps = p->slots[k];
    // Levels 0 .. L-2 are prefiltered on the side stream (frame 0 as soon as
    // it is resident, level l after its reduction); each seeded solve waits
    // for its level's prefilter.  The coarsest level stays on `s`.
    const bool branch = L > 1 && p->rt->opts().o.interpolation == GBDIC_INTERP_BSPLINE;
    if (branch) {
        check_cuda(cudaEventRecord(p->fork_ev, s), "fork");
        check_cuda(cudaStreamWaitEvent(p->side, p->fork_ev, 0), "fork");
        rt.enqueue_prefilter(*p->levels[0], *p->levels[0]->slots[k], frame0, p->side);
        check_cuda(cudaEventRecord(p->filtered_ev[0], p->side), "prefilter event");
    }
    const uint8_t *prev = frame0;
    for (int l = 1; l < L; ++l) {
        auto &lvl = *p->levels[l];
        auto &src = *p->levels[l - 1];
        check_cuda(gbdic::launch_reduce_half(prev, src.W, src.H, lvl.slots[k]->frame.as<uint8_t>(), s), "reduce launch");
        prev = lvl.slots[k]->frame.as<uint8_t>();
        if (branch && l < L - 1) {
            check_cuda(cudaEventRecord(p->reduced_ev[l], s), "reduce event");
            check_cuda(cudaStreamWaitEvent(p->side, p->reduced_ev[l], 0), "reduce event");
            rt.enqueue_prefilter(lvl, *lvl.slots[k], nullptr, p->side);
            check_cuda(cudaEventRecord(p->filtered_ev[l], p->side), "prefilter event");
        }
    }
    check_cuda(cudaMemsetAsync(ps.counters.get(), 0, 4 * sizeof(uint32_t), s), "counter reset");
    const int c = L - 1;
    auto &coarse = *p->levels[c];
    auto &cslot = *coarse.slots[k];
    const uint8_t *cframe = c == 0 ? frame0 : nullptr;
    bool seeded = false;
    if (p->global()) {
        // full_pyramid_backend.py:1704-1714: every ROI-selected coarsest
        // subset starts from (dx, dy) / 2^(levels - 1).
        check_cuda(cudaMemcpyAsync(ps.shift_dev.get(), ps.shift_host.as<float>(), 2 * sizeof(float),
                                   cudaMemcpyHostToDevice, s), "translation seed upload");
        check_cuda(gbdic::launch_uniform_seed(cslot.seed.as<float>(), cslot.active.as<uint32_t>(),
                                              coarse.roi ? coarse.selected.as<uint8_t>() : nullptr, coarse.count, model,
                                              ps.shift_dev.as<float>(), 1.0f / (float)(1 << c), s),
                   "translation seed launch");
        seeded = true;
    }
    if (p->temporal()) {
        auto &fine = *p->levels[0];
        gbdic::TemporalArgs t{};
        t.history = p->history.as<float>();
        t.ages = p->ages.as<uint32_t>();
        t.prev_history = p->prev_history.as<float>();
        t.prev_ages = p->prev_ages.as<uint32_t>();
        t.prediction = p->prediction.as<float>();
        t.counters = ps.counters.as<unsigned>();
        t.count = fine.count;
        t.model = model;
        if (p->velocity()) check_cuda(gbdic::launch_temporal_predict(t, s), "prediction launch");
        gbdic::SeedArgs a{};
        a.source = p->velocity() ? p->prediction.as<float>() : p->history.as<float>();
        a.seed = cslot.seed.as<float>();
        a.active = cslot.active.as<uint32_t>();
        if (c == 0 && p->po.adaptive)
            a.links = p->fine_links.as<uint32_t>();  // finest grid alone: selected windows only
        else
            a.links = p->has_temporal_links && c == p->L() - 1 ? p->temporal_links.as<uint32_t>() : nullptr;
        a.src_grid_w = fine.gw; a.src_grid_h = fine.gh;
        a.dst_grid_w = coarse.gw; a.dst_count = coarse.count;
        a.src_scale = 1.0f; a.dst_scale = (float)(1 << c);
        a.subset_size = (float)p->po.base.subset_size; a.subset_stride = (float)p->po.base.subset_stride;
        a.model = model;
        a.projected = ps.counters.as<unsigned>();
        a.mark_missing = p->search() ? 1 : 0;
        a.track = p->fine_correction() ? 1 : 0;
        check_cuda(gbdic::launch_transfer_seed(a, s), "projection launch");
        seeded = true;
    }
    if (p->search() && c == p->L() - 1) {
        // ZNCC integer search at the coarsest level: every subset (zncc
        // initialization), only those without a temporal seed, or every
        // subset around the global translation seed (Fourier).
        gbdic::SearchArgs q{};
        q.ref = coarse.ref_image.as<uint8_t>();
        q.tgt = cframe ? cframe : cslot.frame.as<uint8_t>();
        q.seed = cslot.seed.as<float>();
        q.active = cslot.active.as<uint32_t>();
        q.selected = coarse.roi ? coarse.selected.as<uint8_t>() : nullptr;
        q.searched = nullptr;
        q.W = coarse.W; q.H = coarse.H; q.grid_w = coarse.gw; q.count = coarse.count;
        q.S = p->po.base.subset_size; q.stride = p->po.base.subset_stride;
        q.radius = p->po.seed_search_radius;
        q.model = model;
        q.only_missing = p->temporal() ? 1 : 0;
        q.centered = p->global() ? 1 : 0;
        check_cuda(gbdic::launch_zncc_search(q, s), "seed search launch");
        seeded = true;
    }
    rt.enqueue_prefilter(coarse, cslot, cframe, s);
    rt.enqueue_solve(coarse, cslot, p->cfg_of(c), seeded, false, cframe, nullptr, s);
    rt.enqueue_uod(coarse, cslot, median && c > 0, nullptr, s);
    for (int l = L - 2; l >= 0; --l) {
        auto &lvl = *p->levels[l];
        auto &src = *p->levels[l + 1];
        auto &slot = *lvl.slots[k];
        gbdic::SeedArgs a{};
        a.source = rt.output_state(*src.slots[k]);
        a.seed = slot.seed.as<float>();
        a.active = slot.active.as<uint32_t>();
        a.links = p->has_seed_links[l] ? p->seed_links[l]->as<uint32_t>() : nullptr;
        a.src_grid_w = src.gw; a.src_grid_h = src.gh;
        a.dst_grid_w = lvl.gw; a.dst_count = lvl.count;
        a.src_scale = (float)(1 << (l + 1)); a.dst_scale = (float)(1 << l);
        a.subset_size = (float)p->po.base.subset_size; a.subset_stride = (float)p->po.base.subset_stride;
        a.model = model;
        a.track = p->fine_correction() ? 1 : 0;
        check_cuda(gbdic::launch_transfer_seed(a, s), "transfer launch");
        if (l == 0 && p->temporal() && p->fine_correction()) {
            gbdic::SeedArgs r = a;
            r.source = p->coarse_history.as<float>();
            r.history = p->history.as<float>();
            r.history_ages = p->ages.as<uint32_t>();
            r.source_ages = p->coarse_ages.as<uint32_t>();
            r.max_age = p->po.temporal_max_age;
            check_cuda(gbdic::launch_refine_temporal_seed(r, s), "temporal correction launch");
        }
        const uint8_t *f = l == 0 ? frame0 : nullptr;
        if (branch) check_cuda(cudaStreamWaitEvent(s, p->filtered_ev[l], 0), "prefilter join");
        else rt.enqueue_prefilter(lvl, slot, f, s);
        rt.enqueue_solve(lvl, slot, p->cfg_of(l), true, false, f, nullptr, s);
        rt.enqueue_uod(lvl, slot, median && l > 0, nullptr, s);
    }
    auto &fine = *p->levels[0];
    auto &fslot = *fine.slots[k];
    if (p->temporal()) {
        gbdic::TemporalArgs t{};
        t.history = p->history.as<float>();
        t.ages = p->ages.as<uint32_t>();
        t.raw = fslot.state.as<float>();
        t.output = rt.output_state(fslot);
        t.prev_history = p->prev_history.as<float>();
        t.prev_ages = p->prev_ages.as<uint32_t>();
        t.counters = ps.counters.as<unsigned>();
        t.count = fine.count;
        t.model = model;
        t.max_age = p->po.temporal_max_age;
        t.use_filtered = (p->po.base.outlier_policy == GBDIC_OUTLIER_REPLACE && !p->velocity()) ? 1 : 0;
        t.report_expiry = p->po.adaptive ? 1 : 0;
        if (p->velocity()) check_cuda(gbdic::launch_temporal_save_previous(t, s), "history save launch");
        check_cuda(gbdic::launch_temporal_merge(t, s), "history merge launch");
        if (p->fine_correction()) {
            // The coarse accepted history (no counters).  A frame that ran the
            // finest level alone left the coarse grid unsolved: its states
            // read as cleared (status 0), which ages the coarse history.
            auto &top = *p->levels[p->L() - 1];
            auto &tslot = *top.slots[k];
            gbdic::TemporalArgs u = t;
            if (L < p->L()) {
                check_cuda(cudaMemsetAsync(tslot.state.get(), 0, p->state_bytes(p->L() - 1), s), "coarse clear");
                if (rt.output_state(tslot) != tslot.state.as<float>())
                    check_cuda(cudaMemsetAsync(tslot.filtered.get(), 0, p->state_bytes(p->L() - 1), s),
                               "coarse clear");
            }
            u.history = p->coarse_history.as<float>();
            u.ages = p->coarse_ages.as<uint32_t>();
            u.raw = tslot.state.as<float>();
            u.output = rt.output_state(tslot);
            u.counters = nullptr;
            u.count = top.count;
            u.report_expiry = 0;
            check_cuda(gbdic::launch_temporal_merge(u, s), "coarse history merge launch");
        }
    }
    if (out_state != nullptr)
        check_cuda(cudaMemcpyAsync(out_state, rt.output_state(fslot), p->state_bytes(0), cudaMemcpyDeviceToDevice, s),
                   "state copy");
}

// The frame's sequence for slot k (its resident target in the slot's frame
// buffer) as a graph, captured on first use for the current level count.
cudaGraphExec_t slot_graph(gbdic_pyramid *p, int k) {
    auto &rt = *p->rt;
    auto &ps = p->slots[k];
    auto &fine = *p->levels[0];
    cudaStream_t s = rt.stream();
    auto body = [&](cudaStream_t st) { enqueue_pyramid(p, k, fine.slots[k]->frame.as<uint8_t>(), nullptr, st); };
    cudaGraphExec_t &exec = ps.graph[p->active_levels == p->L() ? 0 : 1];
    if (exec == nullptr) {
        cudaGraph_t graph = nullptr;
        check_cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "graph capture");
        try {
            body(s);
        } catch (...) {
            cudaStreamEndCapture(s, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        check_cuda(cudaStreamEndCapture(s, &graph), "graph capture end");
        cudaError_t err = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        check_cuda(err, "graph instantiate");
    }
    return exec;
}

// Upload (upload stream) -> the frame as a graph (the engine's stream) ->
// readback into the slot's pinned buffers (readback stream).  A slot is
// reused only after its retire waited for its readback, so its buffers are
// free when the next upload starts.
void launch_slot(gbdic_pyramid *p, int k) {
    auto &rt = *p->rt;
    auto &ps = p->slots[k];
    auto &fine = *p->levels[0];
    cudaStream_t s = rt.stream();
    const size_t bytes = p->state_bytes(0);
    ps.out.ensure(bytes);
    cudaGraphExec_t exec = slot_graph(p, k);
    check_cuda(cudaMemcpyAsync(fine.slots[k]->frame.get(), ps.in.as<uint8_t>(), (size_t)fine.W * fine.H,
                               cudaMemcpyHostToDevice, p->upload), "frame upload");
    check_cuda(cudaEventRecord(ps.uploaded, p->upload), "event");
    check_cuda(cudaStreamWaitEvent(s, ps.uploaded, 0), "upload wait");
    check_cuda(cudaEventRecord(ps.begin, s), "event");
    check_cuda(cudaGraphLaunch(exec, s), "graph launch");
    check_cuda(cudaEventRecord(ps.computed, s), "event");
    check_cuda(cudaStreamWaitEvent(p->readback, ps.computed, 0), "compute wait");
    check_cuda(cudaMemcpyAsync(ps.out.as<float>(), rt.output_state(*fine.slots[k]), bytes, cudaMemcpyDeviceToHost,
                               p->readback), "state readback");
    check_cuda(cudaMemcpyAsync(ps.counters_host.as<uint32_t>(), ps.counters.get(), 4 * sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, p->readback), "counter readback");
    check_cuda(cudaEventRecord(ps.end, p->readback), "event");
}

}  // namespace

extern "C" {

const char *gbdic_pyramid_last_error(const gbdic_pyramid *p) { return p ? p->error.c_str() : g_pyramid_error.c_str(); }

int gbdic_pyramid_create(const gbdic_pyramid_options *options, gbdic_pyramid **out) {
    if (!options || !out) {
        g_pyramid_error = "options and output handle are required";
        return GBDIC_EINVAL;
    }
    *out = nullptr;
    auto *p = new gbdic_pyramid();
    try {
        const auto &po = *options;
        if (po.levels < 1 || po.levels > 4) fail(GBDIC_EINVAL, "pyramid_levels must be an integer from 1 to 4");
        for (int i = 0; i < po.levels; ++i) {
            gbdic_solver_cfg c{po.iterations[i], po.tolerance[i], po.zncc_min};
            gbdic::validate_cfg(&c);
        }
        if (po.initialization < 0 || po.initialization > 3) fail(GBDIC_EINVAL, "unsupported initialization");
        if (po.seed_search_radius < 0 || po.seed_search_radius > 64)
            fail(GBDIC_EINVAL, "seed_search_radius must be an integer from 1 to 64");
        if (po.initialization == 2 && po.seed_search_radius < 1)
            fail(GBDIC_EINVAL, "initialization='zncc' requires seed_search_radius >= 1");
        if (po.seed_search_radius > 0 && gbdic::zncc_search_smem(po.base.subset_size, po.seed_search_radius) > 48 * 1024)
            fail(GBDIC_EINVAL, "subset_size + 2 * seed_search_radius is too large for the seed search tile");
        if (po.temporal_prediction != 0 && po.initialization != 1)
            fail(GBDIC_EINVAL, "temporal_prediction requires temporal initialization");
        if (po.temporal_fine_correction && (po.initialization != 1 || po.levels != 2))
            fail(GBDIC_EINVAL, "temporal_fine_correction requires temporal initialization and two levels");
        if (po.adaptive && (po.initialization != 1 || po.levels != 2))
            fail(GBDIC_EINVAL, "adaptive pyramid requires temporal initialization and two levels");
        gbdic::validate_options(po.base);
        p->po = po;
        p->device = po.base.device;
        p->rt = std::make_unique<gbdic::Runtime>(po.base);
        check_cuda(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking), "stream");
        check_cuda(cudaStreamCreateWithFlags(&p->upload, cudaStreamNonBlocking), "stream");
        check_cuda(cudaStreamCreateWithFlags(&p->readback, cudaStreamNonBlocking), "stream");
        check_cuda(cudaEventCreateWithFlags(&p->fork_ev, cudaEventDisableTiming), "event");
        for (int l = 0; l < 4; ++l) {
            check_cuda(cudaEventCreateWithFlags(&p->reduced_ev[l], cudaEventDisableTiming), "event");
            check_cuda(cudaEventCreateWithFlags(&p->filtered_ev[l], cudaEventDisableTiming), "event");
        }
        p->slots = std::vector<PyramidSlot>(po.base.pipeline_slots);
        for (auto &s : p->slots) s.create();
    } catch (const Failure &x) {
        g_pyramid_error = x.message;
        delete p;
        return x.code;
    }
    *out = p;
    return GBDIC_OK;
}

void gbdic_pyramid_destroy(gbdic_pyramid *p) { delete p; }

int gbdic_pyramid_set_reference(gbdic_pyramid *p, const uint8_t *image, int32_t width, int32_t height,
                                int64_t row_stride, const gbdic_level_roi *rois, const uint32_t *temporal_links,
                                gbdic_ref_info *info) {
    return pguarded(p, [&] {
        const auto &o = p->po.base;
        if (!image) fail(GBDIC_EINVAL, "image is required");
        if (width < 16 || height < 16) fail(GBDIC_EINVAL, "Image dimensions must each be at least 16 pixels.");
        if (row_stride < width) fail(GBDIC_EINVAL, "row_stride must be at least the width");
        const int L = p->po.levels;
        int W = width, H = height;
        std::vector<std::pair<int, int>> dims;
        for (int l = 0; l < L; ++l) {
            int gw, gh;
            gbdic::grid_of(W, H, o.subset_size, o.subset_stride, gw, gh);
            if (gw < 1 || gh < 1)
                fail(GBDIC_EINVAL, "Reference dimensions must each be at least " + std::to_string(o.subset_size) + " pixels.");
            dims.emplace_back(W, H);
            W /= 2;
            H /= 2;
        }
        // in-flight frames (and their copies) end before the buffers go
        for (cudaStream_t st : {p->rt->stream(), p->upload, p->readback})
            check_cuda(cudaStreamSynchronize(st), "pending work");
        p->ready = false;
        for (auto &s : p->slots) {
            s.drop_graphs();
            s.pending = false;
        }
        p->levels.clear();
        const int slots = (int)p->slots.size();
        for (int l = 0; l < L; ++l) {
            p->levels.push_back(std::make_unique<gbdic::Level>());
            p->rt->configure_level(*p->levels[l], dims[l].first, dims[l].second, slots);
            // A premature coarse stop would poison every finer seed: the
            // divergence stop applies at the finest level only (1215-1223).
            p->levels[l]->divergence = l == 0;
        }
        auto &rt = *p->rt;
        cudaStream_t s = rt.stream();
        rt.upload_frame(*p->levels[0], *p->levels[0]->slots[0], image, row_stride, p->slots[0].in, s);
        for (int l = 1; l < L; ++l)
            check_cuda(gbdic::launch_reduce_half(p->levels[l - 1]->slots[0]->frame.as<uint8_t>(), p->levels[l - 1]->W,
                                                 p->levels[l - 1]->H, p->levels[l]->slots[0]->frame.as<uint8_t>(), s),
                       "reduce launch");
        double ms = 0.0;
        for (int l = 0; l < L; ++l) {
            const gbdic_level_roi *r = rois ? &rois[l] : nullptr;
            ms += rt.prepare_reference(*p->levels[l], p->levels[l]->slots[0]->frame.as<uint8_t>(),
                                       r ? r->selected : nullptr, r ? r->links : nullptr);
        }
        p->seed_links.clear();
        p->has_seed_links.assign(L, false);
        for (int l = 0; l < L; ++l) {
            p->seed_links.push_back(std::make_unique<gbdic::DeviceBuffer>());
            if (l < L - 1 && rois && rois[l].seed_links) {
                const size_t b = (size_t)p->levels[l]->count * sizeof(uint32_t);
                p->seed_links[l]->ensure(b);
                check_cuda(cudaMemcpy(p->seed_links[l]->get(), rois[l].seed_links, b, cudaMemcpyHostToDevice), "links");
                p->has_seed_links[l] = true;
            }
        }
        p->has_temporal_links = false;
        if (temporal_links) {
            const size_t b = (size_t)p->levels[L - 1]->count * sizeof(uint32_t);
            p->temporal_links.ensure(b);
            check_cuda(cudaMemcpy(p->temporal_links.get(), temporal_links, b, cudaMemcpyHostToDevice), "links");
            p->has_temporal_links = true;
        }
        if (p->temporal()) {
            const size_t sb = p->state_bytes(0), ab = (size_t)p->levels[0]->count * sizeof(uint32_t);
            p->history.ensure(sb);
            p->ages.ensure(ab);
            if (p->velocity()) {
                p->prev_history.ensure(sb);
                p->prev_ages.ensure(ab);
                p->prediction.ensure(sb);
            }
            if (p->fine_correction()) {
                p->coarse_history.ensure(p->state_bytes(L - 1));
                p->coarse_ages.ensure((size_t)p->levels[L - 1]->count * sizeof(uint32_t));
            }
            if (p->po.adaptive) {
                // full_pyramid_backend.py:628-634: 31 for selected windows, 0 outside the ROI.
                const int n = p->levels[0]->count;
                std::vector<uint32_t> links((size_t)n, 31u);
                if (rois && rois[0].selected)
                    for (int i = 0; i < n; ++i) links[i] = rois[0].selected[i] ? 31u : 0u;
                p->fine_links.ensure((size_t)n * sizeof(uint32_t));
                check_cuda(cudaMemcpy(p->fine_links.get(), links.data(), links.size() * sizeof(uint32_t),
                                      cudaMemcpyHostToDevice), "links");
            }
            reset_temporal(p, s);
        }
        p->active_levels = L;
        check_cuda(cudaStreamSynchronize(s), "reference preparation");
        p->ready = true;
        if (info) {
            info->width = width; info->height = height;
            info->grid_width = p->levels[0]->gw; info->grid_height = p->levels[0]->gh;
            info->valid_count = p->levels[0]->valid_count;
            info->device_ms = ms;
        }
    });
}

int gbdic_pyramid_level_grid(gbdic_pyramid *p, int32_t level, int32_t *gw, int32_t *gh) {
    return pguarded(p, [&] {
        if (level < 0 || level >= p->L()) fail(GBDIC_EINVAL, "level out of range");
        if (gw) *gw = p->levels[level]->gw;
        if (gh) *gh = p->levels[level]->gh;
    });
}

int gbdic_pyramid_submit(gbdic_pyramid *p, int32_t slot, const uint8_t *frame, int64_t row_stride) {
    return pguarded(p, [&] {
        if (!p->ready) fail(GBDIC_ESTATE, "Call set_reference() before register().");
        if (slot < 0 || slot >= (int)p->slots.size()) fail(GBDIC_EINVAL, "slot index out of range");
        if (!frame) fail(GBDIC_EINVAL, "frame is required");
        auto &fine = *p->levels[0];
        if (row_stride < fine.W) fail(GBDIC_EINVAL, "row_stride must be at least the width");
        auto &ps = p->slots[slot];
        if (ps.pending) fail(GBDIC_ESTATE, "slot is still in flight; retire it first");
        ps.submitted = std::chrono::steady_clock::now();
        ps.in.ensure((size_t)fine.W * fine.H);
        uint8_t *dst = ps.in.as<uint8_t>();
        gbdic::host_copy_rows(dst, frame, (size_t)fine.W, (size_t)fine.H, row_stride);
        ps.upload_ms = gbdic::ms_since(ps.submitted);
        launch_slot(p, slot);
        ps.pending = true;
    });
}

int gbdic_pyramid_retire(gbdic_pyramid *p, int32_t slot, float *out_state, uint32_t *counters, gbdic_timing *timing) {
    return pguarded(p, [&] {
        if (slot < 0 || slot >= (int)p->slots.size()) fail(GBDIC_EINVAL, "slot index out of range");
        auto &ps = p->slots[slot];
        if (!ps.pending) fail(GBDIC_ESTATE, "slot has no registration in flight");
        ps.pending = false;
        const auto t_wait = std::chrono::steady_clock::now();
        gbdic::wait_event(ps.end, gbdic::kWaitMs);
        const double wait_ms = gbdic::ms_since(t_wait);
        const auto t_copy = std::chrono::steady_clock::now();
        if (out_state) gbdic::host_copy(out_state, ps.out.as<float>(), p->state_bytes(0));
        if (counters) std::memcpy(counters, ps.counters_host.as<uint32_t>(), 4 * sizeof(uint32_t));
        if (timing) {
            float dev = 0.0f;
            cudaEventElapsedTime(&dev, ps.begin, ps.end);
            timing->upload_ms = ps.upload_ms;
            timing->execute_ms = wait_ms;
            timing->readback_ms = gbdic::ms_since(t_copy);
            timing->total_ms = gbdic::ms_since(ps.submitted);
            timing->device_ms = dev;
        }
    });
}

int gbdic_pyramid_register(gbdic_pyramid *p, const uint8_t *frame, int64_t row_stride, float *out_state,
                           uint32_t *counters, gbdic_timing *timing) {
    int rc = gbdic_pyramid_submit(p, 0, frame, row_stride);
    if (rc != GBDIC_OK) return rc;
    return gbdic_pyramid_retire(p, 0, out_state, counters, timing);
}

int gbdic_pyramid_register_device(gbdic_pyramid *p, const uint8_t *device_frame, float *device_state, void *stream) {
    return pguarded(p, [&] {
        if (!p->ready) fail(GBDIC_ESTATE, "Call set_reference() before register().");
        if (!device_frame || !device_state) fail(GBDIC_EINVAL, "device_frame and device_state are required");
        cudaStream_t s = stream ? (cudaStream_t)stream : p->rt->stream();
        if (p->rt->profiling()) {
            // per-launch solver events: the launches are issued directly
            enqueue_pyramid(p, 0, device_frame, device_state, s);
            return;
        }
        // Slot 0's graph between two device copies (the frame in, the
        // output state out), in the order of `s`.
        auto &fine = *p->levels[0];
        auto &slot = *fine.slots[0];
        cudaGraphExec_t exec = slot_graph(p, 0);
        check_cuda(cudaMemcpyAsync(slot.frame.get(), device_frame, (size_t)fine.W * fine.H, cudaMemcpyDeviceToDevice, s),
                   "frame copy");
        check_cuda(cudaGraphLaunch(exec, s), "graph launch");
        check_cuda(cudaMemcpyAsync(device_state, p->rt->output_state(slot), p->state_bytes(0), cudaMemcpyDeviceToDevice,
                                   s), "state copy");
    });
}

int gbdic_pyramid_reset_temporal(gbdic_pyramid *p) {
    return pguarded(p, [&] {
        if (!p->ready) return;
        check_cuda(cudaStreamSynchronize(p->rt->stream()), "pending work");
        reset_temporal(p, p->rt->stream());
    });
}

int gbdic_pyramid_export(gbdic_pyramid *p, int32_t level, int32_t what, void *host_out, int64_t bytes) {
    return pguarded(p, [&] {
        if (!p->ready) fail(GBDIC_ESTATE, "Call set_reference() before export().");
        if (level < 0 || level >= p->L()) fail(GBDIC_EINVAL, "level out of range");
        if (!host_out) fail(GBDIC_EINVAL, "output is required");
        auto &lvl = *p->levels[level];
        auto &slot = *lvl.slots[0];
        const int model = p->po.base.motion_model, n = gbdic::parameter_count(model);
        const void *src = nullptr;
        size_t size = 0;
        switch (what) {
        case GBDIC_EXPORT_COEFFICIENTS: src = slot.coef.get(); size = (size_t)lvl.W * lvl.H * sizeof(float); break;
        case GBDIC_EXPORT_PLANE: src = lvl.plane.get(); size = (size_t)lvl.W * lvl.H * sizeof(float4); break;
        case GBDIC_EXPORT_METADATA: src = lvl.meta.get(); size = (size_t)lvl.count * gbdic::meta_stride(model) * sizeof(float); break;
        case GBDIC_EXPORT_INVERSE: src = lvl.inv.get(); size = (size_t)lvl.count * n * n * sizeof(float); break;
        case GBDIC_EXPORT_RAW_STATE: src = slot.state.get(); size = p->state_bytes(level); break;
        case GBDIC_EXPORT_OUTPUT_STATE: src = p->rt->output_state(slot); size = p->state_bytes(level); break;
        case GBDIC_EXPORT_WEIGHTS: src = p->rt->weights().get(); size = p->rt->opts().weights.size() * sizeof(float); break;
        case GBDIC_EXPORT_FRAME: src = slot.frame.get(); size = (size_t)lvl.W * lvl.H; break;
        case GBDIC_EXPORT_ADMISSIBLE: src = lvl.admissible.get(); size = (size_t)lvl.count; break;
        case GBDIC_EXPORT_SEED: src = slot.seed.get(); size = p->state_bytes(level); break;
        case GBDIC_EXPORT_ACTIVE: src = slot.active.get(); size = (size_t)lvl.count * sizeof(uint32_t); break;
        default: fail(GBDIC_EINVAL, "unknown export selector");
        }
        if (src == nullptr) fail(GBDIC_ESTATE, "buffer not available in this configuration");
        if ((size_t)bytes < size) fail(GBDIC_EINVAL, "output buffer too small: need " + std::to_string(size) + " bytes");
        check_cuda(cudaStreamSynchronize(p->rt->stream()), "pending work");
        check_cuda(cudaMemcpy(host_out, src, size, cudaMemcpyDeviceToHost), "export");
    });
}

}  // extern "C"

extern "C" {

int gbdic_pyramid_set_translation(gbdic_pyramid *p, int32_t slot, float dx, float dy) {
    return pguarded(p, [&] {
        if (slot < 0 || slot >= (int)p->slots.size()) fail(GBDIC_EINVAL, "slot index out of range");
        auto &ps = p->slots[slot];
        if (ps.pending) fail(GBDIC_ESTATE, "slot is still in flight; retire it first");
        ps.shift_host.as<float>()[0] = dx;
        ps.shift_host.as<float>()[1] = dy;
    });
}

int gbdic_pyramid_set_partial_support(gbdic_pyramid *p, int32_t level, int32_t count, const int32_t *indices,
                                      const uint32_t *words, int32_t words_per_window, const float *boxes,
                                      const float *metadata_rows, const float *inverse_rows) {
    return pguarded(p, [&] {
        if (!p->ready) fail(GBDIC_ESTATE, "Call set_reference() before set_partial_support().");
        if (level < 0 || level >= p->L()) fail(GBDIC_EINVAL, "level out of range");
        for (auto &s : p->slots)
            if (s.pending) fail(GBDIC_ESTATE, "retire every slot before changing the partial windows");
        p->rt->set_partial_support(*p->levels[level], count, indices, words, words_per_window, boxes, metadata_rows,
                                   inverse_rows);
        for (auto &s : p->slots) s.drop_graphs();
    });
}

int gbdic_pyramid_set_active_levels(gbdic_pyramid *p, int32_t levels) {
    return pguarded(p, [&] {
        if (!p->ready) fail(GBDIC_ESTATE, "Call set_reference() before set_active_levels().");
        if (levels != p->L() && !(levels == 1 && p->po.adaptive))
            fail(GBDIC_EINVAL, "levels must be the pyramid's level count, or 1 under the adaptive policy");
        p->active_levels = levels;
    });
}

int gbdic_pyramid_set_solver_variant(gbdic_pyramid *p, int32_t threads_per_subset, int32_t persistent) {
    return pguarded(p, [&] {
        for (auto &s : p->slots)
            if (s.pending) fail(GBDIC_ESTATE, "retire every slot before switching the solver variant");
        check_cuda(cudaStreamSynchronize(p->rt->stream()), "pending work");
        p->rt->set_variant(threads_per_subset, persistent != 0);
        for (auto &s : p->slots) s.drop_graphs();
    });
}

int gbdic_pyramid_set_solver_mode(gbdic_pyramid *p, int32_t mode) {
    return pguarded(p, [&] {
        for (auto &s : p->slots)
            if (s.pending) fail(GBDIC_ESTATE, "retire every slot before switching the solver mode");
        check_cuda(cudaStreamSynchronize(p->rt->stream()), "pending work");
        p->rt->set_mode(mode);
        for (auto &s : p->slots) s.drop_graphs();
    });
}

int gbdic_pyramid_profile(gbdic_pyramid *p, int32_t enable) {
    return pguarded(p, [&] {
        check_cuda(cudaStreamSynchronize(p->rt->stream()), "pending work");
        p->rt->set_profiling(enable != 0);
    });
}

int gbdic_pyramid_profile_read(gbdic_pyramid *p, double *solver_ms, int64_t *launches, int64_t *timed_launches,
                               uint64_t *iterations) {
    return pguarded(p, [&] {
        double ms = 0.0;
        long long n = 0, t = 0;
        unsigned long long it = 0;
        p->rt->profile_read(ms, n, t, it);
        if (solver_ms) *solver_ms = ms;
        if (launches) *launches = n;
        if (timed_launches) *timed_launches = t;
        if (iterations) *iterations = it;
    });
}

}  // extern "C"
