// Batched registration of many fixed-reference jobs (declarations in
// include/gbdic.h).  Each job owns a Runtime (its reference preparation,
// coefficient plane and states); the batch owns the work-queue tables, the
// pinned staging buffers and the step graphs.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "engine.h"

using gbdic::check_cuda;
using gbdic::fail;
using gbdic::Failure;

namespace {

struct BatchJobHost {
    gbdic_batch_job desc{};
    std::unique_ptr<gbdic::Runtime> rt;
    gbdic::Level level;
    size_t in_offset = 0, out_offset = 0, state_bytes = 0;
};

// Work-queue tables of one shape-function class.
struct ClassQueue {
    std::vector<int> order;  // job indices in queue order
    gbdic::DeviceBuffer args, models, first, counter;
    int grid = 0;
};

bool is_quadratic(const BatchJobHost &j) { return j.desc.motion_model == GBDIC_MODEL_QUADRATIC; }

}  // namespace

struct gbdic_batch {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, begin = nullptr, end = nullptr, solve_begin = nullptr,
                solve_end = nullptr;
    std::string error;
    std::vector<std::unique_ptr<BatchJobHost>> jobs;
    int lanes = 16, mode = GBDIC_BATCH_SINGLE, ctas_per_sm = 0;
    ClassQueue light, heavy, all;  // per-class queues, and the single queue
    gbdic::HostBuffer in, out;
    size_t in_bytes = 0, out_bytes = 0;
    cudaGraphExec_t host_graph = nullptr, device_graph = nullptr;
    bool dirty = true;

    ~gbdic_batch() {
        cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        if (side) cudaStreamSynchronize(side);
        drop_graphs();
        for (cudaEvent_t ev : {fork, join, begin, end, solve_begin, solve_end})
            if (ev) cudaEventDestroy(ev);
        jobs.clear();
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }

    void drop_graphs() {
        if (host_graph) cudaGraphExecDestroy(host_graph);
        if (device_graph) cudaGraphExecDestroy(device_graph);
        host_graph = device_graph = nullptr;
    }

    void invalidate() {
        drop_graphs();
        dirty = true;
    }

    // Queue tables, persistent grids and staging offsets for the current
    // jobs and variant.  Runs outside any capture (occupancy queries, H2D).
    void rebuild() {
        if (!dirty) return;
        const int units = gbdic::batch_units(lanes);
        // Queue 0: light class, 1: quadratic class, 2: every job (SINGLE).
        for (int cls = 0; cls < 3; ++cls) {
            ClassQueue &q = cls == 0 ? light : cls == 1 ? heavy : all;
            q.order.clear();
            if ((cls == 2) != (mode == GBDIC_BATCH_SINGLE)) {
                q.grid = 0;
                continue;
            }
            for (int j = 0; j < (int)jobs.size(); ++j)
                if (cls == 2 || is_quadratic(*jobs[j]) == (cls == 1)) q.order.push_back(j);
            // Costliest subsets first so the cheap ones fill the tail (a
            // quadratic subset costs about 1.5 affine ones of its size).
            std::stable_sort(q.order.begin(), q.order.end(), [&](int a, int b) {
                const double ca = (is_quadratic(*jobs[a]) ? 1.5 : 1.0) * jobs[a]->desc.subset_size *
                                  jobs[a]->desc.subset_size;
                const double cb = (is_quadratic(*jobs[b]) ? 1.5 : 1.0) * jobs[b]->desc.subset_size *
                                  jobs[b]->desc.subset_size;
                return ca > cb;
            });
            if (q.order.empty()) {
                q.grid = 0;
                continue;
            }
            std::vector<gbdic::SolveArgs> args;
            std::vector<int> models, first(1, 0);
            for (int j : q.order) {
                auto &job = *jobs[j];
                gbdic::SolveArgs a = job.rt->solve_args(job.level, *job.level.slots[0], job.desc.cfg, false, false,
                                                        nullptr, nullptr);
                a.persistent = 1;
                args.push_back(a);
                models.push_back(job.desc.motion_model);
                const int padded = (job.level.count + units - 1) / units * units;
                first.push_back(first.back() + padded);
            }
            q.args.ensure(args.size() * sizeof(gbdic::SolveArgs));
            q.models.ensure(models.size() * sizeof(int));
            q.first.ensure(first.size() * sizeof(int));
            q.counter.ensure(sizeof(unsigned));
            check_cuda(cudaMemcpy(q.args.get(), args.data(), args.size() * sizeof(gbdic::SolveArgs),
                                  cudaMemcpyHostToDevice), "batch table");
            check_cuda(cudaMemcpy(q.models.get(), models.data(), models.size() * sizeof(int), cudaMemcpyHostToDevice),
                       "batch table");
            check_cuda(cudaMemcpy(q.first.get(), first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice),
                       "batch table");
            const int resident =
                cls == 2 ? gbdic::icgn_batch_any_occupancy(lanes) : gbdic::icgn_batch_occupancy(lanes, cls == 1);
            if (resident <= 0) fail(GBDIC_ECUDA, "batch solver occupancy query failed");
            const int per_sm = ctas_per_sm > 0 ? std::min(ctas_per_sm, resident) : resident;
            q.grid = per_sm * sm_count;
        }
        in_bytes = out_bytes = 0;
        for (auto &jp : jobs) {
            auto &job = *jp;
            job.in_offset = in_bytes;
            in_bytes += ((size_t)job.level.W * job.level.H + 255) / 256 * 256;
            job.out_offset = out_bytes;
            out_bytes += (job.state_bytes + 255) / 256 * 256;
            job.rt->set_variant(lanes, false);
        }
        in.ensure(in_bytes);
        out.ensure(out_bytes);
        dirty = false;
    }

    // quadratic: 0 light class, 1 quadratic class, 2 every job.
    void launch_class(ClassQueue &q, int quadratic, cudaStream_t s) {
        if (q.order.empty()) return;
        gbdic::BatchSolveArgs b{};
        b.args = q.args.as<gbdic::SolveArgs>();
        b.models = q.models.as<int>();
        b.first = q.first.as<int>();
        b.work_counter = q.counter.as<unsigned>();
        b.jobs = (int)q.order.size();
        check_cuda(cudaMemsetAsync(q.counter.get(), 0, sizeof(unsigned), s), "queue reset");
        check_cuda(quadratic == 2 ? gbdic::launch_icgn_batch_any(b, lanes, q.grid, s)
                                  : gbdic::launch_icgn_batch(b, lanes, quadratic == 1, q.grid, s),
                   "batch solver launch");
    }

    // Prefilter -> solver launches -> outlier passes on `s`; with `timed`,
    // events bracket the solver section.
    void enqueue_compute(cudaStream_t s, bool timed) {
        for (auto &jp : jobs) jp->rt->enqueue_prefilter(jp->level, *jp->level.slots[0], nullptr, s);
        if (timed) check_cuda(cudaEventRecord(solve_begin, s), "event");
        if (mode == GBDIC_BATCH_PER_JOB) {
            for (auto &jp : jobs)
                jp->rt->enqueue_solve(jp->level, *jp->level.slots[0], jp->desc.cfg, false, false, nullptr, nullptr, s);
        } else if (mode == GBDIC_BATCH_SINGLE) {
            launch_class(all, 2, s);
        } else {
            const bool both = !light.order.empty() && !heavy.order.empty();
            if (both) {
                check_cuda(cudaEventRecord(fork, s), "fork");
                check_cuda(cudaStreamWaitEvent(side, fork, 0), "fork");
                launch_class(heavy, 1, side);
                launch_class(light, 0, s);
                check_cuda(cudaEventRecord(join, side), "join");
                check_cuda(cudaStreamWaitEvent(s, join, 0), "join");
            } else {
                launch_class(heavy, 1, s);
                launch_class(light, 0, s);
            }
        }
        if (timed) check_cuda(cudaEventRecord(solve_end, s), "event");
        for (auto &jp : jobs) jp->rt->enqueue_uod(jp->level, *jp->level.slots[0], false, nullptr, s);
    }

    cudaGraphExec_t capture(bool with_copies) {
        cudaGraph_t graph = nullptr;
        check_cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "capture");
        try {
            if (with_copies)
                for (auto &jp : jobs)
                    check_cuda(cudaMemcpyAsync(jp->level.slots[0]->frame.get(), in.as<uint8_t>() + jp->in_offset,
                                               (size_t)jp->level.W * jp->level.H, cudaMemcpyHostToDevice, stream),
                               "frame upload");
            enqueue_compute(stream, false);
            if (with_copies)
                for (auto &jp : jobs)
                    check_cuda(cudaMemcpyAsync(out.as<uint8_t>() + jp->out_offset,
                                               jp->rt->output_state(*jp->level.slots[0]), jp->state_bytes,
                                               cudaMemcpyDeviceToHost, stream),
                               "state readback");
        } catch (...) {
            cudaStreamEndCapture(stream, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        check_cuda(cudaStreamEndCapture(stream, &graph), "capture");
        cudaGraphExec_t exec = nullptr;
        const cudaError_t err = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        check_cuda(err, "graph instantiate");
        return exec;
    }

    BatchJobHost &job_at(int j) {
        if (j < 0 || j >= (int)jobs.size()) fail(GBDIC_EINVAL, "job index out of range");
        return *jobs[j];
    }
};

namespace {

thread_local std::string g_batch_error;

template <typename F>
int guarded(gbdic_batch *b, F &&f) {
    if (b == nullptr) {
        g_batch_error = "null handle";
        return GBDIC_EINVAL;
    }
    try {
        check_cuda(cudaSetDevice(b->device), "cudaSetDevice");
        f();
        return GBDIC_OK;
    } catch (const Failure &x) {
        b->error = x.message;
        return x.code;
    } catch (const std::exception &x) {
        b->error = x.what();
        return GBDIC_ECUDA;
    }
}

}  // namespace

extern "C" {

const char *gbdic_batch_last_error(const gbdic_batch *b) { return b ? b->error.c_str() : g_batch_error.c_str(); }

int gbdic_batch_create(int32_t device, gbdic_batch **out) {
    if (!out) {
        g_batch_error = "output handle is required";
        return GBDIC_EINVAL;
    }
    *out = nullptr;
    auto *b = new gbdic_batch();
    try {
        int count = 0;
        check_cuda(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
        if (device < 0 || device >= count) fail(GBDIC_EINVAL, "device index out of range");
        b->device = device;
        check_cuda(cudaSetDevice(device), "cudaSetDevice");
        check_cuda(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, device), "SM count");
        check_cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream");
        check_cuda(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking), "stream");
        check_cuda(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "event");
        check_cuda(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming), "event");
        check_cuda(cudaEventCreate(&b->begin), "event");
        check_cuda(cudaEventCreate(&b->end), "event");
        check_cuda(cudaEventCreate(&b->solve_begin), "event");
        check_cuda(cudaEventCreate(&b->solve_end), "event");
    } catch (const Failure &x) {
        g_batch_error = x.message;
        delete b;
        return x.code;
    }
    *out = b;
    return GBDIC_OK;
}

int gbdic_batch_destroy(gbdic_batch *b) {
    delete b;
    return GBDIC_OK;
}

int gbdic_batch_add(gbdic_batch *b, const gbdic_batch_job *job, const uint8_t *reference, int32_t width,
                    int32_t height, int64_t row_stride, const uint8_t *roi_selected, const float *roi_links,
                    gbdic_ref_info *info, int32_t *job_index) {
    return guarded(b, [&] {
        if (!job || !reference) fail(GBDIC_EINVAL, "job and reference are required");
        if ((int)b->jobs.size() >= gbdic::kMaxBatchJobs)
            fail(GBDIC_EINVAL, "a batch holds at most " + std::to_string(gbdic::kMaxBatchJobs) + " jobs");
        if (width < 16 || height < 16) fail(GBDIC_EINVAL, "Image dimensions must each be at least 16 pixels.");
        if (row_stride < width) fail(GBDIC_EINVAL, "row_stride must be at least the width");
        if (job->outlier_policy == GBDIC_OUTLIER_MEDIAN) fail(GBDIC_EINVAL, "batch jobs support the disabled, replace and flag outlier policies");
        if (roi_selected && job->motion_model == GBDIC_MODEL_QUADRATIC)
            fail(GBDIC_EINVAL, "ROI masks currently support translation and affine motion models.");
        gbdic::validate_cfg(&job->cfg);
        gbdic_options o{};
        o.device = b->device;
        o.motion_model = job->motion_model;
        o.interpolation = GBDIC_INTERP_BSPLINE;
        o.subset_size = job->subset_size;
        o.subset_stride = job->subset_stride;
        o.spatial_weighting = 0;
        o.gaussian_sigma = 0.0f;
        o.outlier_policy = job->outlier_policy;
        o.median_filter_size = 3;
        o.median_filter_scope = 0;
        o.threads_per_subset = b->lanes;
        o.divergence_patience = 0;
        o.divergence_min_iterations = 4;
        o.pipeline_slots = 1;
        o.persistent = 0;
        gbdic::validate_options(o);
        int gw, gh;
        gbdic::grid_of(width, height, o.subset_size, o.subset_stride, gw, gh);
        if (gw < 1 || gh < 1)
            fail(GBDIC_EINVAL, "Reference dimensions must each be at least " + std::to_string(o.subset_size) + " pixels.");
        auto host = std::make_unique<BatchJobHost>();
        host->desc = *job;
        host->rt = std::make_unique<gbdic::Runtime>(o);
        host->rt->configure_level(host->level, width, height, 1);
        auto &slot = *host->level.slots[0];
        gbdic::HostBuffer staging;
        host->rt->upload_frame(host->level, slot, reference, row_stride, staging, host->rt->stream());
        const double ms = host->rt->prepare_reference(host->level, slot.frame.as<uint8_t>(), roi_selected, roi_links);
        host->state_bytes = (size_t)host->level.count * gbdic::state_stride(o.motion_model) * sizeof(float);
        if (info) {
            info->width = width; info->height = height;
            info->grid_width = gw; info->grid_height = gh;
            info->valid_count = host->level.valid_count;
            info->device_ms = ms;
        }
        check_cuda(cudaStreamSynchronize(b->stream), "pending work");
        b->jobs.push_back(std::move(host));
        b->invalidate();
        if (job_index) *job_index = (int32_t)b->jobs.size() - 1;
    });
}

int gbdic_batch_set_variant(gbdic_batch *b, int32_t lanes, int32_t mode, int32_t ctas_per_sm) {
    return guarded(b, [&] {
        if (lanes != 16 && lanes != 32 && lanes != 64 && lanes != 128)
            fail(GBDIC_EINVAL, "threads_per_subset must be 16, 32, 64, or 128");
        if (mode != GBDIC_BATCH_PERSISTENT && mode != GBDIC_BATCH_PER_JOB && mode != GBDIC_BATCH_SINGLE)
            fail(GBDIC_EINVAL, "unknown batch mode");
        if (ctas_per_sm < 0 || ctas_per_sm > 32) fail(GBDIC_EINVAL, "ctas_per_sm must be in [0, 32]");
        check_cuda(cudaStreamSynchronize(b->stream), "pending work");
        b->lanes = lanes;
        b->mode = mode;
        b->ctas_per_sm = ctas_per_sm;
        b->invalidate();
    });
}

int gbdic_batch_register(gbdic_batch *b, const uint8_t *const *frames, const int64_t *row_strides,
                         float *const *out_states, gbdic_timing *timing) {
    return guarded(b, [&] {
        if (b->jobs.empty()) fail(GBDIC_ESTATE, "Add at least one job before register().");
        if (!frames || !out_states) fail(GBDIC_EINVAL, "frames and out_states are required");
        const auto t0 = std::chrono::steady_clock::now();
        b->rebuild();
        for (size_t j = 0; j < b->jobs.size(); ++j) {
            auto &job = *b->jobs[j];
            if (!frames[j] || !out_states[j]) fail(GBDIC_EINVAL, "every job needs a frame and an output");
            const size_t W = (size_t)job.level.W, H = (size_t)job.level.H;
            const int64_t stride = row_strides ? row_strides[j] : (int64_t)W;
            if (stride < (int64_t)W) fail(GBDIC_EINVAL, "row_stride must be at least the width");
            uint8_t *dst = b->in.as<uint8_t>() + job.in_offset;
            gbdic::host_copy_rows(dst, frames[j], W, H, stride);
        }
        const double upload_ms = gbdic::ms_since(t0);
        if (!b->host_graph) b->host_graph = b->capture(true);
        const auto t1 = std::chrono::steady_clock::now();
        check_cuda(cudaEventRecord(b->begin, b->stream), "event");
        check_cuda(cudaGraphLaunch(b->host_graph, b->stream), "graph launch");
        check_cuda(cudaEventRecord(b->end, b->stream), "event");
        gbdic::wait_event(b->end, gbdic::kWaitMs);
        const double execute_ms = gbdic::ms_since(t1);
        const auto t2 = std::chrono::steady_clock::now();
        for (size_t j = 0; j < b->jobs.size(); ++j) {
            auto &job = *b->jobs[j];
            gbdic::host_copy(out_states[j], b->out.as<uint8_t>() + job.out_offset, job.state_bytes);
        }
        if (timing) {
            float dev = 0.0f;
            cudaEventElapsedTime(&dev, b->begin, b->end);
            timing->upload_ms = upload_ms;
            timing->execute_ms = execute_ms;
            timing->readback_ms = gbdic::ms_since(t2);
            timing->total_ms = gbdic::ms_since(t0);
            timing->device_ms = dev;
        }
    });
}

int gbdic_batch_load_device(gbdic_batch *b, int32_t j, const uint8_t *device_frame, int64_t row_stride, void *stream) {
    return guarded(b, [&] {
        auto &job = b->job_at(j);
        if (!device_frame) fail(GBDIC_EINVAL, "device_frame is required");
        if (row_stride < job.level.W) fail(GBDIC_EINVAL, "row_stride must be at least the width");
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->stream;
        check_cuda(cudaMemcpy2DAsync(job.level.slots[0]->frame.get(), (size_t)job.level.W, device_frame,
                                     (size_t)row_stride, (size_t)job.level.W, (size_t)job.level.H,
                                     cudaMemcpyDeviceToDevice, s),
                   "frame copy");
        if (!stream) check_cuda(cudaStreamSynchronize(s), "frame copy");
    });
}

int gbdic_batch_run_device(gbdic_batch *b, void *stream, int32_t profile, gbdic_timing *timing) {
    return guarded(b, [&] {
        if (b->jobs.empty()) fail(GBDIC_ESTATE, "Add at least one job before run_device().");
        const auto t0 = std::chrono::steady_clock::now();
        b->rebuild();
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->stream;
        if (profile) {
            // Direct launches; the side stream joins `s` through the fork event.
            b->enqueue_compute(s, true);
        } else {
            if (!b->device_graph) b->device_graph = b->capture(false);
            if (timing) check_cuda(cudaEventRecord(b->begin, s), "event");
            check_cuda(cudaGraphLaunch(b->device_graph, s), "graph launch");
            if (timing) check_cuda(cudaEventRecord(b->end, s), "event");
        }
        if (timing) {
            cudaEvent_t e0 = profile ? b->solve_begin : b->begin, e1 = profile ? b->solve_end : b->end;
            gbdic::wait_event(e1, gbdic::kWaitMs);
            float dev = 0.0f;
            cudaEventElapsedTime(&dev, e0, e1);
            timing->upload_ms = 0.0;
            timing->execute_ms = gbdic::ms_since(t0);
            timing->readback_ms = 0.0;
            timing->total_ms = timing->execute_ms;
            timing->device_ms = dev;
        }
    });
}

int gbdic_batch_export(gbdic_batch *b, int32_t j, int32_t what, void *host_out, int64_t bytes) {
    return guarded(b, [&] {
        auto &job = b->job_at(j);
        if (!host_out) fail(GBDIC_EINVAL, "output is required");
        auto &lvl = job.level;
        auto &slot = *lvl.slots[0];
        const int model = job.desc.motion_model;
        const void *src = nullptr;
        size_t size = 0;
        switch (what) {
        case GBDIC_EXPORT_COEFFICIENTS: src = slot.coef.get(); size = (size_t)lvl.W * lvl.H * sizeof(float); break;
        case GBDIC_EXPORT_METADATA: src = lvl.meta.get(); size = (size_t)lvl.count * gbdic::meta_stride(model) * sizeof(float); break;
        case GBDIC_EXPORT_RAW_STATE: src = slot.state.get(); size = job.state_bytes; break;
        case GBDIC_EXPORT_OUTPUT_STATE: src = job.rt->output_state(slot); size = job.state_bytes; break;
        case GBDIC_EXPORT_FRAME: src = slot.frame.get(); size = (size_t)lvl.W * lvl.H; break;
        case GBDIC_EXPORT_ADMISSIBLE: src = lvl.admissible.get(); size = (size_t)lvl.count; break;
        default: fail(GBDIC_EINVAL, "unknown export selector");
        }
        if (src == nullptr) fail(GBDIC_ESTATE, "buffer not available in this configuration");
        if ((size_t)bytes < size) fail(GBDIC_EINVAL, "output buffer too small: need " + std::to_string(size) + " bytes");
        check_cuda(cudaDeviceSynchronize(), "pending work");
        check_cuda(cudaMemcpy(host_out, src, size, cudaMemcpyDeviceToHost), "export");
    });
}

}  // extern "C"
