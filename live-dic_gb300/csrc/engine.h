// Host runtime of the gbdic library: device buffers, levels, slots.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gbdic.h"
#include "gbdic_kernels.h"

namespace gbdic {

// Failure carrying a gbdic return code and a message.
struct Failure {
    int code;
    std::string message;
};

void check_cuda(cudaError_t err, const char *what);
[[noreturn]] void fail(int code, const std::string &message);
double ms_since(std::chrono::steady_clock::time_point t0);
// Bounded host wait on an event (GBDIC_ETIMEOUT after `timeout_ms`).
void wait_event(cudaEvent_t ev, double timeout_ms);
void validate_options(const gbdic_options &o);
void validate_cfg(const gbdic_solver_cfg *c);
void grid_of(int W, int H, int S, int st, int &gw, int &gh);
// The 25 float32 runtime taps of the target FIR (offsets -12..12).
void fir_taps(float out[25]);
// Message returned by gbdic_last_error(NULL) on the calling thread.
void set_thread_error(const std::string &message);
// Host copies of frames and fields into / out of pinned staging, split over
// a small pool of worker threads when large (one core's memcpy bandwidth is
// a frame's largest host cost at UHD).  Rows: `height` rows of `width`
// bytes, source rows `stride` bytes apart.
void host_copy(void *dst, const void *src, size_t bytes);
void host_copy_rows(uint8_t *dst, const uint8_t *src, size_t width, size_t height, int64_t stride);
constexpr double kWaitMs = 120000.0;

// Owning device allocation.
class DeviceBuffer {
  public:
    DeviceBuffer() = default;
    ~DeviceBuffer() { reset(); }
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    void ensure(size_t bytes);  // (re)allocates when the size grows
    void reset();
    template <typename T> T *as() const { return static_cast<T *>(ptr_); }
    size_t bytes() const { return bytes_; }
    void *get() const { return ptr_; }

  private:
    void *ptr_ = nullptr;
    size_t bytes_ = 0;
};

// Owning pinned host allocation.
class HostBuffer {
  public:
    HostBuffer() = default;
    ~HostBuffer() { reset(); }
    HostBuffer(const HostBuffer &) = delete;
    HostBuffer &operator=(const HostBuffer &) = delete;
    void ensure(size_t bytes);
    void reset();
    template <typename T> T *as() const { return static_cast<T *>(ptr_); }

  private:
    void *ptr_ = nullptr;
    size_t bytes_ = 0;
};

// Per-frame mutable buffers of one level.
struct LevelSlot {
    DeviceBuffer frame;     // W*H bytes
    DeviceBuffer coef;      // W*H floats
    DeviceBuffer state;     // raw solver state
    DeviceBuffer filtered;  // UOD output
    DeviceBuffer seed;      // seed states
    DeviceBuffer active;    // seed activity
    DeviceBuffer counter;   // persistent work-queue head
};

// One image scale: reference data plus its per-slot buffers.
struct Level {
    int W = 0, H = 0, gw = 0, gh = 0, count = 0;
    bool roi = false;
    DeviceBuffer plane, meta, inv, links, selected;
    DeviceBuffer intensity, spline, scratch, valid;  // preparation scratch
    DeviceBuffer admissible;                         // u8 per subset, ROI ignored
    DeviceBuffer moments;                            // quadratic row path: moments per subset
    DeviceBuffer ref_image;                          // reference bytes (seed search)
    DeviceBuffer partial_index, partial_words, partial_boxes;  // partial-support windows
    int partial_count = 0, support_words = 0;
    bool divergence = true;  // apply the divergence stop here (pyramids: finest level only)
    std::vector<std::unique_ptr<LevelSlot>> slots;
    int valid_count = 0;
};

struct Options {
    gbdic_options o;
    int lanes = 32;
    std::vector<float> weights;  // S*S integration weights
    float weight_sum = 0.0f;
};

// Shared machinery of both engine kinds.
class Runtime {
  public:
    explicit Runtime(const gbdic_options &options);
    ~Runtime();
    const Options &opts() const { return opt_; }
    cudaStream_t stream() const { return stream_; }
    int sm_count() const { return sm_count_; }

    void configure_level(Level &level, int W, int H, int slots);
    void ensure_slots(Level &level, int slots);
    // GPU reference preparation from a device image (dense rows).
    double prepare_reference(Level &level, const uint8_t *device_image, const uint8_t *roi_selected,
                             const float *roi_links);
    void upload_reference_arrays(Level &level, const float *plane, const float *meta,
                                 const float *inverse, const float *links);
    // Partial-support windows: replaces the metadata / inverse rows of
    // `count` windows by host-prepared ones and stores their support tables;
    // every later solve of the level runs the partial solver after the
    // complete windows.  count = 0 clears them.
    void set_partial_support(Level &level, int count, const int32_t *indices, const uint32_t *words,
                             int words_per_window, const float *boxes, const float *metadata_rows,
                             const float *inverse_rows);
    // Per-frame stages of one level on `stream`.
    // `frame` (device bytes) and `state` / `out` override the slot's own
    // buffers when non-null.
    void enqueue_prefilter(Level &level, LevelSlot &slot, const uint8_t *frame, cudaStream_t stream);
    void enqueue_solve(Level &level, LevelSlot &slot, const gbdic_solver_cfg &cfg, bool seeded,
                       bool preserve, const uint8_t *frame, float *state, cudaStream_t stream);
    // The solver arguments enqueue_solve launches with (work_counter = the
    // slot's queue head; the persistent flag of the current variant).
    SolveArgs solve_args(Level &level, LevelSlot &slot, const gbdic_solver_cfg &cfg, bool seeded,
                         bool preserve, const uint8_t *frame, float *state) const;
    // Seeded solve of the listed subsets only (list[0 .. length), or
    // list[0 .. min(length, *list_count)) when list_count is set): every row
    // first as a disabled subset, then the exact loop over the list.  Equal
    // to enqueue_solve(seeded) when the list holds exactly the active
    // subsets and the same lanes per subset (`lanes`, 0: the engine's);
    // complete windows only.
    void enqueue_solve_list(Level &level, LevelSlot &slot, const gbdic_solver_cfg &cfg, const int *list,
                            int length, const unsigned *list_count, int lanes, const uint8_t *frame, float *state,
                            cudaStream_t stream);
    void enqueue_uod(Level &level, LevelSlot &slot, bool seed_mode, float *out, cudaStream_t stream);
    const float *output_state(LevelSlot &slot) const;
    void upload_frame(Level &level, LevelSlot &slot, const uint8_t *frame, int64_t row_stride,
                      HostBuffer &staging, cudaStream_t stream);
    int persistent_grid(int lanes);
    // Switch the solver variant (lanes per subset, persistent queue).
    void set_variant(int lanes, bool persistent);
    // Switch the pixel loop (GBDIC_SOLVER_*).
    void set_mode(int mode);
    // The fast loop runs for this configuration.
    bool fast_active() const;
    const DeviceBuffer &weights() const { return weights_; }
    const DeviceBuffer &axis_weights() const { return axis_weights_; }
    // Solver profiling: CUDA events around every solver launch (outside graph
    // capture) and a device counter of executed Gauss-Newton iterations.
    void set_profiling(bool enable);
    void profile_reset();
    void profile_read(double &solver_ms, long long &launches, long long &timed, unsigned long long &iterations);
    bool profiling() const { return profiling_; }

  private:
    Options opt_;
    cudaStream_t stream_ = nullptr;
    DeviceBuffer weights_;
    DeviceBuffer axis_weights_;  // S factors; weights_ is their outer product (Gaussian) or ones
    int sm_count_ = 0;
    int device_ = 0;
    int persistent_grid_ = 0;
    int persistent_lanes_ = 0;
    int persistent_variant_ = 0;  // 0 exact, 1 fast, 2 / 3 staged tile 1 / 2
    bool profiling_ = false;
    std::vector<cudaEvent_t> profile_begin_, profile_end_;
    int profile_used_ = 0;
    long long profile_launches_ = 0;
    DeviceBuffer profile_iterations_;
};

}  // namespace gbdic
