/*
 * gbdic — GB300-native IC-GN digital image correlation, C ABI.
 *
 * This is the drop-in boundary for the live-dic native registration path.
 * Every entry point takes plain pointers and sizes; no CUDA or framework type
 * appears in a signature.  Each entry cites the reference interface it
 * replaces (paths relative to DIC/LucasKanadeICGN/python/src/live_dic/).
 *
 * Return codes: GBDIC_OK, or a negative code; gbdic_last_error() returns the
 * message of the last failed call on that handle (or, for a NULL handle, of
 * the last failed create call on the calling thread).  Argument errors are
 * reported before any device work and leave the handle's state unchanged.
 *
 * Threading: a handle owns one CUDA stream and is not thread-safe; callers
 * serialise calls per handle (the Python layer holds a non-blocking lock, as
 * the reference does, wgpu_backend.py:826-853).
 *
 * Layouts (identical to the reference's GPU buffers):
 *   state       per subset 8 floats [tx, ux, uy, ty, vx, vy, status, iterations]
 *               (affine / translation) or 16 floats [tx, ux, uy, ty, vx, vy,
 *               uxx, uxy, uyy, vxx, vxy, vyy, status, iterations, 0, 0]
 *               (quadratic), row-major over the subset grid.
 *   plane       per pixel 4 floats [f, df/dx, df/dy, 0]
 *   metadata    per subset 16 (n=6) or 28 (n=12) floats [sqrt(energy), valid,
 *               J^T f (n), sum J (n), mean, sum of weights, padding]
 *   inverse     per subset n*n floats, row-major inverse Hessian
 *   roi_links   per subset 4 floats: UOD neighbour permission words
 *               (bit (dy+1)*3+dx+1 for the 3x3 stencil, or the 9x9 lattice
 *               packed in four 24-bit words for larger median filters)
 */
#ifndef GBDIC_H
#define GBDIC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBDIC_ABI_VERSION 2

enum {
    GBDIC_OK = 0,
    GBDIC_EINVAL = -1,   /* invalid argument (Python: ValueError) */
    GBDIC_ESTATE = -2,   /* call out of order, e.g. before set_reference (ICGNError) */
    GBDIC_ECUDA = -3,    /* CUDA / device error (ICGNError) */
    GBDIC_ETIMEOUT = -4  /* a bounded device wait gave up (ICGNError) */
};

enum { GBDIC_MODEL_AFFINE = 0, GBDIC_MODEL_TRANSLATION = 1, GBDIC_MODEL_QUADRATIC = 2 };
enum { GBDIC_INTERP_BSPLINE = 0, GBDIC_INTERP_LINEAR = 1, GBDIC_INTERP_KEYS = 2 };
/* IC-GN pixel loop: EXACT keeps the reference's pixel-to-lane order and
 * summation (bit-exact against the oracle); FAST walks column runs with a
 * sliding register window of B-spline taps (translation and affine models,
 * B-spline interpolation, 16 or 32 lanes; every other configuration runs the
 * exact loop), within the parity tolerances of the exact one.  STAGED and
 * STAGED_WIDE run the exact loop on B-spline taps staged per warp in a
 * shared-memory tile by TMA (56 x 44 or 72 x 56 floats), bit-identical to
 * EXACT (translation and affine, B-spline, 16 or 32 lanes, image width a
 * multiple of 4; elsewhere the exact loop). */
enum { GBDIC_SOLVER_EXACT = 0, GBDIC_SOLVER_FAST = 1, GBDIC_SOLVER_STAGED = 2, GBDIC_SOLVER_STAGED_WIDE = 3 };
enum { GBDIC_OUTLIER_FLAG = 0, GBDIC_OUTLIER_REPLACE = 1, GBDIC_OUTLIER_DISABLED = 2,
       GBDIC_OUTLIER_MEDIAN = 3 };
enum { GBDIC_EXPORT_COEFFICIENTS = 0, GBDIC_EXPORT_PLANE = 1, GBDIC_EXPORT_METADATA = 2,
       GBDIC_EXPORT_INVERSE = 3, GBDIC_EXPORT_RAW_STATE = 4, GBDIC_EXPORT_OUTPUT_STATE = 5,
       GBDIC_EXPORT_WEIGHTS = 6, GBDIC_EXPORT_FRAME = 7, GBDIC_EXPORT_ADMISSIBLE = 8,
       GBDIC_EXPORT_SEED = 9, GBDIC_EXPORT_ACTIVE = 10 };

typedef struct gbdic_engine gbdic_engine;
typedef struct gbdic_pyramid gbdic_pyramid;

/* Construction options; mirrors ICGNWGPU.__init__ (wgpu_backend.py:889-906). */
typedef struct {
    int32_t device;                    /* CUDA device ordinal */
    int32_t motion_model;              /* GBDIC_MODEL_* */
    int32_t interpolation;             /* GBDIC_INTERP_* */
    int32_t subset_size;               /* 4 .. 46340 */
    int32_t subset_stride;             /* 1 .. subset_size */
    int32_t spatial_weighting;         /* 0 uniform, 1 Gaussian */
    float gaussian_sigma;              /* pixels, > 0 */
    int32_t outlier_policy;            /* GBDIC_OUTLIER_* */
    int32_t median_filter_size;        /* 3, 5, 7, 9 */
    int32_t median_filter_scope;       /* 0 rejected only, 1 all */
    int32_t threads_per_subset;        /* 16, 32, 64, 128 (lanes per subset) */
    int32_t divergence_patience;       /* 0 disables the stagnation check */
    int32_t divergence_min_iterations; /* >= 1 */
    int32_t pipeline_slots;            /* frames that may be in flight, >= 1 */
    int32_t persistent;                /* 1: one persistent launch over a work queue */
    int32_t solver_mode;               /* GBDIC_SOLVER_* (no reference counterpart) */
} gbdic_options;

/* Per-call solver controls; mirrors _validated_config (wgpu_backend.py:504-524). */
typedef struct {
    int32_t iterations;  /* 1 .. 30 */
    float tolerance;     /* > 0, pixels of corner motion */
    float zncc_min;      /* 0 .. 1 */
} gbdic_solver_cfg;

typedef struct {
    int32_t width, height, grid_width, grid_height;
    int32_t valid_count;  /* subsets whose reference is numerically admissible */
    double device_ms;     /* CUDA-event time of the preparation kernels */
} gbdic_ref_info;

typedef struct {
    double upload_ms;     /* host wall: staging + host->device copy issue */
    double execute_ms;    /* host wall: submit to completion */
    double readback_ms;   /* host wall: device->host copy into the caller's buffer */
    double total_ms;      /* host wall of the whole call */
    double device_ms;     /* CUDA-event time of the frame's kernels */
} gbdic_timing;

/* ---------------------------------------------------------- single scale */

/* ICGNWGPU(...) construction (wgpu_backend.py:889-1179). */
int gbdic_create(const gbdic_options *options, gbdic_engine **out);
/* ICGNWGPU.close() (wgpu_backend.py:3078-3093); NULL is ignored. */
void gbdic_destroy(gbdic_engine *engine);
/* Message of the last failed call (ICGNError text). */
const char *gbdic_last_error(const gbdic_engine *engine);
/* Library ABI version (GBDIC_ABI_VERSION). */
int gbdic_abi_version(void);

/* ICGNWGPU.set_reference (wgpu_backend.py:2364-2560), GPU reference
 * preparation: Gaussian, recursive B-spline, gradients, per-subset sums,
 * Cholesky inverses.  roi_selected (grid bytes, 1 = selected) and roi_links
 * may be NULL; excluded subsets get validity -3 (wgpu_backend.py:2433-2446). */
int gbdic_set_reference(gbdic_engine *engine, const uint8_t *image, int32_t width, int32_t height,
                        int64_t row_stride, const uint8_t *roi_selected, const float *roi_links,
                        gbdic_ref_info *info);

/* set_reference() of a device-resident image (dense 8-bit rows `row_stride`
 * bytes apart): a reference rebuilt on the GPU for every pair without a host
 * copy (config "reference rebuilt every pair"); same preparation. */
int gbdic_set_reference_device(gbdic_engine *engine, const uint8_t *device_image, int32_t width, int32_t height,
                               int64_t row_stride, const uint8_t *roi_selected, const float *roi_links,
                               gbdic_ref_info *info);

/* Upload of host-prepared reference arrays in the reference's own layout
 * (_allocate_runtime, wgpu_backend.py:1569-1590), e.g. from _reference_arrays. */
int gbdic_set_reference_arrays(gbdic_engine *engine, int32_t width, int32_t height,
                               const float *plane, const float *metadata, const float *inverse,
                               const float *roi_links, gbdic_ref_info *info);

/* ICGNWGPU.register (wgpu_backend.py:2893-2944): upload, FIR prefilter,
 * IC-GN, UOD, readback of the output state (UOD output unless disabled). */
int gbdic_register(gbdic_engine *engine, const uint8_t *frame, int64_t row_stride,
                   const gbdic_solver_cfg *cfg, float *out_state, gbdic_timing *timing);

/* ICGNWGPU.register_seeded / _register_seeded_frame (wgpu_backend.py:
 * 2774-2819, 1951-2036): solve active subsets from seed states (state
 * layout); inactive subsets get status -1 (-3 when ROI-excluded). */
int gbdic_register_seeded(gbdic_engine *engine, const uint8_t *frame, int64_t row_stride,
                          const float *seed_state, const uint32_t *active,
                          const gbdic_solver_cfg *cfg, float *out_state, gbdic_timing *timing);

/* Selective pyramid recovery on the device (wgpu_backend.py:2038-2197, whose
 * per-level targets are _reduce_half of the frame, 318-334): the target held
 * in `finer`'s slot, reduced by one pyramid level (the exact integer 5x5
 * reduction, full_pyramid.wgsl:218-249) into this engine's slot 0, whose
 * reference must be width // 2 x height // 2 of the finer one's; ordered
 * after the finer engine's queued work. */
int gbdic_reduce_frame(gbdic_engine *engine, const gbdic_engine *finer, int32_t finer_slot);
/* register_seeded() of the target already in slot 0 (gbdic_reduce_frame or
 * an earlier upload): prefilter, seeded IC-GN, UOD, readback. */
int gbdic_register_seeded_resident(gbdic_engine *engine, const float *seed_state, const uint32_t *active,
                                   const gbdic_solver_cfg *cfg, float *out_state, gbdic_timing *timing);

/* ICGNWGPU._retry_seeded (wgpu_backend.py:1893-1949): re-solve active
 * subsets on the target resident in `slot` (0 after gbdic_register; a
 * retired stream slot before its next submit), keeping inactive subsets'
 * last raw state, then UOD. */
int gbdic_retry_seeded(gbdic_engine *engine, int32_t slot, const float *seed_state, const uint32_t *active,
                       const gbdic_solver_cfg *cfg, float *out_state, gbdic_timing *timing);

/* ICGNWGPU._final_affine_zncc (wgpu_backend.py:2843-2890, affine_zncc.wgsl):
 * ZNCC of the last output state on the resident target; -2 = unavailable. */
int gbdic_final_zncc(gbdic_engine *engine, float *out_zncc);

/* ICGNWGPU._submit_slot / _retire_slot (wgpu_backend.py:2946-2994): the two
 * halves of register() on one of `pipeline_slots` independent slots, so that
 * register_stream can keep several frames in flight. */
int gbdic_submit(gbdic_engine *engine, int32_t slot, const uint8_t *frame, int64_t row_stride,
                 const gbdic_solver_cfg *cfg);
int gbdic_retire(gbdic_engine *engine, int32_t slot, float *out_state, gbdic_timing *timing);

/* Resident variant of register(): `device_frame` and `device_state` are
 * device pointers (8-bit frame, dense rows; output state); `stream` is a
 * cudaStream_t or NULL for the engine's stream.  No host synchronisation. */
int gbdic_register_device(gbdic_engine *engine, const uint8_t *device_frame,
                          const gbdic_solver_cfg *cfg, float *device_state, void *stream);

/* Partial-support ROI windows (roi_policy="partial": prepare_partial_reference,
 * partial.py:26-121, and solve_partial, icgn.wgsl:1042-1085): `count` windows
 * given by grid index, support bits (words_per_window = ceil(S*S / 32) words,
 * row-major pixels, bit 0 first), support boxes (x0, y0, x1, y1 local
 * pixels) and their host-prepared metadata / inverse rows (validity -4 for
 * admitted windows), which replace the full-window rows.  Each registration
 * then solves them after the complete windows.  count = 0 clears them. */
int gbdic_set_partial_support(gbdic_engine *engine, int32_t count, const int32_t *indices, const uint32_t *words,
                              int32_t words_per_window, const float *boxes, const float *metadata_rows,
                              const float *inverse_rows);

/* Resident variant of register_seeded(): device frame, seed states (state
 * layout), activity words and output state; `stream` as for
 * gbdic_register_device.  Inactive subsets get status -1 (-3 ROI-excluded). */
int gbdic_register_seeded_device(gbdic_engine *engine, const uint8_t *device_frame, const float *device_seed,
                                 const uint32_t *device_active, const gbdic_solver_cfg *cfg, float *device_state,
                                 void *stream);
/* Second seeded solve (new here; the learned seeding's retry, nearest
 * reference component the selective retry wgpu_backend.py:1893-2036) of the
 * same device frame as the previous
 * gbdic_register_seeded_device call (its B-spline coefficients are reused,
 * not recomputed): typically only a few subsets active after a reseeding
 * search.  Calling it with another frame solves against stale coefficients. */
int gbdic_resolve_seeded_device(gbdic_engine *engine, const uint8_t *device_frame, const float *device_seed,
                                const uint32_t *device_active, const gbdic_solver_cfg *cfg, float *device_state,
                                void *stream);

/* Integer ZNCC search (new here; nearest reference component
 * spatial_seed.wgsl:65-190) of the device target against the prepared
 * reference for the subsets whose device_mask byte is non-zero (all when
 * NULL): shifts within +-radius, around the rounded seed translation when
 * `centered`; writes translation seeds and activity in place. */
int gbdic_search_seeds_device(gbdic_engine *engine, const uint8_t *device_frame, float *device_seed,
                              uint32_t *device_active, const uint8_t *device_mask, int32_t radius, int32_t centered,
                              void *stream);
/* The same search for the subsets device_list[0 .. *device_list_count)
 * (device count, e.g. from gbdic_nn_reseed_select_list), on a fixed grid
 * that strides over the list instead of one CTA per subset of the grid. */
int gbdic_search_seeds_listed_device(gbdic_engine *engine, const uint8_t *device_frame, float *device_seed,
                                     uint32_t *device_active, const int32_t *device_list,
                                     const uint32_t *device_list_count, int32_t radius, int32_t centered,
                                     void *stream);
/* Seeded solve of the listed subsets only: device_list[0 .. list_length),
 * or [0 .. min(list_length, *device_list_count)) when device_list_count is
 * not NULL (then one persistent launch over the list), with
 * threads_per_subset lanes per subset (16, 32, 64, 128; 0: the engine's).
 * Equal, bit for bit, to gbdic_register_seeded_device (prefilter != 0) or
 * gbdic_resolve_seeded_device (prefilter == 0) of an engine running the
 * same lanes, with the same seed and activity, when the list holds exactly
 * the active subsets (any order): every other row is written as those
 * calls write a disabled subset, then the listed ones are solved with the
 * exact pixel loop, then the outlier pass runs over the whole grid.
 * Complete windows only (no partial-support reference).  Few listed
 * subsets run latency-bound; more lanes per subset shorten each
 * iteration. */
int gbdic_solve_listed_device(gbdic_engine *engine, const uint8_t *device_frame, const float *device_seed,
                              const uint32_t *device_active, const int32_t *device_list, int32_t list_length,
                              const uint32_t *device_list_count, int32_t prefilter, int32_t threads_per_subset,
                              const gbdic_solver_cfg *cfg, float *device_state, void *stream);

/* Copies an internal buffer (GBDIC_EXPORT_*) to host memory. */
int gbdic_export(gbdic_engine *engine, int32_t what, void *host_out, int64_t bytes);

/* One registration (FIR prefilter + IC-GN, no outlier pass) for callers that
 * cannot allocate GPU memory: code running inside a stream capture, real-time
 * loops that forbid allocator calls, plug-ins whose host framework owns every
 * device allocation.  No counterpart in the reference.  Every pointer is a
 * device pointer supplied by the caller (reference arrays in the layout of
 * gbdic_set_reference_arrays, state as in gbdic_register); `weights` is NULL
 * for uniform integration or S*S Gaussian weights.  The coefficient scratch is
 * a fixed 8 MiB array in the library (frames up to 2,097,152 pixels, larger
 * ones return GBDIC_EINVAL), held by every GPU that loads the library until
 * exit and shared by all calls: calls that overlap on the GPU race.  The first
 * call on a device sets that device up and should come before any stream
 * capture; the device address it caches does not survive cudaDeviceReset, so
 * the entry point must not be used on a device after a reset.  Only complete
 * windows are solved: partial-support windows (metadata validity -4, prepared
 * with roi_policy "partial") come back with status -4 (roi_enabled) or -1 and
 * zero parameters, and the stagnation stop (divergence_patience) is off, so
 * results equal gbdic_register only on an engine without partial windows and
 * with divergence_patience 0.  Errors: message in gbdic_last_error(NULL). */
typedef struct {
    const uint8_t *frame;      /* width*height target bytes, dense rows */
    const float *plane;        /* width*height*4 floats */
    const float *metadata;     /* 16 (n=6) or 28 (n=12) floats per subset */
    const float *inverse;      /* n*n floats per subset */
    const float *weights;      /* S*S Gaussian weights, or NULL */
    int32_t width, height;
    int32_t motion_model, interpolation;
    int32_t subset_size, subset_stride;
    int32_t threads_per_subset;
    int32_t roi_enabled;       /* propagate validity -3 of ROI-excluded windows */
    gbdic_solver_cfg cfg;
} gbdic_noalloc_frame;
int gbdic_register_noalloc(const gbdic_noalloc_frame *frame, float *device_state, void *stream);

/* The engine's outlier pass (median_filter / median_filter_seed,
 * icgn.wgsl:1325-1605) on a caller-supplied state field, with the prepared
 * reference's validity and ROI links.  seed_mode selects the
 * median_filter_seed entry (repaired windows become status 0). */
int gbdic_apply_uod(gbdic_engine *engine, const float *state_in, int32_t seed_mode, float *state_out);

/* ICGNWGPU.affine_frontier_seeds (wgpu_backend.py:2671-2771,
 * spatial_seed.wgsl:268-309): for every permitted, not yet accepted subset,
 * the component-wise median of its accepted 3x3 neighbours' first-order
 * affine transports.  `states` holds grid*8 floats ([tx,ux,uy,ty],[vx,vy,
 * accepted 0/1, 0]); `permissions` one word per subset (bits 0-8 = 3x3
 * neighbourhood, bit 4 = the subset itself usable).  Writes grid*8 seed
 * floats (zero where no seed) and grid activity bytes. */
int gbdic_affine_frontier(gbdic_engine *engine, const float *states, const uint32_t *permissions,
                          float *out_seeds, uint8_t *out_active);

typedef struct {
    int32_t sample_step;        /* every k-th pixel of the window in x and y */
    float min_gain;             /* best ZNCC must beat the own hypothesis by this */
    float min_displacement;     /* ... and move the seed by more than this (px) */
    int32_t failed_only;        /* score only subsets whose status < 0.5 */
    int32_t candidate_mode;     /* 0 neighbours, 1 neighbour median only, 2 both */
} gbdic_choose_cfg;

/* Translation seed selection (spatial_seed.wgsl:65-190, `choose`): ZNCC of
 * up to 11 hypotheses (own, prior, 8 neighbours, neighbour median) on the
 * last registered target.  `states` / `prior` (NULL: zero hypothesis) as for
 * gbdic_affine_frontier.  Writes grid*8 seed floats for improved subsets,
 * grid*4 score floats (own rho, best rho, improved, 0) and activity bytes. */
int gbdic_spatial_choose(gbdic_engine *engine, const float *states, const float *prior,
                         const uint32_t *permissions, const gbdic_choose_cfg *cfg, float *out_seeds,
                         float *out_scores, uint8_t *out_active);

/* --------------------------------------------------------- full pyramid */

/* ICGNWGPUFullPyramid(...) (full_pyramid_backend.py:202-431). */
typedef struct {
    gbdic_options base;
    int32_t levels;                 /* 1 .. 4 */
    int32_t iterations[4];          /* per level, coarsest first */
    float tolerance[4];             /* per level, coarsest first */
    float zncc_min;
    int32_t initialization;         /* 0 zero, 1 temporal, 2 ZNCC seed search, 3 global translation */
    uint32_t temporal_max_age;      /* 0xFFFFFFFE = never expire */
    int32_t temporal_prediction;    /* 0 none, 1 velocity */
    int32_t seed_search_radius;     /* integer search radius (pixels, coarsest level) */
    int32_t temporal_fine_correction; /* 1: finest seeds = fine history + coarse change (temporal, 2 levels) */
    int32_t adaptive;               /* 1: pyramid_policy="adaptive" (temporal, 2 levels); the caller picks
                                       the levels of each frame with gbdic_pyramid_set_active_levels() */
} gbdic_pyramid_options;

/* Static per-level ROI tables produced by host-side planning (roi.py). */
typedef struct {
    const uint8_t *selected;        /* grid bytes, 1 = selected; NULL = all */
    const float *links;             /* 4 floats per subset (UOD permissions) or NULL */
    const uint32_t *seed_links;     /* finer levels: transfer permissions per subset, or NULL */
} gbdic_level_roi;

int gbdic_pyramid_create(const gbdic_pyramid_options *options, gbdic_pyramid **out);
void gbdic_pyramid_destroy(gbdic_pyramid *pyramid);
const char *gbdic_pyramid_last_error(const gbdic_pyramid *pyramid);
/* ICGNWGPUFullPyramid.set_reference (full_pyramid_backend.py:1135-1368).
 * `rois` has `levels` entries (finest first) or is NULL; temporal_links are
 * the projection permissions of the coarsest grid (NULL = 31 everywhere). */
int gbdic_pyramid_set_reference(gbdic_pyramid *pyramid, const uint8_t *image, int32_t width,
                                int32_t height, int64_t row_stride, const gbdic_level_roi *rois,
                                const uint32_t *temporal_links, gbdic_ref_info *info);
/* Grid shape of one level (0 = finest). */
int gbdic_pyramid_level_grid(gbdic_pyramid *pyramid, int32_t level, int32_t *grid_width,
                             int32_t *grid_height);
/* ICGNWGPUFullPyramid._submit_slot / _retire_slot / register
 * (full_pyramid_backend.py:1693-1832).  counters receives the temporal
 * counters [projected, accepted updates, velocity predicted, expired]. */
int gbdic_pyramid_submit(gbdic_pyramid *pyramid, int32_t slot, const uint8_t *frame,
                         int64_t row_stride);
int gbdic_pyramid_retire(gbdic_pyramid *pyramid, int32_t slot, float *out_state,
                         uint32_t *counters, gbdic_timing *timing);
int gbdic_pyramid_register(gbdic_pyramid *pyramid, const uint8_t *frame, int64_t row_stride,
                           float *out_state, uint32_t *counters, gbdic_timing *timing);
/* Resident variant: device frame in, device state out, no host sync. */
int gbdic_pyramid_register_device(gbdic_pyramid *pyramid, const uint8_t *device_frame,
                                  float *device_state, void *stream);
/* ICGNWGPUFullPyramid.reset_temporal_state (full_pyramid_backend.py:676-694). */
int gbdic_pyramid_reset_temporal(gbdic_pyramid *pyramid);
/* Copies one level's internal buffer (GBDIC_EXPORT_*). */
int gbdic_pyramid_export(gbdic_pyramid *pyramid, int32_t level, int32_t what, void *host_out,
                         int64_t bytes);

/* ------------------------------------------------------------ profiling */

/* Solver profiling (no reference counterpart; the reference reports wall-clock
 * timing dicts only): CUDA events around every IC-GN launch issued outside
 * graph capture, and a device counter of executed Gauss-Newton iterations.
 * Enabling resets the counters; read waits for the recorded launches. */
int gbdic_profile(gbdic_engine *engine, int32_t enable);
int gbdic_profile_read(gbdic_engine *engine, double *solver_ms, int64_t *launches,
                       int64_t *timed_launches, uint64_t *iterations);
int gbdic_pyramid_profile(gbdic_pyramid *pyramid, int32_t enable);
int gbdic_pyramid_profile_read(gbdic_pyramid *pyramid, double *solver_ms, int64_t *launches,
                               int64_t *timed_launches, uint64_t *iterations);
/* Measured FP32 fused multiply-add throughput of `device` (TFLOP/s), the
 * denominator of the solver's FP32 roofline. */
int gbdic_fp32_peak_probe(int32_t device, double *tflops);

/* Host summary of one packed field (`count` states of `stride` floats, the
 * status at float `n`): the number of subsets with status > 0.5 and > 1.5,
 * and the translations (floats 0 and 3) and iteration counts (float n + 1)
 * of the accepted subsets in grid order, for the FP64 means of
 * RegistrationResult (engine.py:106-327; wgpu_backend.py:2595-2668). */
int gbdic_field_summary(const float *packed, int64_t count, int32_t stride, int32_t n, float *accepted_tx,
                        float *accepted_ty, float *accepted_iterations, int64_t *accepted, int64_t *replaced);

/* Switch the IC-GN solver variant (lanes per subset 16/32/64/128, persistent
 * work queue on/off) of a prepared handle without re-preparing the reference;
 * the autotuner's actuator (reference: ICGNWGPU._autotune_solver,
 * wgpu_backend.py:2213-2296, which switches between solver pipelines). */
int gbdic_set_solver_variant(gbdic_engine *engine, int32_t threads_per_subset, int32_t persistent);
int gbdic_pyramid_set_solver_variant(gbdic_pyramid *pyramid, int32_t threads_per_subset, int32_t persistent);
/* Switch the pixel loop (GBDIC_SOLVER_*) of a prepared handle; no reference
 * counterpart (the autotuner's third axis). */
int gbdic_set_solver_mode(gbdic_engine *engine, int32_t mode);
int gbdic_pyramid_set_solver_mode(gbdic_pyramid *pyramid, int32_t mode);

/* Global translation seed (full-resolution pixels) of the next frame run on
 * `slot` (0 for gbdic_pyramid_register / register_device) when the pyramid
 * was created with initialization 3 ("fourier"): every ROI-selected coarsest
 * subset starts from (dx, dy) / 2^(levels - 1)
 * (full_pyramid_backend.py:1704-1714). */
int gbdic_pyramid_set_translation(gbdic_pyramid *pyramid, int32_t slot, float dx, float dy);

/* Levels the next submitted frames run (pyramid_policy="adaptive",
 * full_pyramid_backend.py:1448-1452,1781-1790): 1 = the finest level alone,
 * seeded from the temporal history; `levels` = the whole pyramid.  Other
 * values, or 1 without the adaptive policy, are rejected. */
int gbdic_pyramid_set_active_levels(gbdic_pyramid *pyramid, int32_t levels);

/* gbdic_set_partial_support() for one level of the pyramid (0 = finest):
 * ICGNWGPUFullPyramid.set_reference applies roi_policy="partial" at every
 * level (full_pyramid_backend.py:1222-1232). */
int gbdic_pyramid_set_partial_support(gbdic_pyramid *pyramid, int32_t level, int32_t count, const int32_t *indices,
                                      const uint32_t *words, int32_t words_per_window, const float *boxes,
                                      const float *metadata_rows, const float *inverse_rows);

/* ------------------------------------------------------------ batch */

/* Batched registration of many fixed-reference jobs of uneven image size,
 * subset size and shape function in one step (no reference counterpart: the
 * reference runs one ICGNWGPU engine per image size and registers pairs one
 * call at a time, wgpu_backend.py:2893-2944).  Each job carries its own
 * GPU-prepared reference (B-spline interpolation, uniform weighting) and is
 * solved from a zero seed exactly like gbdic_register, followed by its own
 * outlier pass.  A step is one CUDA graph: prefilter of every target, the
 * IC-GN launches of the step mode over a device work queue (by default one
 * persistent launch over every job, heavy subsets first), then the outlier
 * passes. */
typedef struct gbdic_batch gbdic_batch;

typedef struct {
    int32_t motion_model;        /* GBDIC_MODEL_* */
    int32_t subset_size;
    int32_t subset_stride;
    int32_t outlier_policy;      /* GBDIC_OUTLIER_DISABLED / REPLACE / FLAG */
    gbdic_solver_cfg cfg;
} gbdic_batch_job;

/* Step modes: PERSISTENT, one persistent launch per shape-function class
 * (affine + translation, quadratic) on two graph branches; PER_JOB, one
 * grid launch per job; SINGLE, one persistent launch over every job. */
enum { GBDIC_BATCH_PERSISTENT = 0, GBDIC_BATCH_PER_JOB = 1, GBDIC_BATCH_SINGLE = 2 };

int gbdic_batch_create(int32_t device, gbdic_batch **out);
int gbdic_batch_destroy(gbdic_batch *batch);
const char *gbdic_batch_last_error(const gbdic_batch *batch);
/* Add a job: its reference image (dense or strided rows) is prepared on the
 * GPU.  roi_selected / roi_links as for gbdic_set_reference (affine and
 * translation only).  Writes the job index. */
int gbdic_batch_add(gbdic_batch *batch, const gbdic_batch_job *job, const uint8_t *reference, int32_t width,
                    int32_t height, int64_t row_stride, const uint8_t *roi_selected, const float *roi_links,
                    gbdic_ref_info *info, int32_t *job_index);
/* Lanes per subset (16, 32, 64, 128; default 16), step mode (default
 * GBDIC_BATCH_SINGLE), and persistent CTAs per SM (0 = as many as are
 * resident). */
int gbdic_batch_set_variant(gbdic_batch *batch, int32_t threads_per_subset, int32_t mode, int32_t ctas_per_sm);
/* One step from host frames: frames[j] is job j's target (rows of its own
 * width, row_strides[j] bytes apart); out_states[j] receives its output
 * state grid (grid_h * grid_w * 8 or 16 floats). */
int gbdic_batch_register(gbdic_batch *batch, const uint8_t *const *frames, const int64_t *row_strides,
                         float *const *out_states, gbdic_timing *timing);
/* Resident path: copy a device frame into job j's target buffer ... */
int gbdic_batch_load_device(gbdic_batch *batch, int32_t job, const uint8_t *device_frame, int64_t row_stride,
                            void *stream);
/* ... then run one step on `stream` (NULL: the batch's stream) from the
 * loaded targets; outputs stay on the device (gbdic_batch_export).  With
 * `profile` set the stages are launched directly rather than as the graph,
 * and timing->device_ms is the solver launches' time alone. */
int gbdic_batch_run_device(gbdic_batch *batch, void *stream, int32_t profile, gbdic_timing *timing);
/* Copy job j's GBDIC_EXPORT_* array to host memory (OUTPUT_STATE, RAW_STATE,
 * METADATA, ADMISSIBLE). */
int gbdic_batch_export(gbdic_batch *batch, int32_t job, int32_t what, void *host_out, int64_t bytes);

/* ------------------------------------------------ Fourier initializer */

/* FourierInitializer (fourier.py:16-111) on the GPU: linear phase
 * correlation of a size x size window (a power of two, 32..1024) between the
 * reference and each target, float64 radix-2 transforms.  Create with the
 * reference window bytes (dense) and its ROI window (or NULL); estimate reads
 * the same window at (x, y) of a target (host, or device when device_frame)
 * and writes out[7] = {dx, dy, peak score, overlap, correlation, peak,
 * target window std}; the caller applies the reference's acceptance rule
 * (score >= 8, overlap >= 0.25, correlation >= 0.2, std >= 1).  Errors:
 * gbdic_fourier_last_error(handle or NULL). */
typedef struct gbdic_fourier gbdic_fourier;
int gbdic_fourier_create(int32_t device, const uint8_t *window, const uint8_t *allowed, int32_t size,
                         gbdic_fourier **out);
int gbdic_fourier_destroy(gbdic_fourier *fourier);
const char *gbdic_fourier_last_error(const gbdic_fourier *fourier);
int gbdic_fourier_estimate(gbdic_fourier *fourier, const uint8_t *frame, int64_t row_stride, int32_t height,
                           int32_t x, int32_t y, int32_t device_frame, double *out);
/* Stream-ordered phase correlation (new here; the computation of
 * FourierInitializer.estimate, fourier.py:59-111) of a device frame's window
 * (no host synchronisation) that writes the accepted integer shift into rows of affine
 * parameters: rows[i * pitch] = dx * multiplier, rows[i * pitch + 3] =
 * dy * multiplier for i < count.  Accepted when the window's standard
 * deviation is >= 1, the peak score >= 8 and the overlap >= 0.25, else zero
 * (the sample-correlation test of gbdic_fourier_estimate is not applied).
 * Calls on one handle run in stream order and must not overlap.  Outside a
 * stream capture the call is also ordered with the handle's own stream
 * (gbdic_fourier_estimate); inside one (a CUDA graph of the caller's frame)
 * it is not, so the graph's replays and host-path estimates must not use the
 * same handle at the same time. */
int gbdic_fourier_shift_device(gbdic_fourier *fourier, const uint8_t *frame, int64_t row_stride, int32_t height,
                               int32_t x, int32_t y, float multiplier, float *rows, int32_t count, int32_t pitch,
                               void *stream);

/* ------------------------------------------------- learned seed network */

/* Building blocks of the learned seed-proposal network (no counterpart in the
 * reference, whose large-motion initialisers are the pyramid, the Fourier
 * phase correlation and wgpu-matching).  All pointers are device pointers;
 * `stream` is a cudaStream_t or NULL.  Errors: message in
 * gbdic_last_error(NULL).
 *
 * BF16 tensor-core GEMM (tcgen05, FP32 accumulation in tensor memory):
 *   D[m][n] (+)= sum_k A[m][k] B[n][k] (+ bias[n]) (ReLU)
 * A: M x K, B: N x K, both BF16 row-major with K contiguous; M % 128 == 0,
 * N % 16 == 0, K % (64 * k_split) == 0.  Split s writes its partial at
 * D + s * split_stride (bias must be NULL when k_split > 1).  A pipeline wait
 * that expires sets *device_error to 1 (device_error may be NULL). */
typedef struct {
    const void *a, *b;
    int32_t M, N, K, k_split;
    float *d_f32;          /* FP32 output, or NULL */
    void *d_bf16;          /* BF16 output, or NULL */
    int32_t ldd;           /* output row stride in elements, multiple of 4 */
    int64_t split_stride;
    const float *bias;
    int32_t relu, accumulate;
} gbdic_nn_gemm_desc;
int gbdic_nn_gemm(const gbdic_nn_gemm_desc *desc, int32_t *device_error, void *stream);


/* 64x64 reference/target patch pairs around `centres` ((x, y) per patch,
 * image pixels) of uint8 images W x H: refs / tgts are device arrays of
 * device image pointers, image_index (or NULL) selects the image of each
 * patch.  With `shift` (or NULL) the target window is displaced by
 * (shift[b][0], shift[b][3]) * shift_scale pixels (a previous prediction,
 * rows of shift_ld floats).  Output [count][64][64][2] BF16, each channel at
 * zero mean and unit variance; coordinates outside the image are clamped. */
int gbdic_nn_patches(const uint8_t *const *refs, const uint8_t *const *tgts, const int32_t *image_index,
                     const float *centres, int32_t count, int32_t width, int32_t height, void *out,
                     const float *shift, int32_t shift_ld, float shift_scale, void *stream);

/* 3x3, stride-2, pad-1 convolution shapes (NHWC BF16 activations). */
typedef struct {
    int32_t B, H, W, C, OH, OW, Cout, Kp;
} gbdic_nn_conv_shape;

/* The same GEMM with operand A gathered in the kernel from an NHWC BF16
 * tensor (implicit GEMM; desc->a is that tensor, not a matrix):
 * mode 1, A[m][k] = the im2col row of the input, as gbdic_nn_im2col writes
 * it (M = B*OH*OW, K = Kp, C % 8 == 0); mode 2, A[m][k] = the data-gradient
 * gather of the output gradient, as gbdic_nn_dgrad_gather writes it
 * (M = B*H*W, K = 9*Cout, Cout % 8 == 0).  k_split may exceed 1 in mode 1
 * only (partials as for gbdic_nn_gemm).  Results are those of
 * gbdic_nn_gemm on the materialised matrix, which is never written. */
int gbdic_nn_conv_gemm(const gbdic_nn_gemm_desc *desc, int32_t mode, const gbdic_nn_conv_shape *shape,
                       int32_t *device_error, void *stream);
/* Forward GEMM operand A[(b, oy, ox)][(ky, kx, ci)] (zero beyond 9 C). */
int gbdic_nn_im2col(const gbdic_nn_conv_shape *shape, const void *x, void *a, void *stream);
/* Inference form of the 2-channel input layer (Cout 32): the 3x3 stride-2
 * convolution, bias and ReLU in one pass, y[(b, oy, ox)][co] BF16 (row of 32),
 * without the im2col operand.  `weights` (32 x 18 floats, taps (ky, kx, ci))
 * and `bias` (32 floats) are HOST arrays, passed by value with the launch. */
int gbdic_nn_conv_c2_direct(const gbdic_nn_conv_shape *shape, const void *x, const float *weights, const float *bias,
                            void *y, void *stream);
/* Data-gradient operand G[(b, iy, ix)][(ky, kx, co)] from output gradients. */
int gbdic_nn_dgrad_gather(const gbdic_nn_conv_shape *shape, const void *dz, void *g, void *stream);
/* dst (Cp x Rp) = src (R x C, row stride ld_src) transposed, zero padded. */
int gbdic_nn_transpose(const void *src, int32_t rows, int32_t cols, int32_t ld_src, void *dst, int32_t rows_padded,
                       int32_t cols_padded, void *stream);
/* dZ (BF16, rows x C) = dY (FP32, row stride ld) where Y > 0, else 0. */
int gbdic_nn_relu_backward(const float *dy, int32_t ld, const void *y, void *dz, int64_t rows, int32_t cols,
                           void *stream);
/* db[c] = sum_r dY[r][c] (masked by Y > 0 when y != NULL). */
int gbdic_nn_bias_grad(const float *dy, int32_t ld, const void *y, int64_t rows, int32_t cols, float *db,
                       void *stream);
/* ReLU backward, bias gradient and transposed output gradient in one pass:
 * dz (BF16, rows x cols) = dY (FP32, row stride ld) where Y > 0 (everywhere
 * when y == NULL); dz_t (BF16, cols x rows, or NULL) its transpose; db[c] =
 * sum_r dz[r][c] before rounding, in a fixed order.  partial: device scratch
 * of cols * ceil(rows / 64) floats.  cols a power of two from 4 to 256,
 * ld % 4 == 0, rows % 8 == 0 when dz_t != NULL. */
int gbdic_nn_relu_bias_backward(const float *dy, int32_t ld, const void *y, int64_t rows, int32_t cols, void *dz,
                                void *dz_t, float *partial, float *db, void *stream);
/* y (BF16, rows x cols) = relu?(sum_s partial[s] + bias) over `splits` FP32
 * partials rows x cols, split_stride floats apart (summed in split order):
 * the epilogue of a split-K gbdic_nn_gemm / gbdic_nn_conv_gemm. */
int gbdic_nn_splitk_bias_relu(const float *partial, int32_t splits, int64_t rows, int32_t cols, int64_t split_stride,
                              const float *bias, int32_t relu, void *y, void *stream);
/* a_t (rows_padded x B*OH*OW) = the im2col operand of x (gbdic_nn_im2col)
 * transposed, without writing the operand itself (the weight-gradient GEMM's
 * A); rows_padded % 64 == 0, B*OH*OW % 8 == 0.  Rows 9 C up to the next
 * multiple of 64 are written as zero; the rows beyond are not written (the
 * caller keeps them zero). */
int gbdic_nn_im2col_t(const gbdic_nn_conv_shape *shape, const void *x, void *a_t, int32_t rows_padded, void *stream);
/* out[n][k] = sum_s partial[s][k][n] for k < Kp (partials Kp_rows x N). */
int gbdic_nn_splitk_reduce(const float *partial, int32_t splits, int32_t kp_rows, int32_t n, int32_t kp, float *out,
                           void *stream);
/* Adam step on `count` FP32 parameters; hyper = {lr, beta1, beta2, eps,
 * 1 - beta1^t, 1 - beta2^t, weight_decay}. */
int gbdic_nn_adam(float *param, const float *grad, float *m, float *v, int64_t count, const float *hyper,
                  void *stream);
/* The same step over 1 to 16 tensors in one launch (host arrays of device
 * pointers and element counts); per element the arithmetic of
 * gbdic_nn_adam. */
int gbdic_nn_adam_many(float *const *params, const float *const *grads, float *const *m, float *const *v,
                       const int64_t *counts, int32_t tensors, const float *hyper, void *stream);
/* BF16 copy of W [Cout][Kp] and, when wt != NULL, the data-gradient operand
 * Wt[ci][(ky, kx, co)] (row length kt). */
int gbdic_nn_pack_weights(const float *w, int32_t cout, int32_t cin, int32_t kp, void *wb, void *wt, int32_t kt,
                          void *stream);
/* Mean squared-error loss over the first `outputs` columns and its gradient
 * (BF16 [B][ldg] and, when grad_f32 != NULL, FP32 [B][ldg]; zero beyond
 * `outputs`). */
int gbdic_nn_regression_loss(const float *pred, int32_t ldp, const float *target, int32_t outputs, int32_t batch,
                             void *grad, float *grad_f32, int32_t ldg, float *loss, void *stream);
/* Half-resolution pyramid level of a device uint8 image (exact integer
 * [1 4 6 4 1]^2 / 256 with reflection, full_pyramid.wgsl:218-249). */
int gbdic_reduce_half(const uint8_t *src, int32_t width, int32_t height, uint8_t *dst, void *stream);
/* Seeds of every subset of a grid_w x grid_h grid from network outputs on a
 * lattice of every `step`-th subset in x and y (lattice_w x lattice_h rows of
 * `pred`, row stride ldp, normalised [tx/ts, ux*gs, uy*gs, ty/ts, vx*gs,
 * vy*gs]; translations plus those of `base`, a first pass, when non-NULL):
 * bilinear blend of the four surrounding lattice warps, each Taylor-recentred
 * to the subset centre.  Writes affine seed states (8 floats) and activity 1. */
int gbdic_nn_lattice_seeds(const float *pred, const float *base, int32_t ldp, int32_t lattice_w, int32_t lattice_h,
                           int32_t step, int32_t grid_w, int32_t grid_h, int32_t subset_stride, float translation_scale,
                           float gradient_scale, float *seeds, uint32_t *active, void *stream);
/* Robust affine field through lattice translations, in one launch: totals
 * (base + pred) * translation_scale (columns 0 and 3 of rows of ldp floats);
 * hypotheses = single-node translations (`singles`) then affine maps through
 * node triples (`triples`, n_triple x 3), scored by the `probes` (at most
 * 256) within tolerances[0] px, as FP32 squared distances (node_xy:
 * normalised node coordinates, nodes x 2 floats);
 * the most supported hypothesis (lowest index on ties) is refitted by least
 * squares on its inliers for each tolerance in turn (n_tol <= 4), stopping
 * below three inliers.  base columns 0 and 3 receive fitted / scale.  Indices
 * outside [0, nodes) are ignored; non-finite totals are outliers. */
int gbdic_nn_consensus(const float *pred, float *base, int32_t ldp, int32_t nodes, const float *node_xy,
                       const int32_t *singles, int32_t n_single, const int32_t *triples, int32_t n_triple,
                       const int32_t *probes, int32_t n_probe, const float *tolerances, int32_t n_tol,
                       float translation_scale, void *stream);
/* Subsets to reseed from an affine state field (rows of row_floats floats,
 * status at column 6): status 0 (not converged) or -2 (below the ZNCC
 * threshold), where usable[i] != 0 (usable may be NULL).  mask / active = 1
 * for those, 0 else; *counter (device, may be NULL) = their number. */
int gbdic_nn_reseed_select(const float *state, int32_t row_floats, const uint8_t *usable, int32_t count,
                           uint8_t *mask, uint32_t *active, uint32_t *counter, void *stream);
/* The same selection, also appending the selected subset indices to `list`
 * (device, `count` entries of room; order arbitrary; *counter = their
 * number), for gbdic_search_seeds_listed_device / gbdic_solve_listed_device. */
int gbdic_nn_reseed_select_list(const float *state, int32_t row_floats, const uint8_t *usable, int32_t count,
                                uint8_t *mask, uint32_t *active, uint32_t *counter, int32_t *list, void *stream);
/* Lattice rows of `pred` (layout of gbdic_nn_lattice_seeds) from solved
 * node subsets: node (lx, ly) is grid subset (lx * step, ly * step) of the
 * affine state field `state` (8 floats per subset); where that subset
 * converged (status >= 1, finite parameters) its row becomes the solved warp,
 * translations relative to `base` (or NULL); other rows are left unchanged. */
int gbdic_nn_node_rows(const float *state, int32_t grid_w, int32_t grid_h, int32_t step, int32_t lattice_w,
                       int32_t lattice_h, float *pred, const float *base, int32_t ldp, float translation_scale,
                       float gradient_scale, void *stream);
/* dst row i = src row i where mask[i] != 0 (rows of row_floats floats). */
int gbdic_nn_merge_rows(const float *src, const uint8_t *mask, int32_t count, int32_t row_floats, float *dst,
                        void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GBDIC_H */
