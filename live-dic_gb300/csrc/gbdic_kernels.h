// Internal launcher declarations and argument blocks (host + device).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gbdic_common.cuh"

namespace gbdic {

// ------------------------------------------------------------ prefilter
cudaError_t set_fir_taps(const float *taps25);
cudaError_t launch_fir_prefilter(const uint8_t *img, int W, int H, int pitch, float *coef,
                                 cudaStream_t stream);

// ------------------------------------------------------------ solver
template <int MODEL>
cudaError_t launch_icgn_model(const SolveArgs &a, int interp, int lanes, bool gauss, int grid,
                              cudaStream_t stream, int *occupancy_only);
// Grid for a non-persistent launch of `count` subsets with `lanes` lanes.
int icgn_grid(int count, int lanes);
// Resident CTAs per SM of the solver variant (for persistent grids).
int icgn_occupancy(int model, int interp, int lanes, bool gauss);
cudaError_t launch_icgn(const SolveArgs &a, int model, int interp, int lanes, bool gauss,
                        int persistent_grid, cudaStream_t stream);
// Rows 0 .. total-1 of a.state as the seeded solver writes disabled subsets
// (from a.seed, a.active, a.meta); list-mode solves start from them.
cudaError_t launch_disabled_rows(const SolveArgs &a, int model, int total, cudaStream_t stream);
// Sliding-window ("fast") pixel loop: supported configurations, the row
// segments per column that minimise its steps, its launcher (grid as for
// launch_icgn; with occupancy_only set, the resident CTAs per SM instead).
bool icgn_fast_supported(int model, int interp, int lanes);
int icgn_fast_segments(int S, int lanes);
cudaError_t launch_icgn_fast(const SolveArgs &a, int model, int lanes, bool gauss, int grid, cudaStream_t stream,
                             int *occupancy_only);
int icgn_fast_occupancy(int model, int lanes, bool gauss);
// TMA-staged coefficient tiles (solver_staged.cu): tile 1 compact (56 x 44),
// 2 wide (72 x 56); bit-identical to the exact loop.
bool icgn_staged_supported(int model, int interp, int lanes, int W);
cudaError_t launch_icgn_staged(const SolveArgs &a, int model, int lanes, bool gauss, int tile, int grid,
                               cudaStream_t stream, int *occupancy_only);
int icgn_staged_occupancy(int model, int lanes, bool gauss, int tile);

// Partial-support windows (a.count = number of partial windows; a.partial_index,
// a.support, a.support_box, a.support_words set); translation and affine.
cudaError_t launch_icgn_partial(const SolveArgs &a, int model, int interp, int lanes, bool gauss,
                                cudaStream_t stream);

// One persistent launch over many jobs (B-spline, uniform weighting).
constexpr int kMaxBatchJobs = 256;
struct BatchSolveArgs {
    const SolveArgs *args;   // per job, in queue order (device)
    const int *models;       // per job, in queue order (device); one shape-function class
    const int *first;        // jobs + 1 queue offsets, each a multiple of batch_units (device)
    unsigned *work_counter;  // queue head, zeroed before the launch
    int jobs;
};
// Subsets one scheduling unit (warp or 128-thread block) claims at a time.
int batch_units(int lanes);
// Launches of the affine/translation class or of the quadratic class.
int icgn_batch_occupancy(int lanes, bool quadratic);
cudaError_t launch_icgn_batch(const BatchSolveArgs &b, int lanes, bool quadratic, int grid, cudaStream_t stream);
// One launch over every class (the shape function dispatched per job).
int icgn_batch_any_occupancy(int lanes);
cudaError_t launch_icgn_batch_any(const BatchSolveArgs &b, int lanes, int grid, cudaStream_t stream);

// ------------------------------------------------------------ UOD
struct UodArgs {
    const float *state;
    float *out;
    const float *meta;
    const float *links;   // 4 floats per subset (ROI), or nullptr
    int grid_w, grid_h, count;
    int subset_stride;
    int model, policy, median_size, scope_all, seed_mode, roi_enabled;
};
cudaError_t launch_uod(const UodArgs &a, cudaStream_t stream);

// ------------------------------------------------------------ reference preparation
struct PrepArgs {
    const uint8_t *img;     // reference bytes, dense rows
    int W, H, pitch;
    int S, stride, grid_w, grid_h, count;
    int model, interp, gaussian_weighting;
    const float *weights;   // S*S integration weights (always provided)
    const float *axis_weights;  // S factors along one axis: weights = outer product (row path)
    float weight_sum;
    const uint8_t *selected;  // ROI selection per subset, or nullptr
    // outputs / scratch
    float *intensity;       // H*W
    float *spline;          // H*W (B-spline coefficients) and transposes
    float *scratch;         // H*W
    float4 *plane;          // H*W
    float *meta;            // count * meta_stride
    float *inv;             // count * n * n
    unsigned *valid_count;
    uint8_t *admissible;    // per subset numerical admissibility, ROI ignored
    // quadratic row path: [71][count] binary32 moments and means, or nullptr
    // (per-window path)
    float *moments;
};
cudaError_t launch_reference_prep(const PrepArgs &a, cudaStream_t stream);
// Quadratic preparation by window rows (column sums shared by the windows of
// a grid row, one thread per 12x12 inverse): uniform or Gaussian weights (the
// Gaussian as the outer product of axis_weights), overlapping windows
// (stride < S <= 256).  moments must hold quadratic_row_prep_moment_floats(count)
// floats.
bool quadratic_row_prep_supported(int model, int gaussian_weighting, int S, int stride, int grid_h);
size_t quadratic_row_prep_moment_floats(int count);
cudaError_t launch_quadratic_row_prep(const PrepArgs &a, cudaStream_t stream);

// ------------------------------------------------------------ final ZNCC
struct ZnccArgs {
    const float *coef;
    const uint8_t *img;
    const float4 *plane;
    const float *state;
    float *out;
    int W, H, grid_w, count, S, stride, interp;
};
cudaError_t launch_final_zncc(const ZnccArgs &a, cudaStream_t stream);

// ------------------------------------------------------------ pyramid
cudaError_t launch_reduce_half(const uint8_t *src, int W, int H, uint8_t *dst, cudaStream_t stream);

struct SeedArgs {
    const float *source;      // coarse (filtered) state
    float *seed;              // destination seed state
    uint32_t *active;         // destination activity
    const uint32_t *links;    // per destination permissions, or nullptr (31)
    int src_grid_w, src_grid_h, dst_grid_w, dst_count;
    float src_scale, dst_scale, subset_size, subset_stride;
    int model;
    unsigned *projected;      // counter for temporal projection, or nullptr
    int mark_missing;         // write status -1 into seeds that received no estimate
    int track;                // seed availability marker in the status slot: 0 complete stencil, -1 otherwise
    // Temporal fine correction only (source = coarse accepted history):
    const float *history;           // fine accepted history
    const uint32_t *history_ages;   // its ages
    const uint32_t *source_ages;    // coarse history ages
    unsigned max_age;
};
cudaError_t launch_transfer_seed(const SeedArgs &a, cudaStream_t stream);
// Temporal fine correction (full_pyramid.wgsl:452-506): the finest seeds
// become the fine history plus the change of the coarse field since the
// frame that history was accepted in.
cudaError_t launch_refine_temporal_seed(const SeedArgs &a, cudaStream_t stream);
// Uniform translation seeds (shift * inv_scale; device shift[2]), activity = ROI selection.
cudaError_t launch_uniform_seed(float *seed, uint32_t *active, const uint8_t *selected, int count, int model,
                                const float *shift, float inv_scale, cudaStream_t stream);

// ------------------------------------------------------------ ZNCC seed search
struct SearchArgs {
    const uint8_t *ref;       // level reference bytes (W*H)
    const uint8_t *tgt;       // level target bytes (W*H)
    float *seed;              // seed states (written)
    uint32_t *active;         // activity (written)
    float *score;             // best ZNCC per subset, or nullptr
    const uint8_t *selected;  // ROI selection, or nullptr
    unsigned *searched;       // count of searched subsets, or nullptr
    int W, H, grid_w, count, S, stride, radius, model;
    int only_missing;         // search only seeds whose status slot is -1
    int centered;             // shifts around the rounded seed translation
    const uint8_t *subset_mask;  // search only where non-zero, or nullptr
    // List mode: search only the subsets subset_list[0 .. *list_count)
    // (a device count, at most `count`), on a fixed grid.
    const int *subset_list;
    const unsigned *list_count;
};
size_t zncc_search_smem(int S, int radius);
cudaError_t launch_zncc_search(const SearchArgs &a, cudaStream_t stream);

// ------------------------------------------------------------ spatial seeds
struct FrontierArgs {
    const float *snapshot;        // states, 8 floats per subset
    const uint32_t *permissions;  // 3x3 bits, bit 4 = own
    float *seeds;                 // written for new frontier subsets
    uint32_t *active;             // set to 1 for new frontier subsets
    int count, grid_w, stride;
};
cudaError_t launch_affine_frontier(const FrontierArgs &a, cudaStream_t stream);

struct ChooseArgs {
    const uint8_t *ref, *tgt;     // reference and target bytes (W*H)
    const float *snapshot;        // states, 8 floats per subset
    const float *prior;           // prior states, or nullptr (zero hypothesis)
    const uint32_t *permissions;
    float *seeds;                 // written for improved subsets
    float *scores;                // (own rho, best rho, improved, 0) per permitted subset
    uint32_t *active;             // set to 1 for improved subsets
    int W, H, grid_w, count, S, stride, sample_step;
    float min_gain, min_displacement;
    int failed_only, candidate_mode;  // candidate_mode 0 neighbours, 1 median only, 2 both
};
cudaError_t launch_spatial_choose(const ChooseArgs &a, cudaStream_t stream);

// ------------------------------------------------------------ learned seeds
struct NnConvShape {
    int B, H, W, C;       // input NHWC
    int OH, OW, Cout;     // 3x3 stride-2 pad-1 output
    int Kp;               // padded reduction length of the forward GEMM (>= 9 C)
};

// Operand A of a convolution GEMM gathered from an NHWC tensor in the
// kernel (implicit GEMM) instead of read from a materialised matrix.
// kGatherDgradClasses is the launcher's internal form of kGatherDgrad for
// even H, W and Cout % 64 == 0: rows ordered by the input pixel's parity
// class, K blocks of the taps that are zero for a tile's class skipped.
enum { kGatherNone = 0, kGatherIm2col = 1, kGatherDgrad = 2, kGatherDgradClasses = 3 };

// D (+)= A B^T on the tensor cores: A M x K, B N x K, BF16 row-major (K
// contiguous); M % 128 == 0, N % 16 == 0, K % (64 k_split) == 0.
struct TcGemmArgs {
    const void *a, *b;        // BF16
    int M, N, K, k_split;     // split s writes its partial at d + s * split_stride
    float *d_f32;             // FP32 output or nullptr
    void *d_bf16;             // BF16 output or nullptr
    int ldd;                  // output row stride (elements, % 4 == 0)
    long long split_stride;
    const float *bias;        // per column, or nullptr
    int relu, accumulate;     // accumulate: D_f32 += result
    int *error;               // set to 1 when a pipeline wait expired
    // kGatherIm2col: A[m][k] = im2col of the input `a` (rows B*OH*OW, K = Kp);
    // kGatherDgrad: A[m][k] = the data-gradient gather of the output
    // gradient `a` (rows B*H*W, K = 9 Cout).  k_split 1.
    int gather;
    NnConvShape conv;
};
int tc_gemm_tile_n(int N);
cudaError_t launch_tc_gemm(const TcGemmArgs &a, cudaStream_t stream);

struct NnPatchArgs {
    const uint8_t *const *refs;   // device array of device image pointers
    const uint8_t *const *tgts;
    const int *image_index;       // per patch, or nullptr (image 0)
    const float *centres;         // per patch (x, y), image pixels
    int count, W, H;
    void *out;                    // [count][64][64][2] BF16
    const float *shift;           // per patch predictions displacing the target window, or nullptr
    int shift_ld;                 // row stride of `shift` (translation at columns 0 and 3)
    float shift_scale;            // prediction units -> image pixels
};
struct NnAdamArgs {
    float *param;
    const float *grad;
    float *m, *v;
    long long count;
    float lr, beta1, beta2, eps, bias1, bias2, weight_decay;
};
// Several tensors in one launch (passed by value with the launch).
constexpr int kMaxAdamTensors = 16;
struct NnAdamMany {
    float *param[kMaxAdamTensors];
    const float *grad[kMaxAdamTensors];
    float *m[kMaxAdamTensors], *v[kMaxAdamTensors];
    long long offset[kMaxAdamTensors + 1];  // element offsets of the tensors in the concatenation
    int n;
    float lr, beta1, beta2, eps, bias1, bias2, weight_decay;
};
cudaError_t launch_nn_adam_many(const NnAdamMany &a, cudaStream_t s);
cudaError_t launch_nn_patches(const NnPatchArgs &a, cudaStream_t s);
cudaError_t launch_nn_im2col(const NnConvShape &sh, const void *x, void *A, cudaStream_t s);
cudaError_t launch_nn_dgrad_gather(const NnConvShape &sh, const void *dz, void *G, cudaStream_t s);
cudaError_t launch_nn_transpose(const void *src, int R, int C, int ld_src, void *dst, int Rp, int Cp, cudaStream_t s);
// dZ = masked dY (BF16, and transposed when dzt != nullptr) and db = its
// column sums; partial: C x ceil(rows / 64) FP32 scratch.
cudaError_t launch_nn_relu_bias_backward(const float *dy, int ld, const void *y, long long rows, int C, void *dz,
                                        void *dzt, float *partial, float *db, cudaStream_t s);
// y (BF16 rows x N) = relu(sum of `splits` FP32 partials + bias).
cudaError_t launch_nn_splitk_bias_relu(const float *partial, int splits, long long rows, int N, long long split_stride,
                                      const float *bias, int relu, void *y, cudaStream_t s);
// At (Kt x M) = the im2col operand of x transposed, without writing it.
cudaError_t launch_nn_im2col_t(const NnConvShape &sh, const void *x, void *At, int Kt, cudaStream_t s);
cudaError_t launch_nn_relu_backward(const float *dy, int ld, const void *y, void *dz, long long rows, int C,
                                    cudaStream_t s);
cudaError_t launch_nn_bias_grad(const float *dy, int ld, const void *y, long long rows, int C, float *db,
                                cudaStream_t s);
cudaError_t launch_nn_splitk_reduce(const float *partial, int splits, int Kp_rows, int N, int Kp, float *out,
                                    cudaStream_t s);
cudaError_t launch_nn_adam(const NnAdamArgs &a, cudaStream_t s);
cudaError_t launch_nn_pack_weights(const float *w, int Cout, int Cin, int Kp, void *wb, void *wt, int Kt,
                                   cudaStream_t s);
cudaError_t launch_nn_regression_loss(const float *pred, int ldp, const float *target, int outputs, int B, void *grad,
                                      float *grad_f32, int ldg, float *loss, cudaStream_t s);
struct NnLatticeArgs {
    const float *pred;    // lattice_w * lattice_h rows, stride ldp, normalised outputs
    const float *base;    // first-pass outputs (translations added), or nullptr
    int ldp, lattice_w, lattice_h, step, grid_w, grid_h, stride;
    float translation_scale, gradient_scale;
    float *seeds;         // grid_w * grid_h * 8
    uint32_t *active;
};
cudaError_t launch_nn_lattice_seeds(const NnLatticeArgs &a, cudaStream_t s);

struct NnConsensusArgs {
    const float *pred;    // nodes rows, stride ldp: network residuals (translation columns 0 and 3)
    float *base;          // nodes rows, stride ldp: shift the pass ran with; receives the fitted field
    int ldp, nodes;
    const float2 *xy;     // normalised node coordinates
    const int *single;    // n_single node indices (translation hypotheses)
    int n_single;
    const int *triple;    // n_triple x 3 node indices (affine hypotheses)
    int n_triple;
    const int *probe;     // n_probe node indices that score hypotheses
    int n_probe;
    float tol[4];         // pixel tolerances, first scores, all refit
    int n_tol;
    float scale;          // pixels per normalised translation unit
};
cudaError_t launch_nn_consensus(const NnConsensusArgs &a, cudaStream_t s);
// First-layer weights passed by value (kernel parameters, read as constant
// operands): 2 input channels, 32 outputs, taps ordered (ky, kx, ci).
struct NnConv1Weights {
    float w[32][18];
    float bias[32];
};
cudaError_t launch_nn_conv_c2_direct(const NnConvShape &sh, const void *x, const NnConv1Weights &w, void *y,
                                     cudaStream_t s);
cudaError_t launch_nn_reseed_select(const float *state, int row_floats, const uint8_t *usable, int count,
                                    uint8_t *mask, uint32_t *active, unsigned *counter, int *list, cudaStream_t s);
cudaError_t launch_nn_node_rows(const float *state, int grid_w, int grid_h, int step, int lattice_w, int lattice_h,
                                float *pred, const float *base, int ldp, float translation_scale, float gradient_scale,
                                cudaStream_t s);
cudaError_t launch_nn_merge_rows(const float *src, const uint8_t *mask, int count, int row_floats, float *dst,
                                 cudaStream_t s);

struct TemporalArgs {
    float *history;           // fine accepted history
    uint32_t *ages;
    const float *raw;         // fine raw state
    const float *output;      // fine output (filtered) state
    float *prev_history;      // velocity: previous accepted history
    uint32_t *prev_ages;
    float *prediction;        // velocity: predicted field
    unsigned *counters;       // [projected, accepted updates, predicted, expired], or nullptr
    int count, model;
    unsigned max_age;
    int use_filtered;
    int report_expiry;        // count histories expiring this frame in counters[3]
};
cudaError_t launch_temporal_predict(const TemporalArgs &a, cudaStream_t stream);
cudaError_t launch_temporal_save_previous(const TemporalArgs &a, cudaStream_t stream);
cudaError_t launch_temporal_merge(const TemporalArgs &a, cudaStream_t stream);

}  // namespace gbdic
