// C ABI of the learned seed network's kernels (declarations in
// include/gbdic.h).  Thin argument checks, then the launchers of tc_gemm.cu
// and nn_ops.cu; errors go to gbdic_last_error(NULL).
#include <string>

#include "engine.h"

namespace {

int rc(cudaError_t err, const char *what) {
    if (err == cudaSuccess) return GBDIC_OK;
    gbdic::set_thread_error(std::string(what) + ": " + cudaGetErrorString(err));
    return err == cudaErrorInvalidValue ? GBDIC_EINVAL : GBDIC_ECUDA;
}

int invalid(const char *message) {
    gbdic::set_thread_error(message);
    return GBDIC_EINVAL;
}

cudaStream_t as_stream(void *s) { return static_cast<cudaStream_t>(s); }

bool valid_shape(const gbdic_nn_conv_shape *s) {
    return s && s->B > 0 && s->H > 0 && s->W > 0 && s->C > 0 && s->Cout > 0 && s->OH == (s->H + 1) / 2 &&
           s->OW == (s->W + 1) / 2 && s->Kp >= 9 * s->C;
}

gbdic::NnConvShape shape_of(const gbdic_nn_conv_shape *s) {
    return {s->B, s->H, s->W, s->C, s->OH, s->OW, s->Cout, s->Kp};
}

}  // namespace

extern "C" {

int gbdic_nn_gemm(const gbdic_nn_gemm_desc *d, int32_t *device_error, void *stream) {
    if (!d) return invalid("gemm descriptor is required");
    gbdic::TcGemmArgs a{};
    a.a = d->a; a.b = d->b;
    a.M = d->M; a.N = d->N; a.K = d->K; a.k_split = d->k_split;
    a.d_f32 = d->d_f32; a.d_bf16 = d->d_bf16; a.ldd = d->ldd; a.split_stride = d->split_stride;
    a.bias = d->bias; a.relu = d->relu; a.accumulate = d->accumulate;
    a.error = device_error;
    return rc(gbdic::launch_tc_gemm(a, as_stream(stream)),
              "tensor-core GEMM (M % 128, N % 16, K % (64 k_split), 16-byte aligned operands, ldd % 4)");
}

int gbdic_nn_conv_gemm(const gbdic_nn_gemm_desc *d, int32_t mode, const gbdic_nn_conv_shape *s,
                       int32_t *device_error, void *stream) {
    if (!d || !valid_shape(s)) return invalid("gemm descriptor and convolution shape are required");
    if (mode != gbdic::kGatherIm2col && mode != gbdic::kGatherDgrad) return invalid("unknown gather mode");
    gbdic::TcGemmArgs a{};
    a.a = d->a; a.b = d->b;
    a.M = d->M; a.N = d->N; a.K = d->K; a.k_split = d->k_split;
    a.d_f32 = d->d_f32; a.d_bf16 = d->d_bf16; a.ldd = d->ldd; a.split_stride = d->split_stride;
    a.bias = d->bias; a.relu = d->relu; a.accumulate = d->accumulate;
    a.error = device_error;
    a.gather = mode;
    a.conv = shape_of(s);
    return rc(gbdic::launch_tc_gemm(a, as_stream(stream)),
              "implicit convolution GEMM (rows and K of the convolution, C or Cout % 8, k_split 1 for mode 2)");
}

int gbdic_nn_patches(const uint8_t *const *refs, const uint8_t *const *tgts, const int32_t *image_index,
                     const float *centres, int32_t count, int32_t width, int32_t height, void *out,
                     const float *shift, int32_t shift_ld, float shift_scale, void *stream) {
    if (!refs || !tgts || !centres || !out || count < 0 || width < 1 || height < 1 || (shift && shift_ld < 4))
        return invalid("patch arguments are incomplete");
    gbdic::NnPatchArgs a{refs, tgts, image_index, centres, count, width, height, out, shift, shift_ld, shift_scale};
    return rc(gbdic::launch_nn_patches(a, as_stream(stream)), "patch extraction");
}

int gbdic_nn_im2col(const gbdic_nn_conv_shape *s, const void *x, void *a, void *stream) {
    if (!valid_shape(s) || !x || !a) return invalid("invalid convolution shape or pointers");
    return rc(gbdic::launch_nn_im2col(shape_of(s), x, a, as_stream(stream)), "im2col");
}

int gbdic_nn_conv_c2_direct(const gbdic_nn_conv_shape *s, const void *x, const float *weights, const float *bias,
                            void *y, void *stream) {
    if (!valid_shape(s) || s->C != 2 || s->Cout != 32 || !x || !y || !weights || !bias ||
        (reinterpret_cast<uintptr_t>(x) & 3) || (reinterpret_cast<uintptr_t>(y) & 15) ||
        (long long)s->B * s->OH * s->OW >= (1ll << 31))
        return invalid("direct convolution needs 2 input and 32 output channels, 4-byte aligned input, "
                       "16-byte aligned output and host weights");
    gbdic::NnConv1Weights w;
    for (int co = 0; co < 32; ++co) {
        for (int k = 0; k < 18; ++k) w.w[co][k] = weights[co * 18 + k];
        w.bias[co] = bias[co];
    }
    return rc(gbdic::launch_nn_conv_c2_direct(shape_of(s), x, w, y, as_stream(stream)), "direct convolution");
}

int gbdic_nn_dgrad_gather(const gbdic_nn_conv_shape *s, const void *dz, void *g, void *stream) {
    if (!valid_shape(s) || !dz || !g) return invalid("invalid convolution shape or pointers");
    return rc(gbdic::launch_nn_dgrad_gather(shape_of(s), dz, g, as_stream(stream)), "gradient gather");
}

int gbdic_nn_transpose(const void *src, int32_t rows, int32_t cols, int32_t ld_src, void *dst, int32_t rows_padded,
                       int32_t cols_padded, void *stream) {
    if (!src || !dst || rows < 0 || cols < 0 || ld_src < cols || rows_padded < rows || cols_padded < cols)
        return invalid("invalid transpose arguments");
    return rc(gbdic::launch_nn_transpose(src, rows, cols, ld_src, dst, rows_padded, cols_padded, as_stream(stream)),
              "transpose");
}

int gbdic_nn_relu_backward(const float *dy, int32_t ld, const void *y, void *dz, int64_t rows, int32_t cols,
                           void *stream) {
    if (!dy || !y || !dz || ld < cols || rows < 0 || cols <= 0) return invalid("invalid ReLU backward arguments");
    return rc(gbdic::launch_nn_relu_backward(dy, ld, y, dz, rows, cols, as_stream(stream)), "ReLU backward");
}

int gbdic_nn_bias_grad(const float *dy, int32_t ld, const void *y, int64_t rows, int32_t cols, float *db,
                       void *stream) {
    if (!dy || !db || ld < cols || rows < 0 || cols <= 0) return invalid("invalid bias gradient arguments");
    return rc(gbdic::launch_nn_bias_grad(dy, ld, y, rows, cols, db, as_stream(stream)), "bias gradient");
}

int gbdic_nn_relu_bias_backward(const float *dy, int32_t ld, const void *y, int64_t rows, int32_t cols, void *dz,
                                void *dz_t, float *partial, float *db, void *stream) {
    if (!dy || !dz || !partial || !db || ld < cols || rows <= 0 || cols <= 0)
        return invalid("invalid ReLU/bias backward arguments");
    return rc(gbdic::launch_nn_relu_bias_backward(dy, ld, y, rows, cols, dz, dz_t, partial, db, as_stream(stream)),
              "ReLU/bias backward (cols a power of two 4..256, ld % 4 == 0, rows % 8 == 0 with dz_t, aligned)");
}

int gbdic_nn_splitk_bias_relu(const float *partial, int32_t splits, int64_t rows, int32_t cols, int64_t split_stride,
                              const float *bias, int32_t relu, void *y, void *stream) {
    return rc(gbdic::launch_nn_splitk_bias_relu(partial, splits, rows, cols, split_stride, bias, relu, y,
                                                as_stream(stream)),
              "split-K epilogue (cols % 4 == 0, split_stride >= rows * cols, aligned)");
}

int gbdic_nn_im2col_t(const gbdic_nn_conv_shape *s, const void *x, void *a_t, int32_t rows_padded, void *stream) {
    if (!valid_shape(s) || !x || !a_t || rows_padded < s->Kp) return invalid("invalid convolution shape or pointers");
    return rc(gbdic::launch_nn_im2col_t(shape_of(s), x, a_t, rows_padded, as_stream(stream)),
              "transposed im2col (B*OH*OW % 8 == 0, rows_padded % 64 == 0, 16-byte aligned)");
}

int gbdic_nn_splitk_reduce(const float *partial, int32_t splits, int32_t kp_rows, int32_t n, int32_t kp, float *out,
                           void *stream) {
    if (!partial || !out || splits < 1 || kp > kp_rows || n <= 0 || kp <= 0) return invalid("invalid split-K reduction");
    return rc(gbdic::launch_nn_splitk_reduce(partial, splits, kp_rows, n, kp, out, as_stream(stream)), "split-K reduce");
}

int gbdic_nn_adam(float *param, const float *grad, float *m, float *v, int64_t count, const float *hyper,
                  void *stream) {
    if (!param || !grad || !m || !v || !hyper || count < 0) return invalid("invalid Adam arguments");
    gbdic::NnAdamArgs a{param, grad, m, v, count, hyper[0], hyper[1], hyper[2], hyper[3], hyper[4], hyper[5], hyper[6]};
    return rc(gbdic::launch_nn_adam(a, as_stream(stream)), "Adam");
}

int gbdic_nn_adam_many(float *const *params, const float *const *grads, float *const *m, float *const *v,
                       const int64_t *counts, int32_t tensors, const float *hyper, void *stream) {
    if (!params || !grads || !m || !v || !counts || !hyper || tensors < 1 || tensors > gbdic::kMaxAdamTensors)
        return invalid("invalid Adam arguments (1 to 16 tensors)");
    gbdic::NnAdamMany a{};
    a.n = tensors;
    a.offset[0] = 0;
    for (int t = 0; t < tensors; ++t) {
        if (!params[t] || !grads[t] || !m[t] || !v[t] || counts[t] < 0) return invalid("invalid Adam tensor");
        a.param[t] = params[t]; a.grad[t] = grads[t]; a.m[t] = m[t]; a.v[t] = v[t];
        a.offset[t + 1] = a.offset[t] + counts[t];
    }
    a.lr = hyper[0]; a.beta1 = hyper[1]; a.beta2 = hyper[2]; a.eps = hyper[3];
    a.bias1 = hyper[4]; a.bias2 = hyper[5]; a.weight_decay = hyper[6];
    return rc(gbdic::launch_nn_adam_many(a, as_stream(stream)), "Adam");
}

int gbdic_nn_pack_weights(const float *w, int32_t cout, int32_t cin, int32_t kp, void *wb, void *wt, int32_t kt,
                          void *stream) {
    if (!w || !wb || cout <= 0 || cin <= 0 || kp < 9 * cin || (wt && kt < 9 * cout))
        return invalid("invalid weight packing arguments");
    return rc(gbdic::launch_nn_pack_weights(w, cout, cin, kp, wb, wt, kt, as_stream(stream)), "weight packing");
}

int gbdic_nn_regression_loss(const float *pred, int32_t ldp, const float *target, int32_t outputs, int32_t batch,
                             void *grad, float *grad_f32, int32_t ldg, float *loss, void *stream) {
    if (!pred || !target || !grad || !loss || outputs <= 0 || ldp < outputs || ldg < outputs || batch <= 0)
        return invalid("invalid loss arguments");
    return rc(gbdic::launch_nn_regression_loss(pred, ldp, target, outputs, batch, grad, grad_f32, ldg, loss,
                                               as_stream(stream)),
              "regression loss");
}

int gbdic_reduce_half(const uint8_t *src, int32_t width, int32_t height, uint8_t *dst, void *stream) {
    if (!src || !dst || width < 2 || height < 2) return invalid("invalid reduction arguments");
    return rc(gbdic::launch_reduce_half(src, width, height, dst, as_stream(stream)), "pyramid reduction");
}

int gbdic_nn_lattice_seeds(const float *pred, const float *base, int32_t ldp, int32_t lattice_w, int32_t lattice_h,
                           int32_t step, int32_t grid_w, int32_t grid_h, int32_t subset_stride, float translation_scale,
                           float gradient_scale, float *seeds, uint32_t *active, void *stream) {
    if (!pred || !seeds || !active || ldp < 6 || lattice_w < 1 || lattice_h < 1 || step < 1 || grid_w < 1 ||
        grid_h < 1 || subset_stride < 1 || (lattice_w - 1) * step < grid_w - step || (lattice_h - 1) * step < grid_h - step ||
        !(gradient_scale != 0.0f))
        return invalid("invalid lattice seed arguments");
    gbdic::NnLatticeArgs a{pred, base, ldp, lattice_w, lattice_h, step, grid_w, grid_h, subset_stride,
                           translation_scale, gradient_scale, seeds, active};
    return rc(gbdic::launch_nn_lattice_seeds(a, as_stream(stream)), "lattice seeds");
}

int gbdic_nn_consensus(const float *pred, float *base, int32_t ldp, int32_t nodes, const float *node_xy,
                       const int32_t *singles, int32_t n_single, const int32_t *triples, int32_t n_triple,
                       const int32_t *probes, int32_t n_probe, const float *tolerances, int32_t n_tol,
                       float translation_scale, void *stream) {
    if (!pred || !base || !node_xy || ldp < 4 || nodes < 0 || n_single < 0 || n_triple < 0 || n_probe < 0 ||
        (n_single && !singles) || (n_triple && !triples) || (n_probe && !probes) || n_probe > 256 || !tolerances || n_tol < 1 ||
        n_tol > 4 || !(translation_scale > 0.0f) || (reinterpret_cast<uintptr_t>(node_xy) & 7))
        return invalid("invalid consensus arguments");
    gbdic::NnConsensusArgs a{};
    a.pred = pred; a.base = base; a.ldp = ldp; a.nodes = nodes;
    a.xy = reinterpret_cast<const float2 *>(node_xy);
    a.single = singles; a.n_single = n_single;
    a.triple = triples; a.n_triple = n_triple;
    a.probe = probes; a.n_probe = n_probe;
    for (int k = 0; k < n_tol; ++k) a.tol[k] = tolerances[k];
    a.n_tol = n_tol;
    a.scale = translation_scale;
    return rc(gbdic::launch_nn_consensus(a, as_stream(stream)), "consensus");
}

int gbdic_nn_reseed_select(const float *state, int32_t row_floats, const uint8_t *usable, int32_t count,
                           uint8_t *mask, uint32_t *active, uint32_t *counter, void *stream) {
    if (!state || !mask || !active || row_floats < 7 || count < 0) return invalid("invalid reseed selection arguments");
    return rc(gbdic::launch_nn_reseed_select(state, row_floats, usable, count, mask, active, counter, nullptr,
                                             as_stream(stream)),
              "reseed selection");
}

int gbdic_nn_reseed_select_list(const float *state, int32_t row_floats, const uint8_t *usable, int32_t count,
                                uint8_t *mask, uint32_t *active, uint32_t *counter, int32_t *list, void *stream) {
    if (!state || !mask || !active || !counter || !list || row_floats < 7 || count < 0)
        return invalid("invalid reseed selection arguments");
    return rc(gbdic::launch_nn_reseed_select(state, row_floats, usable, count, mask, active, counter,
                                             reinterpret_cast<int *>(list), as_stream(stream)),
              "reseed selection");
}

int gbdic_nn_merge_rows(const float *src, const uint8_t *mask, int32_t count, int32_t row_floats, float *dst,
                        void *stream) {
    if (!src || !mask || !dst || count < 0 || row_floats < 1) return invalid("invalid merge arguments");
    return rc(gbdic::launch_nn_merge_rows(src, mask, count, row_floats, dst, as_stream(stream)), "row merge");
}

int gbdic_nn_node_rows(const float *state, int32_t grid_w, int32_t grid_h, int32_t step, int32_t lattice_w,
                       int32_t lattice_h, float *pred, const float *base, int32_t ldp, float translation_scale,
                       float gradient_scale, void *stream) {
    if (!state || !pred || ldp < 6 || grid_w < 1 || grid_h < 1 || step < 1 || lattice_w < 1 || lattice_h < 1 ||
        (lattice_w - 1) * step >= grid_w || (lattice_h - 1) * step >= grid_h || !(translation_scale != 0.0f) ||
        (reinterpret_cast<uintptr_t>(state) & 15))
        return invalid("invalid node row arguments");
    return rc(gbdic::launch_nn_node_rows(state, grid_w, grid_h, step, lattice_w, lattice_h, pred, base, ldp,
                                         translation_scale, gradient_scale, as_stream(stream)),
              "node rows");
}

}  // extern "C"
