"""The seed network's fused glue kernels against their unfused forms: the
one-pass ReLU/bias backward (dZ, its transpose, the bias gradient) and the
transposed im2col the weight-gradient GEMM reads."""

from __future__ import annotations

import ctypes as C

import pytest

from live_dic_gb300 import _native

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("rows,cols,ld,masked", [(1024, 32, 32, True), (1000, 64, 64, True), (512, 16, 64, False),
                                                 (8192, 128, 128, True), (64, 4, 8, True)])
def test_relu_bias_backward_matches_unfused(rows, cols, ld, masked):
    lib = _native.load()
    g = torch.Generator(device="cuda").manual_seed(rows + cols)
    dy = torch.randn(rows, ld, generator=g, device="cuda")
    y = torch.randn(rows, cols, generator=g, device="cuda").to(torch.bfloat16) if masked else None
    dz = torch.empty(rows, cols, dtype=torch.bfloat16, device="cuda")
    dzt = torch.empty(cols, rows, dtype=torch.bfloat16, device="cuda")
    partial = torch.empty(cols * ((rows + 63) // 64), device="cuda")
    db = torch.empty(cols, device="cuda")
    code = lib.gbdic_nn_relu_bias_backward(_p(dy), ld, _p(y), rows, cols, _p(dz), _p(dzt), _p(partial), _p(db), None)
    _native.check(code, lib.gbdic_last_error(None))
    torch.cuda.synchronize()
    grad = dy[:, :cols] * (y.float() > 0) if masked else dy[:, :cols]
    assert torch.equal(dz, grad.to(torch.bfloat16))
    assert torch.equal(dzt, dz.T.contiguous())
    want = grad.double().sum(0)
    assert (db.double() - want).abs().max().item() <= 1e-5 * max(1.0, grad.abs().sum(0).max().item())
    # the unfused bias gradient gives the same column sums within rounding
    db_old = torch.empty(cols, device="cuda")
    _native.check(lib.gbdic_nn_bias_grad(_p(dy), ld, _p(y), rows, cols, _p(db_old), None), lib.gbdic_last_error(None))
    torch.cuda.synchronize()
    assert (db - db_old).abs().max().item() <= 1e-5 * max(1.0, grad.abs().sum(0).max().item())


def test_relu_bias_backward_rejects_unsupported_widths():
    lib = _native.load()
    dy = torch.zeros(64, 48, device="cuda")
    dz = torch.empty(64, 48, dtype=torch.bfloat16, device="cuda")
    part = torch.empty(48, device="cuda")
    db = torch.empty(48, device="cuda")
    with pytest.raises(ValueError, match="ReLU/bias backward"):
        _native.check(lib.gbdic_nn_relu_bias_backward(_p(dy), 48, None, 64, 48, _p(dz), None, _p(part), _p(db), None),
                      lib.gbdic_last_error(None))


@pytest.mark.parametrize("B,H,Cin,kp_rows", [(512, 64, 2, 128), (64, 32, 32, 384), (16, 16, 16, 256),
                                             (8, 15, 64, 640), (128, 4, 128, 1152)])
def test_transposed_im2col_equals_transpose_of_im2col(B, H, Cin, kp_rows):
    lib = _native.load()
    OH = (H + 1) // 2
    kp = -(-9 * Cin // 64) * 64
    shape = _native.NnConvShape(B, H, H, Cin, OH, OH, 32, kp)
    g = torch.Generator(device="cuda").manual_seed(B + H + Cin)
    x = torch.randn(B, H, H, Cin, generator=g, device="cuda").to(torch.bfloat16)
    M = B * OH * OH
    a = torch.empty(M, kp, dtype=torch.bfloat16, device="cuda")
    _native.check(lib.gbdic_nn_im2col(C.byref(shape), _p(x), _p(a), None), lib.gbdic_last_error(None))
    want = torch.full((kp_rows, M), 7.0, dtype=torch.bfloat16, device="cuda")
    _native.check(lib.gbdic_nn_transpose(_p(a), M, kp, kp, _p(want), M, kp_rows, None), lib.gbdic_last_error(None))
    # rows beyond the last 64-row tile holding k < 9 C are the caller's (kept zero)
    got = torch.zeros((kp_rows, M), dtype=torch.bfloat16, device="cuda")
    live = min(kp_rows, -(-9 * Cin // 64) * 64)
    got[live:] = 7.0
    _native.check(lib.gbdic_nn_im2col_t(C.byref(shape), _p(x), _p(got), kp_rows, None), lib.gbdic_last_error(None))
    torch.cuda.synchronize()
    assert torch.equal(got[:live], want[:live])
    assert (got[live:] == 7.0).all() and (want[live:] == 0).all()


def test_adam_many_equals_per_tensor_steps():
    """One multi-tensor Adam launch against one launch per tensor: the same
    parameters and moments bit for bit."""
    lib = _native.load()
    g = torch.Generator(device="cuda").manual_seed(5)
    sizes = [32 * 64, 64 * 320, 128, 16 * 256, 7]
    mk = lambda: [torch.randn(n, generator=g, device="cuda") for n in sizes]  # noqa: E731
    params, grads, ms, vs = mk(), mk(), mk(), [t.abs() for t in mk()]
    copies = [[t.clone() for t in group] for group in (params, grads, ms, vs)]
    hyper = (ctypes_float7 := (C.c_float * 7)(2e-3, 0.9, 0.999, 1e-8, 0.1, 0.001, 1e-4))
    for p, gr, m, v in zip(*copies, strict=True):
        _native.check(lib.gbdic_nn_adam(_p(p), _p(gr), _p(m), _p(v), p.numel(), ctypes_float7, None),
                      lib.gbdic_last_error(None))
    n = len(sizes)
    arr = lambda ts: (C.c_void_p * n)(*[t.data_ptr() for t in ts])  # noqa: E731
    _native.check(lib.gbdic_nn_adam_many(arr(params), arr(grads), arr(ms), arr(vs), (C.c_int64 * n)(*sizes), n, hyper,
                                         None), lib.gbdic_last_error(None))
    torch.cuda.synchronize()
    for a, b in zip(params + ms + vs, copies[0] + copies[2] + copies[3], strict=True):
        assert torch.equal(a, b)
