"""The tcgen05 BF16 GEMM against an FP32 PyTorch product of the same BF16
operands (FP32 accumulation; relative tolerance 2e-3 of the result scale),
across tile widths, multi-stage K loops, epilogues and split-K."""

from __future__ import annotations

import ctypes as C

import pytest

from live_dic_gb300 import _native

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _gemm(a, b, *, d_f32=None, d_bf16=None, bias=None, relu=False, accumulate=False, k_split=1, split_stride=0,
          ldd=None):
    lib = _native.load()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    M, K = a.shape
    N = b.shape[0]
    desc = _native.NnGemmDesc(
        a.data_ptr(), b.data_ptr(), M, N, K, k_split,
        d_f32.data_ptr() if d_f32 is not None else None, d_bf16.data_ptr() if d_bf16 is not None else None,
        ldd or N, split_stride, bias.data_ptr() if bias is not None else None, int(relu), int(accumulate))
    code = lib.gbdic_nn_gemm(C.byref(desc), C.c_void_p(err.data_ptr()), None)
    _native.check(code, lib.gbdic_last_error(None))
    torch.cuda.synchronize()
    assert int(err.item()) == 0


def _operands(M, N, K, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    a = torch.randn(M, K, generator=g, device="cuda").to(torch.bfloat16)
    b = torch.randn(N, K, generator=g, device="cuda").to(torch.bfloat16)
    return a, b, a.float() @ b.float().T


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 64, 512), (128, 16, 192), (384, 32, 320), (128, 256, 1152)])
def test_gemm_matches_fp32_product(M, N, K):
    a, b, ref = _operands(M, N, K, M + N + K)
    out = torch.empty(M, N, device="cuda")
    _gemm(a, b, d_f32=out)
    scale = ref.abs().max().item()
    assert (out - ref).abs().max().item() <= 2e-3 * scale


def test_gemm_epilogue_bias_relu_bf16_and_accumulate():
    M, N, K = 256, 64, 256
    a, b, ref = _operands(M, N, K, 7)
    bias = torch.randn(N, device="cuda")
    out = torch.empty(M, N, device="cuda")
    out16 = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    _gemm(a, b, d_f32=out, d_bf16=out16, bias=bias, relu=True)
    expected = torch.relu(ref + bias)
    scale = expected.abs().max().item()
    assert (out - expected).abs().max().item() <= 2e-3 * scale
    assert (out16.float() - out).abs().max().item() <= 1e-2 * scale
    base = torch.randn(M, N, device="cuda")
    acc = base.clone()
    _gemm(a, b, d_f32=acc, accumulate=True)
    assert (acc - (base + ref)).abs().max().item() <= 2e-3 * ref.abs().max().item()


def test_gemm_split_k_partials_sum_to_product():
    M, N, K, S = 128, 32, 2048, 4
    a, b, ref = _operands(M, N, K, 11)
    partial = torch.empty(S, M, N, device="cuda")
    _gemm(a, b, d_f32=partial, k_split=S, split_stride=M * N)
    total = partial.sum(0)
    assert (total - ref).abs().max().item() <= 2e-3 * ref.abs().max().item()
    for s in range(S):
        chunk = a[:, s * K // S:(s + 1) * K // S].float() @ b[:, s * K // S:(s + 1) * K // S].float().T
        assert (partial[s] - chunk).abs().max().item() <= 2e-3 * chunk.abs().max().item()


def test_gemm_rejects_unpadded_shapes():
    a, b, _ = _operands(128, 16, 64, 3)
    out = torch.empty(128, 16, device="cuda")
    with pytest.raises(ValueError, match="tensor-core GEMM"):
        _gemm(a[:100], b, d_f32=out)


def _conv_gemm(src, b, mode, shape, M, K, d_f32):
    lib = _native.load()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    desc = _native.NnGemmDesc(src.data_ptr(), b.data_ptr(), M, b.shape[0], K, 1, d_f32.data_ptr(), None,
                              b.shape[0], 0, None, 0, 0)
    code = lib.gbdic_nn_conv_gemm(C.byref(desc), mode, C.byref(shape), C.c_void_p(err.data_ptr()), None)
    _native.check(code, lib.gbdic_last_error(None))
    torch.cuda.synchronize()
    assert int(err.item()) == 0


def _conv_case(B, H, Cin, Cout, seed):
    OH = (H + 1) // 2
    return _native.NnConvShape(B, H, H, Cin, OH, OH, Cout, -(-9 * Cin // 64) * 64), torch.Generator(
        device="cuda").manual_seed(seed)


@pytest.mark.parametrize("B,H,Cin,Cout", [(8, 32, 32, 64), (4, 16, 64, 128), (16, 8, 128, 32), (2, 32, 16, 16),
                                        (2, 16, 8, 64), (1, 31, 32, 64)])
def test_implicit_im2col_gemm_equals_materialised_operand(B, H, Cin, Cout):
    """Operand A gathered in the kernel as im2col rows of the NHWC input
    gives the GEMM of the materialised im2col matrix bit for bit: the same
    operand values reach the tensor cores in the same K order (zero taps at
    the border and in the K padding beyond 9 C)."""
    lib = _native.load()
    shape, g = _conv_case(B, H, Cin, Cout, B * H + Cin)
    M = B * shape.OH * shape.OW
    if M % 128:
        pytest.skip("rows must fill 128-row tiles")
    x = torch.randn(B, H, H, Cin, generator=g, device="cuda").to(torch.bfloat16)
    w = torch.randn(Cout, shape.Kp, generator=g, device="cuda").to(torch.bfloat16)
    a = torch.empty(M, shape.Kp, dtype=torch.bfloat16, device="cuda")
    _native.check(lib.gbdic_nn_im2col(C.byref(shape), C.c_void_p(x.data_ptr()), C.c_void_p(a.data_ptr()), None),
                  lib.gbdic_last_error(None))
    want = torch.empty(M, Cout, device="cuda")
    _gemm(a, w, d_f32=want)
    got = torch.empty(M, Cout, device="cuda")
    _conv_gemm(x, w, 1, shape, M, shape.Kp, got)
    assert torch.equal(got, want)


@pytest.mark.parametrize("B,H,Cin,Cout", [(8, 32, 32, 64), (4, 16, 64, 128), (16, 8, 128, 64), (2, 32, 16, 64),
                                        (1, 32, 64, 192), (1, 16, 32, 64), (128, 15, 16, 64)])
def test_implicit_dgrad_gemm_equals_materialised_operand(B, H, Cin, Cout):
    """Operand A gathered in the kernel as the data-gradient rows of the
    output gradient (stride-2 transposed taps) gives the GEMM of the
    materialised gather matrix bit for bit.  The first five shapes take the
    parity-class form (rows by the input pixel's parity, zero tap blocks
    skipped); B 1 x 16^2 (a class of 64 rows) and the odd side 15 take the
    plain gather."""
    lib = _native.load()
    shape, g = _conv_case(B, H, Cin, Cout, B * H + Cout)
    OH = shape.OH
    dz = torch.randn(B, OH, OH, Cout, generator=g, device="cuda").to(torch.bfloat16)
    wt = torch.randn(Cin, 9 * Cout, generator=g, device="cuda").to(torch.bfloat16)
    Min = B * H * H
    gmat = torch.empty(Min, 9 * Cout, dtype=torch.bfloat16, device="cuda")
    _native.check(lib.gbdic_nn_dgrad_gather(C.byref(shape), C.c_void_p(dz.data_ptr()), C.c_void_p(gmat.data_ptr()),
                                            None), lib.gbdic_last_error(None))
    want = torch.empty(Min, Cin, device="cuda")
    _gemm(gmat, wt, d_f32=want)
    got = torch.empty(Min, Cin, device="cuda")
    _conv_gemm(dz, wt, 2, shape, Min, 9 * Cout, got)
    assert torch.equal(got, want)


@pytest.mark.parametrize("B,H,Cin,Cout,splits", [(512, 8, 128, 128, 3), (512, 4, 128, 64, 18), (128, 8, 64, 128, 9)])
def test_split_k_implicit_im2col_gemm(B, H, Cin, Cout, splits):
    """Split-K implicit GEMM: every split's partial equals the materialised
    split GEMM's bit for bit, and the split-K epilogue gives bias + ReLU of
    their ordered sum in BF16."""
    lib = _native.load()
    shape, g = _conv_case(B, H, Cin, Cout, B + H + splits)
    M = B * shape.OH * shape.OW
    x = torch.randn(B, H, H, Cin, generator=g, device="cuda").to(torch.bfloat16)
    w = torch.randn(Cout, shape.Kp, generator=g, device="cuda").to(torch.bfloat16)
    bias = torch.randn(Cout, generator=g, device="cuda")
    a = torch.empty(M, shape.Kp, dtype=torch.bfloat16, device="cuda")
    _native.check(lib.gbdic_nn_im2col(C.byref(shape), C.c_void_p(x.data_ptr()), C.c_void_p(a.data_ptr()), None),
                  lib.gbdic_last_error(None))
    want = torch.empty(splits, M, Cout, device="cuda")
    _gemm(a, w, d_f32=want, k_split=splits, split_stride=M * Cout)
    got = torch.empty(splits, M, Cout, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    desc = _native.NnGemmDesc(x.data_ptr(), w.data_ptr(), M, Cout, shape.Kp, splits, got.data_ptr(), None, Cout,
                              M * Cout, None, 0, 0)
    _native.check(lib.gbdic_nn_conv_gemm(C.byref(desc), 1, C.byref(shape), C.c_void_p(err.data_ptr()), None),
                  lib.gbdic_last_error(None))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.equal(got, want)
    y = torch.empty(M, Cout, dtype=torch.bfloat16, device="cuda")
    _native.check(lib.gbdic_nn_splitk_bias_relu(C.c_void_p(got.data_ptr()), splits, M, Cout, M * Cout,
                                                C.c_void_p(bias.data_ptr()), 1, C.c_void_p(y.data_ptr()), None),
                  lib.gbdic_last_error(None))
    total = got[0].clone()
    for s in range(1, splits):
        total += got[s]
    assert torch.equal(y, torch.relu(total + bias).to(torch.bfloat16))


def test_implicit_conv_gemm_rejects_mismatched_shapes():
    x = torch.zeros(2, 16, 16, 32, dtype=torch.bfloat16, device="cuda")
    w = torch.zeros(64, 320, dtype=torch.bfloat16, device="cuda")
    out = torch.empty(128, 64, device="cuda")
    shape = _native.NnConvShape(2, 16, 16, 32, 8, 8, 64, 320)
    with pytest.raises(ValueError, match="implicit convolution GEMM"):
        _conv_gemm(x, w, 1, shape, 256, 320, out)   # rows are 2 * 8 * 8 = 128
