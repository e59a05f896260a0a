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
