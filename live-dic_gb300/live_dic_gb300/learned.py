"""Learned seed proposal: a small CNN that maps a reference/target patch pair
to an initial affine warp for IC-GN.

No counterpart in the reference (its large-motion initialisers are the image
pyramid, the Fourier phase correlation of fourier.py and the optional
wgpu-matching package).  The network, its training and its use are built on
the library's own kernels:

* ``SeedNet`` -- five 3x3 stride-2 convolutions with ReLU (channels 32, 64,
  128, 128, 64) and a linear layer to 6 outputs (315,878 parameters) on
  64 x 64 x 2 patches.  Forward and backward run as GEMMs on the tcgen05
  tensor cores (BF16 operands, FP32 accumulation in tensor memory): the
  im2col rows of the forward and the gathered output gradients of the data
  gradient are built inside the GEMM kernel from the NHWC tensors (implicit
  GEMM, gbdic_nn_conv_gemm; the 2-channel input layer keeps a materialised
  im2col), then GEMM(+bias, ReLU); weight gradients are transposed im2col
  (written straight from the layer input) x transposed output gradients
  (written by the one-pass ReLU/bias backward), split-K with a fixed-order
  reduction.
  FP32 master weights, Adam.  PyTorch only allocates the device buffers and
  owns the stream.
* ``training_pairs`` -- subset pairs the engine generates itself: seeded
  speckle under random affine warps (translation +-20 px, strain +-5 %,
  rotation +-3 deg), labelled by IC-GN converged from the imposed warp.
* ``LearnedSeeder`` -- per frame: half-resolution pyramid level, the network
  on a lattice of every `step`-th subset in several passes (after each, a
  robust affine fit of the lattice translations displaces the target
  windows and the next pass predicts the residual warp), lattice ->
  per-subset seeds (bilinear blend of Taylor-recentred warps), seeded IC-GN;
  subsets that do not converge or whose ZNCC falls below the threshold are
  reseeded by the integer ZNCC search around their proposal and solved
  again.

Outputs are normalised as [tx / 16, ux * 20, uy * 20, ty / 16, vx * 20,
vy * 20] (translations in full-resolution pixels).
"""

from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np

from . import _native
from .engine import ICGNError

CONV_CHANNELS = ((2, 32), (32, 64), (64, 128), (128, 128), (128, 64))
PATCH = 64
OUTPUTS = 6
OUT_PAD = 16          # linear-layer output columns (GEMM tile)
LOSS_PAD = 64         # K padding of the output gradient
TRANSLATION_SCALE = 16.0
GRADIENT_SCALE = 20.0
CONSENSUS_TOLERANCES = (8.0, 6.0, 4.0, 3.0)   # px: hypothesis scoring, then refits
NODE_ITERATIONS = 8   # Gauss-Newton iterations of the lattice-node solve
NORMALISATION = np.array([1 / TRANSLATION_SCALE, GRADIENT_SCALE, GRADIENT_SCALE, 1 / TRANSLATION_SCALE,
                          GRADIENT_SCALE, GRADIENT_SCALE], np.float32)


def _torch():
    import torch

    return torch


def _pad(x: int, m: int) -> int:
    return (x + m - 1) // m * m


def _ptr(t) -> C.c_void_p | None:
    return None if t is None else C.c_void_p(t.data_ptr())


def _call(lib, name: str, *args) -> None:
    code = getattr(lib, name)(*args)
    _native.check(code, lib.gbdic_last_error(None))


@dataclass
class _Conv:
    cin: int
    cout: int
    H: int            # input side
    OH: int           # output side
    kp: int           # forward reduction length (padded 9 cin)
    kp_rows: int      # kp padded to 128 (rows of the weight-gradient GEMM)
    kt: int           # data-gradient reduction length (9 cout)
    M: int            # output rows (B OH^2)
    Min: int          # input rows (B H^2)


class SeedNet:
    """The proposal network and its optimiser state on one CUDA device.
    ``batch`` (a multiple of 128) fixes the buffer shapes.  ``split_forward``
    (inference copies) runs the deep gathered layers split-K; it changes the
    forward's summation order, so training keeps it off."""

    def __init__(self, batch: int = 512, *, device: int = 0, seed: int = 0, split_forward: bool = False) -> None:
        torch = _torch()
        if batch <= 0 or batch % 128:
            raise ValueError("batch must be a positive multiple of 128")
        self.lib = _native.load()
        self.B = batch
        self.device = torch.device("cuda", device)
        dev = self.device
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.convs: list[_Conv] = []
        H = PATCH
        for cin, cout in CONV_CHANNELS:
            oh = (H + 1) // 2
            kp = _pad(9 * cin, 64)
            self.convs.append(_Conv(cin, cout, H, oh, kp, _pad(kp, 128), 9 * cout, batch * oh * oh, batch * H * H))
            H = oh
        self.features = CONV_CHANNELS[-1][1] * H * H  # 64 x 2 x 2 = 256
        bf16, f32 = torch.bfloat16, torch.float32
        self.params: list = []
        # conv weights [Cout][kp] (zero beyond 9 cin), He initialisation
        self.w, self.b = [], []
        for c in self.convs:
            w = torch.zeros(c.cout, c.kp)
            w[:, :9 * c.cin] = torch.randn(c.cout, 9 * c.cin, generator=g) * math.sqrt(2.0 / (9 * c.cin))
            self.w.append(w.to(dev))
            self.b.append(torch.zeros(c.cout, device=dev))
        w6 = torch.zeros(OUT_PAD, self.features)
        w6[:OUTPUTS] = torch.randn(OUTPUTS, self.features, generator=g) * math.sqrt(1.0 / self.features)
        self.w6 = w6.to(dev)
        self.b6 = torch.zeros(OUT_PAD, device=dev)
        self.params = [*self.w, *self.b, self.w6, self.b6]
        self.grads = [torch.zeros_like(p) for p in self.params]
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.steps = 0
        self._adam_tables = None  # device pointers and sizes of params / grads / moments (fixed)
        # BF16 operands
        self.wb = [torch.zeros(c.cout, c.kp, dtype=bf16, device=dev) for c in self.convs]
        self.wt = [torch.zeros(c.cin, c.kt, dtype=bf16, device=dev) for c in self.convs]
        self.w6b = torch.zeros(OUT_PAD, self.features, dtype=bf16, device=dev)
        self.w6t = torch.zeros(self.features, LOSS_PAD, dtype=bf16, device=dev)
        # activations
        self.x0 = torch.zeros(batch, PATCH, PATCH, 2, dtype=bf16, device=dev)
        # materialised im2col operand only for layers whose channel count is
        # not a multiple of 8 (the 2-channel input layer); the others gather
        # it inside the GEMM
        self.a = [torch.zeros(c.M, c.kp, dtype=bf16, device=dev) if c.cin % 8 else None for c in self.convs]
        self.y = [torch.zeros(c.M, c.cout, dtype=bf16, device=dev) for c in self.convs]
        # Split-K forward for the gathered layers whose output tiles would not
        # fill one wave of CTAs (the deep layers at small batches): FP32
        # partials, then one fixed-order reduction with bias and ReLU.
        self.fwd_splits = [self._forward_splits(c) if split_forward and c.cin % 8 == 0 else 1 for c in self.convs]
        self.fwd_partial = [torch.zeros(s, c.M, c.cout, dtype=f32, device=dev) if s > 1 else None
                            for s, c in zip(self.fwd_splits, self.convs, strict=True)]
        self.out = torch.zeros(batch, OUT_PAD, dtype=f32, device=dev)
        # backward buffers (allocated on first backward)
        self._bwd = None
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.loss = torch.zeros(1, dtype=f32, device=dev)
        self.pack()

    # ------------------------------------------------------------ kernels
    def _gemm(self, a, b, M, N, K, *, d_f32=None, d_bf16=None, ldd=None, bias=None, relu=False, k_split=1,
              split_stride=0, stream=None, gather: int = 0, shape=None):
        """D = A B^T on the tensor cores; with `gather` (1 im2col of the
        input `a`, 2 data-gradient gather of the output gradient `a`) operand
        A is gathered in the kernel from the NHWC tensor `a` of `shape`."""
        desc = _native.NnGemmDesc(a.data_ptr(), b.data_ptr(), M, N, K, k_split,
                                  d_f32.data_ptr() if d_f32 is not None else None,
                                  d_bf16.data_ptr() if d_bf16 is not None else None, ldd or N, split_stride,
                                  bias.data_ptr() if bias is not None else None, int(relu), 0)
        if gather:
            _call(self.lib, "gbdic_nn_conv_gemm", C.byref(desc), gather, C.byref(shape), _ptr(self.err), stream)
        else:
            _call(self.lib, "gbdic_nn_gemm", C.byref(desc), _ptr(self.err), stream)

    def _shape(self, i: int) -> _native.NnConvShape:
        c = self.convs[i]
        return _native.NnConvShape(self.B, c.H, c.H, c.cin, c.OH, c.OH, c.cout, c.kp)

    def pack(self, stream=None) -> None:
        """BF16 operands from the FP32 master weights."""
        for i, c in enumerate(self.convs):
            _call(self.lib, "gbdic_nn_pack_weights", _ptr(self.w[i]), c.cout, c.cin, c.kp, _ptr(self.wb[i]),
                  _ptr(self.wt[i]), c.kt, stream)
        _call(self.lib, "gbdic_nn_pack_weights", _ptr(self.w6), OUT_PAD, 1, self.features, _ptr(self.w6b), None, 0,
              stream)
        _call(self.lib, "gbdic_nn_transpose", _ptr(self.w6b), OUT_PAD, self.features, self.features, _ptr(self.w6t),
              LOSS_PAD, self.features, stream)

    def use_direct_first_layer(self) -> None:
        """Inference copies: run the 2-channel input layer as one direct
        convolution (gbdic_nn_conv_c2_direct) with the current BF16 weights,
        read to the host once here; later weight updates are not seen, and
        the layer's im2col operand (needed by backward) is not written."""
        torch = _torch()
        c = self.convs[0]
        w = self.w[0][:, :9 * c.cin].to(torch.bfloat16).float().cpu().numpy()
        self._direct = (np.ascontiguousarray(w, dtype=np.float32),
                        np.ascontiguousarray(self.b[0].cpu().numpy(), dtype=np.float32))

    # ------------------------------------------------------------ forward
    def forward(self, stream=None):
        """self.x0 (B x 64 x 64 x 2 BF16) -> self.out (B x 16 FP32, first 6 used)."""
        x = self.x0
        direct = getattr(self, "_direct", None)
        for i, c in enumerate(self.convs):
            if i == 0 and direct is not None:
                _call(self.lib, "gbdic_nn_conv_c2_direct", C.byref(self._shape(0)), _ptr(x),
                      direct[0].ctypes.data_as(C.c_void_p), direct[1].ctypes.data_as(C.c_void_p), _ptr(self.y[0]),
                      stream)
                x = self.y[0]
                continue
            if c.cin % 8 == 0 and self.fwd_splits[i] > 1:
                # implicit GEMM, split K, then bias + ReLU over the partials
                s, part = self.fwd_splits[i], self.fwd_partial[i]
                self._gemm(x, self.wb[i], c.M, c.cout, c.kp, d_f32=part, k_split=s, split_stride=c.M * c.cout,
                           stream=stream, gather=1, shape=self._shape(i))
                _call(self.lib, "gbdic_nn_splitk_bias_relu", _ptr(part), s, c.M, c.cout, c.M * c.cout, _ptr(self.b[i]),
                      1, _ptr(self.y[i]), stream)
            elif c.cin % 8 == 0:
                # implicit GEMM: the im2col rows are gathered in the kernel
                self._gemm(x, self.wb[i], c.M, c.cout, c.kp, d_bf16=self.y[i], bias=self.b[i], relu=True,
                           stream=stream, gather=1, shape=self._shape(i))
            else:
                _call(self.lib, "gbdic_nn_im2col", C.byref(self._shape(i)), _ptr(x), _ptr(self.a[i]), stream)
                self._gemm(self.a[i], self.wb[i], c.M, c.cout, c.kp, d_bf16=self.y[i], bias=self.b[i], relu=True,
                           stream=stream)
            x = self.y[i]
        self._gemm(self.y[-1], self.w6b, self.B, OUT_PAD, self.features, d_f32=self.out, bias=self.b6, stream=stream)
        return self.out

    # ------------------------------------------------------------ backward
    def _backward_buffers(self):
        torch = _torch()
        dev, bf16, f32 = self.device, torch.bfloat16, torch.float32
        B = self.B
        bufs = {
            "dout": torch.zeros(B, LOSS_PAD, dtype=bf16, device=dev),
            "dout_f32": torch.zeros(B, LOSS_PAD, dtype=f32, device=dev),
            "doutT": torch.zeros(OUT_PAD, B, dtype=bf16, device=dev),
            "y5T": torch.zeros(self.features, B, dtype=bf16, device=dev),
            "dw6T": torch.zeros(self.features, OUT_PAD, dtype=f32, device=dev),
            "dy": [torch.zeros(c.M, c.cout, dtype=f32, device=dev) for c in self.convs],
            "dz": [torch.zeros(c.M, c.cout, dtype=bf16, device=dev) for c in self.convs],
            "db_partial": [torch.zeros(c.cout * ((c.M + 63) // 64), dtype=f32, device=dev) for c in self.convs],
            "dzT": [torch.zeros(c.cout, c.M, dtype=bf16, device=dev) for c in self.convs],
            "aT": [torch.zeros(c.kp_rows, c.M, dtype=bf16, device=dev) for c in self.convs],
        }
        bufs["splits"] = [self._splits(c) for c in self.convs]
        bufs["partial"] = [torch.zeros(s, c.kp_rows, c.cout, dtype=f32, device=dev)
                           for s, c in zip(bufs["splits"], self.convs, strict=True)]
        return bufs

    @staticmethod
    def _forward_splits(c: _Conv, sms: int = 152) -> int:
        """Smallest divisor s of the K blocks with (output tiles) x s >= one
        wave of CTAs (1 when the tiles already fill it)."""
        tiles = (c.M // 128) * max(1, c.cout // min(128, c.cout))
        blocks = c.kp // 64
        if tiles >= sms:
            return 1
        for s in range(2, blocks + 1):
            if blocks % s == 0 and tiles * s >= sms:
                return s
        return blocks

    @staticmethod
    def _splits(c: _Conv) -> int:
        tiles = (c.kp_rows // 128) * max(1, c.cout // 128)
        want = max(1, 304 // tiles)
        s = 1
        while s * 2 <= want and c.M % (64 * s * 2) == 0 and c.M // (s * 2) >= 256:
            s *= 2
        return s

    def loss_and_grad(self, target, stream=None) -> None:
        """Loss of self.out against `target` (B x 6 FP32, normalised) into
        self.loss and the output gradient."""
        if self._bwd is None:
            self._bwd = self._backward_buffers()
        b = self._bwd
        _call(self.lib, "gbdic_nn_regression_loss", _ptr(self.out), OUT_PAD, _ptr(target), OUTPUTS, self.B,
              _ptr(b["dout"]), _ptr(b["dout_f32"]), LOSS_PAD, _ptr(self.loss), stream)

    def backward(self, stream=None) -> None:
        """Gradients of every parameter into self.grads (after loss_and_grad)."""
        b = self._bwd
        lib, B, F = self.lib, self.B, self.features
        nconv = len(self.convs)
        # linear layer: dW6^T = Y5^T dOut, db6 = sum dOut, dY5 = dOut W6
        _call(lib, "gbdic_nn_transpose", _ptr(self.y[-1]), B, F, F, _ptr(b["y5T"]), B, F, stream)
        _call(lib, "gbdic_nn_transpose", _ptr(b["dout"]), B, OUT_PAD, LOSS_PAD, _ptr(b["doutT"]), B, OUT_PAD, stream)
        self._gemm(b["y5T"], b["doutT"], F, OUT_PAD, B, d_f32=b["dw6T"], stream=stream)
        _call(lib, "gbdic_nn_splitk_reduce", _ptr(b["dw6T"]), 1, F, OUT_PAD, F, _ptr(self.grads[2 * nconv]), stream)
        _call(lib, "gbdic_nn_bias_grad", _ptr(b["dout_f32"]), LOSS_PAD, None, B, OUT_PAD,
              _ptr(self.grads[2 * nconv + 1]), stream)
        self._gemm(b["dout"], self.w6t, B, F, LOSS_PAD, d_f32=b["dy"][-1].view(B, F), stream=stream)
        for i in range(nconv - 1, -1, -1):
            c = self.convs[i]
            dy, dz = b["dy"][i], b["dz"][i]
            # dZ, its transpose and the bias gradient in one pass over dY
            _call(lib, "gbdic_nn_relu_bias_backward", _ptr(dy), c.cout, _ptr(self.y[i]), c.M, c.cout, _ptr(dz),
                  _ptr(b["dzT"][i]), _ptr(b["db_partial"][i]), _ptr(self.grads[nconv + i]), stream)
            # weight gradient: dW^T[k][co] = sum_m A[m][k] dZ[m][co], with A^T
            # written straight from the layer input (A is never materialised)
            x = self.x0 if i == 0 else self.y[i - 1]
            _call(lib, "gbdic_nn_im2col_t", C.byref(self._shape(i)), _ptr(x), _ptr(b["aT"][i]), c.kp_rows, stream)
            splits = b["splits"][i]
            self._gemm(b["aT"][i], b["dzT"][i], c.kp_rows, c.cout, c.M, d_f32=b["partial"][i], k_split=splits,
                       split_stride=c.kp_rows * c.cout, stream=stream)
            _call(lib, "gbdic_nn_splitk_reduce", _ptr(b["partial"][i]), splits, c.kp_rows, c.cout, c.kp,
                  _ptr(self.grads[i]), stream)
            if i > 0:
                # data gradient: dY_{i-1}[m][ci] = sum_(ky,kx,co) G[m][.] Wt[ci][.],
                # G gathered from dZ in the kernel (implicit GEMM)
                self._gemm(dz, self.wt[i], c.Min, c.cin, c.kt, d_f32=b["dy"][i - 1], stream=stream, gather=2,
                           shape=self._shape(i))

    def adam_step(self, lr: float = 1e-3, *, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
                  weight_decay: float = 0.0, stream=None) -> None:
        self.steps += 1
        t = self.steps
        hyper = (C.c_float * 7)(lr, beta1, beta2, eps, 1 - beta1 ** t, 1 - beta2 ** t, weight_decay)
        if self._adam_tables is None:
            n = len(self.params)
            ptrs = (C.c_void_p * n)
            self._adam_tables = (ptrs(*[p.data_ptr() for p in self.params]), ptrs(*[g.data_ptr() for g in self.grads]),
                                 ptrs(*[m.data_ptr() for m in self.m]), ptrs(*[v.data_ptr() for v in self.v]),
                                 (C.c_int64 * n)(*[p.numel() for p in self.params]), n)
        params, grads, ms, vs, counts, n = self._adam_tables
        # every parameter tensor in one launch, per element gbdic_nn_adam's update
        _call(self.lib, "gbdic_nn_adam_many", params, grads, ms, vs, counts, n, hyper, stream)
        self.pack(stream)

    def check_device_errors(self) -> None:
        if int(self.err.item()) != 0:
            raise ICGNError("a tensor-core GEMM pipeline wait expired")

    # ------------------------------------------------------------ patches
    def load_patches(self, refs, tgts, image_index, centres, count: int, width: int, height: int, stream=None):
        """Patches into self.x0 (rows beyond `count` keep their contents)."""
        _call(self.lib, "gbdic_nn_patches", _ptr(refs), _ptr(tgts), _ptr(image_index), _ptr(centres), count, width,
              height, _ptr(self.x0), None, 0, C.c_float(0.0), stream)

    def state_dict(self) -> dict[str, np.ndarray]:
        names = [f"w{i}" for i in range(len(self.w))] + [f"b{i}" for i in range(len(self.b))] + ["w6", "b6"]
        return {n: p.detach().cpu().numpy() for n, p in zip(names, self.params, strict=True)}

    def load_state_dict(self, state: dict[str, np.ndarray]) -> None:
        torch = _torch()
        names = [f"w{i}" for i in range(len(self.w))] + [f"b{i}" for i in range(len(self.b))] + ["w6", "b6"]
        for n, p in zip(names, self.params, strict=True):
            p.copy_(torch.as_tensor(state[n], device=self.device))
        self.pack()
        if getattr(self, "_direct", None) is not None:
            self.use_direct_first_layer()


# ---------------------------------------------------------------- training data
def random_warp(rng: np.random.Generator, *, translation: float = 20.0, strain: float = 0.05,
                rotation_deg: float = 3.0) -> tuple[np.ndarray, np.ndarray]:
    """(t, G): translation and displacement gradient R (I + E) - I."""
    t = rng.uniform(-translation, translation, 2)
    exx, eyy, exy = rng.uniform(-strain, strain, 3)
    th = math.radians(rng.uniform(-rotation_deg, rotation_deg))
    R = np.array([[math.cos(th), -math.sin(th)], [math.sin(th), math.cos(th)]])
    G = R @ (np.eye(2) + np.array([[exx, exy], [exy, eyy]])) - np.eye(2)
    return t, G


@dataclass
class TrainingSet:
    """Level-1 images on the device and labelled patch centres."""

    refs: object          # torch uint8 [n, h, w]
    tgts: object
    ref_ptrs: object      # torch int64 [n] device pointers
    tgt_ptrs: object
    image_index: object   # torch int32 [P]
    centres: object       # torch float32 [P, 2] level-1 pixels
    labels: object        # torch float32 [P, 6] normalised
    width: int
    height: int

    @property
    def size(self) -> int:
        return int(self.labels.shape[0])


def training_pairs(images: int, *, size: int = 512, subset_size: int = 31, subset_stride: int = 8, seed: int = 0,
                   device: int = 0, translation: float = 20.0, strain: float = 0.05,
                   rotation_deg: float = 3.0) -> TrainingSet:
    """Subset pairs generated by the engine: speckle under random affine
    warps, labelled by IC-GN converged from the imposed warp (status 1 only)."""
    torch = _torch()
    from . import synthetic
    from .native_backend import ICGNWGPU

    lib = _native.load()
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda", device)
    half = size // 2
    refs = torch.empty(images, half, half, dtype=torch.uint8, device=dev)
    tgts = torch.empty_like(refs)
    idx_all, cen_all, lab_all = [], [], []
    with ICGNWGPU(subset_size=subset_size, subset_stride=subset_stride, outlier_policy="disabled",
                  device=device) as engine:
        for k in range(images):
            ref, sp = synthetic.reference_image(size, size, seed=seed * 100003 + 2 * k, device=f"cuda:{device}")
            t, G = random_warp(rng, translation=translation, strain=strain, rotation_deg=rotation_deg)
            c = 0.5 * (size - 1)

            def field(X, Y, t=t, G=G, c=c):
                return (t[0] + G[0, 0] * (X - c) + G[0, 1] * (Y - c), t[1] + G[1, 0] * (X - c) + G[1, 1] * (Y - c))

            tgt = synthetic.deformed_image(sp, field, noise_seed=seed * 100003 + 2 * k + 1, device=f"cuda:{device}")
            engine.set_reference(ref)
            gh, gw = engine.grid_height, engine.grid_width
            cx, cy = synthetic.subset_centres(size, size, subset_size, subset_stride)
            truth = np.zeros((gh, gw, 6), np.float32)
            u, v = field(cx, cy)
            truth[..., 0], truth[..., 3] = u, v
            truth[..., 1], truth[..., 2], truth[..., 4], truth[..., 5] = G[0, 0], G[0, 1], G[1, 0], G[1, 1]
            result = engine.register_seeded(tgt, truth, np.ones((gh, gw), bool))
            ok = np.asarray(result.status) == 1
            r_dev = torch.from_numpy(ref).to(dev)
            t_dev = torch.from_numpy(tgt).to(dev)
            _call(lib, "gbdic_reduce_half", _ptr(r_dev), size, size, _ptr(refs[k]), None)
            _call(lib, "gbdic_reduce_half", _ptr(t_dev), size, size, _ptr(tgts[k]), None)
            idx_all.append(np.full(int(ok.sum()), k, np.int32))
            cen_all.append(np.stack([cx[ok] / 2.0, cy[ok] / 2.0], -1).astype(np.float32))
            lab_all.append((np.asarray(result.parameters)[ok] * NORMALISATION).astype(np.float32))
    torch.cuda.synchronize(dev)
    ptr = lambda t: torch.tensor([t[i].data_ptr() for i in range(images)], dtype=torch.int64, device=dev)  # noqa: E731
    return TrainingSet(refs, tgts, ptr(refs), ptr(tgts), torch.from_numpy(np.concatenate(idx_all)).to(dev),
                       torch.from_numpy(np.concatenate(cen_all)).to(dev), torch.from_numpy(np.concatenate(lab_all)).to(dev),
                       half, half)


def train(net: SeedNet, data: TrainingSet, *, steps: int, lr: float = 2e-3, seed: int = 0,
          log_every: int = 0) -> list[float]:
    """Adam on shuffled mini-batches of `data`; returns the loss of every step."""
    torch = _torch()
    g = torch.Generator(device=net.device).manual_seed(seed)
    B = net.B
    losses = []
    target = torch.zeros(B, OUTPUTS, device=net.device)
    idx = torch.empty(B, dtype=torch.int32, device=net.device)
    cen = torch.empty(B, 2, device=net.device)
    order = torch.randperm(data.size, generator=g, device=net.device)
    cursor = 0
    for step in range(steps):
        if cursor + B > data.size:
            order = torch.randperm(data.size, generator=g, device=net.device)
            cursor = 0
        pick = order[cursor:cursor + B]
        cursor += B
        idx.copy_(data.image_index[pick])
        cen.copy_(data.centres[pick])
        target.copy_(data.labels[pick])
        net.load_patches(data.ref_ptrs, data.tgt_ptrs, idx, cen, B, data.width, data.height)
        # cosine decay
        rate = lr * 0.5 * (1 + math.cos(math.pi * step / max(1, steps)))
        net.forward()
        net.loss_and_grad(target)
        net.backward()
        net.adam_step(rate)
        if log_every and (step % log_every == 0 or step == steps - 1):
            losses.append(float(net.loss.item()))
    torch.cuda.synchronize(net.device)
    net.check_device_errors()
    return losses


def predict(net: SeedNet, refs_ptrs, tgts_ptrs, image_index, centres, width: int, height: int):
    """Normalised predictions (P x 6, numpy) for P patch centres."""
    torch = _torch()
    P = int(centres.shape[0])
    out = np.empty((P, OUTPUTS), np.float32)
    for s in range(0, P, net.B):
        n = min(net.B, P - s)
        net.load_patches(refs_ptrs, tgts_ptrs, None if image_index is None else image_index[s:s + n],
                         centres[s:s + n], n, width, height)
        net.forward()
        out[s:s + n] = net.out[:n, :OUTPUTS].cpu().numpy()
    torch.cuda.synchronize(net.device)
    return out


# ---------------------------------------------------------------- inference
def consensus_tables(nodes: int, *, trials: int = 128, seed: int = 12345):
    """Hypothesis and probe tables of the lattice consensus: 2 * trials
    single-node translations, `trials` node triples, and the probe nodes
    (all nodes up to 256, else 256 distinct ones), from a fixed seed."""
    rng = np.random.default_rng(seed)
    probes = np.arange(nodes) if nodes <= 256 else rng.choice(nodes, 256, replace=False)
    singles = rng.integers(0, nodes, 2 * trials)
    triples = rng.integers(0, nodes, (trials, 3))
    return singles.astype(np.int32), np.ascontiguousarray(triples, dtype=np.int32), np.asarray(probes, np.int32)


def fit_consensus(translations: np.ndarray, xy: np.ndarray, tables, tolerances=CONSENSUS_TOLERANCES) -> np.ndarray:
    """Affine field through lattice translations (P x 2, px) at normalised
    node coordinates xy (P x 2) by random sample consensus -- the host
    statement of gbdic_nn_consensus.  Hypotheses are single-node
    translations (likely inliers even when few predictions are right), then
    affine maps through node triples with |det| > 1e-9; the one agreeing with
    the most probe nodes within the first tolerance wins (lowest index on
    ties), and is refitted by least squares on its inliers while the
    tolerance tightens, stopping below three inliers.  Non-finite
    translations are outliers; fewer than three finite ones return the input.
    A global affine fit is what lets the next network pass displace every
    window, including those whose motion exceeded the training range."""
    singles, triples, probes = tables
    A = np.concatenate([np.ones((len(xy), 1)), xy], 1)
    finite = np.isfinite(translations).all(1)
    if finite.sum() < 3:
        return translations
    hyp = []
    for j in singles:
        if finite[j]:
            hyp.append(np.stack([translations[j], np.zeros(2), np.zeros(2)]))
    for t in triples:
        sub = A[t]
        if finite[t].all() and abs(np.linalg.det(sub)) > 1e-9:
            hyp.append(np.linalg.solve(sub, translations[t]))
    if not hyp:
        return translations
    coef = np.stack(hyp)
    probe = probes[finite[probes]]
    # scoring in FP32 squared distances, as on the device
    c32 = coef.astype(np.float32)
    x, y = xy[probe, 0].astype(np.float32)[None], xy[probe, 1].astype(np.float32)[None]
    t = translations[probe].astype(np.float32)
    du = c32[:, 0, 0:1] + c32[:, 1, 0:1] * x + c32[:, 2, 0:1] * y - t[None, :, 0]
    dv = c32[:, 0, 1:2] + c32[:, 1, 1:2] * x + c32[:, 2, 1:2] * y - t[None, :, 1]
    tol2 = np.float32(tolerances[0]) * np.float32(tolerances[0])
    fit_coef = coef[int(np.argmax((du * du + dv * dv <= tol2).sum(1)))]
    A32, t32 = A.astype(np.float32), np.where(finite[:, None], translations, 0.0).astype(np.float32)
    for tol in tolerances:
        d = A32 @ fit_coef.astype(np.float32) - t32
        best = finite & ((d * d).sum(1) <= np.float32(tol) * np.float32(tol))
        if best.sum() < 3:
            break
        fit_coef, *_ = np.linalg.lstsq(A[best], translations[best], rcond=None)
    return A @ fit_coef


class HalfResolutionShift:
    """Global translation of a frame by GPU phase correlation of a 256-pixel
    window at the centre of its half-resolution level (a 512-pixel region of
    the frame; the shift is resolved to 2 frame pixels), the computation of
    FourierInitializer.estimate (fourier.py:59-111) run in stream order on
    the device without host synchronisation (gbdic_fourier_shift_device).
    The learned seeder removes it before its first network pass; a plain
    pyramid can take it as its global seed."""

    def __init__(self, width: int, height: int, *, device: int = 0) -> None:
        torch = _torch()
        self.W, self.H = int(width), int(height)
        self.lib = _native.load()
        self.device = torch.device("cuda", device)
        self.tgt_half = torch.empty(self.H // 2, self.W // 2, dtype=torch.uint8, device=self.device)
        self.fourier = None
        self.window = None

    def set_reference_half(self, half: np.ndarray) -> None:
        """The reference's half-resolution level (host bytes)."""
        from .fourier import FourierInitializer

        self.close()
        hh, hw = half.shape
        side = min(256, hh, hw)
        x0, y0 = (hw - side) // 2, (hh - side) // 2
        try:
            self.fourier = FourierInitializer(np.ascontiguousarray(half[y0:y0 + side, x0:x0 + side]),
                                              device=self.device.index or 0)
        except ValueError:
            self.fourier = None
        if self.fourier is not None:
            win = self.fourier.window
            self.window = (x0 + win["x"], y0 + win["y"])

    def set_reference_frame(self, frame) -> None:
        """The reference as a device frame (uint8 H x W)."""
        torch = _torch()
        half = torch.empty_like(self.tgt_half)
        _call(self.lib, "gbdic_reduce_half", _ptr(frame), self.W, self.H, _ptr(half), None)
        torch.cuda.synchronize(self.device)
        self.set_reference_half(half.cpu().numpy())

    @property
    def available(self) -> bool:
        return self.fourier is not None

    def write(self, frame_half_ptr: int, rows_ptr: int, count: int, pitch: int, multiplier: float, stream) -> None:
        """Writes dx * multiplier and dy * multiplier (dx, dy in half-level
        pixels) into rows[i * pitch] and rows[i * pitch + 3], i < count; zero
        when the estimate is not accepted."""
        fx, fy = self.window
        code = self.lib.gbdic_fourier_shift_device(
            self.fourier._handle, C.c_void_p(frame_half_ptr), self.W // 2, self.H // 2, fx, fy,
            C.c_float(multiplier), C.c_void_p(rows_ptr), count, pitch, stream)
        _native.check(code, self.lib.gbdic_fourier_last_error(self.fourier._handle))

    def shift_of(self, frame, stream=None) -> tuple[float, float]:
        """(dx, dy) in frame pixels of device frame `frame` (uint8 H x W),
        computed on `stream` (a torch.cuda.Stream; None: the current one),
        which is synchronised to read it; (0, 0) when not accepted."""
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        handle = C.c_void_p(s.cuda_stream)
        with torch.cuda.stream(s):
            rows = torch.zeros(8, device=self.device)
        _call(self.lib, "gbdic_reduce_half", _ptr(frame), self.W, self.H, _ptr(self.tgt_half), handle)
        if self.available:
            self.write(self.tgt_half.data_ptr(), rows.data_ptr(), 1, 8, 2.0, handle)
        s.synchronize()
        values = rows.cpu()
        return float(values[0]), float(values[3])

    def close(self) -> None:
        if self.fourier is not None:
            self.fourier.close()
        self.fourier = None
        self.window = None


class LearnedSeeder:
    """Learned-seed registration for one fixed reference on the single-scale
    engine: the global translation by GPU phase correlation, network
    proposals on a subset lattice (two passes with an affine consensus
    between them), IC-GN on the lattice nodes from those proposals (with
    `refine_nodes`), every subset seeded by interpolation of the node warps,
    seeded IC-GN, and ZNCC reseeding of failed or low-ZNCC subsets.  Every
    step runs on the device in stream order, without host round trips; with
    `graph` (the default) register_device captures that sequence once as a
    CUDA graph (frame read from a fixed buffer) and replays it per frame.
    With `listed` (the default) the node solve, the reseeding search and the
    reseeding solve run over compact subset lists (the nodes; the subsets
    the selection picked, counted on the device) instead of masked
    full-grid launches, with `list_lanes` lanes per subset (these few
    subsets run latency-bound: more lanes shorten each iteration; the fields
    are those of masked full-grid solves at that lane count, bit for bit)."""

    def __init__(self, engine, net: SeedNet, *, step: int = 4, reseed_radius: int = 10, passes: int = 2,
                 global_alignment: bool = True, refine_nodes: bool = True, graph: bool = True,
                 listed: bool = True, list_lanes: int = 128) -> None:
        torch = _torch()
        if not engine._reference_ready or engine.motion_model != "affine":
            raise ValueError("LearnedSeeder needs an affine engine with a prepared reference")
        self.engine, self.net, self.step, self.radius = engine, net, int(step), int(reseed_radius)
        self.passes = max(1, int(passes))
        self.global_alignment = bool(global_alignment)
        self.refine_nodes = bool(refine_nodes)
        self.lib = _native.load()
        dev = net.device
        W, H = engine.width, engine.height
        self.W, self.H, self.gw, self.gh = W, H, engine.grid_width, engine.grid_height
        self.lw, self.lh = (self.gw + self.step - 1) // self.step, (self.gh + self.step - 1) // self.step
        self.lattice = self.lw * self.lh
        S, s = engine.subset_size, engine.subset_stride
        gy, gx = np.mgrid[0:self.lh, 0:self.lw] * self.step
        cx = gx * s + 0.5 * (S - 1)
        cy = gy * s + 0.5 * (S - 1)
        self.centres = torch.from_numpy(np.stack([cx.ravel() / 2.0, cy.ravel() / 2.0], -1).astype(np.float32)).to(dev)
        self.node_xy = np.stack([cx.ravel(), cy.ravel()], -1).astype(np.float64)
        self.ref_half = torch.empty(H // 2, W // 2, dtype=torch.uint8, device=dev)
        self.tgt_half = torch.empty_like(self.ref_half)
        self.ref_ptrs = torch.tensor([self.ref_half.data_ptr()], dtype=torch.int64, device=dev)
        self.tgt_ptrs = torch.tensor([self.tgt_half.data_ptr()], dtype=torch.int64, device=dev)
        self._ref_full = torch.empty(H, W, dtype=torch.uint8, device=dev)
        self.global_shift = HalfResolutionShift(W, H, device=dev.index or 0)
        usable = np.asarray(engine.reference_valid, dtype=bool)
        if engine.roi is not None:
            usable = usable & np.asarray(engine.roi.selected, dtype=bool)
        self.usable = torch.from_numpy(np.array(usable, dtype=bool).ravel()).to(dev)
        self.pred = torch.zeros(self.lattice, OUT_PAD, device=dev)
        self.base = torch.zeros(self.lattice, OUT_PAD, device=dev)
        self.seeds = torch.zeros(self.gh * self.gw * 8, device=dev)
        self.active = torch.zeros(self.gh * self.gw, dtype=torch.int32, device=dev)
        self.state = torch.zeros(self.gh * self.gw * 8, device=dev)
        self.mask = torch.zeros(self.gh * self.gw, dtype=torch.uint8, device=dev)
        # Inference copy of the network sized to the whole lattice: one
        # forward per pass.
        self.inet = SeedNet(batch=_pad(self.lattice, 128), device=net.device.index or 0, split_forward=True)
        self.inet.load_state_dict(net.state_dict())
        self.inet.use_direct_first_layer()
        self.batches = 1
        # One non-default stream carries the network, the engine's kernels and
        # the mask arithmetic in order (a NULL stream would select the
        # engine's own stream).
        self.stream = torch.cuda.Stream(device=dev)
        self._handle = C.c_void_p(self.stream.cuda_stream)
        # Consensus tables (fixed seed): single-node and triple hypotheses and
        # the probe nodes that score them; node coordinates centred and in
        # units of 1000 px.
        singles, triples, probes = consensus_tables(self.lattice)
        xy = (self.node_xy - self.node_xy.mean(0)) / 1000.0
        self._xy = torch.from_numpy(np.ascontiguousarray(xy, dtype=np.float32)).to(dev)
        self._singles = torch.from_numpy(singles.astype(np.int32)).to(dev)
        self._triples = torch.from_numpy(np.ascontiguousarray(triples, dtype=np.int32)).to(dev)
        self._probes = torch.from_numpy(np.asarray(probes, dtype=np.int32)).to(dev)
        self._tolerances = np.array(CONSENSUS_TOLERANCES, np.float32)
        self._usable8 = self.usable.to(torch.uint8)
        self._retry = torch.empty_like(self.state)
        node_active = np.zeros((self.gh, self.gw), np.int32)
        node_active[::self.step, ::self.step] = 1
        self._node_active = torch.from_numpy(node_active.ravel()).to(dev)
        self.listed = bool(listed)
        if list_lanes not in (0, 16, 32, 64, 128):
            raise ValueError("list_lanes must be 0 (the engine's), 16, 32, 64 or 128")
        self.list_lanes = int(list_lanes)
        self._node_list = torch.from_numpy(np.flatnonzero(node_active.ravel()).astype(np.int32)).to(dev)
        self._reseed_list = torch.zeros(self.gh * self.gw, dtype=torch.int32, device=dev)
        self._shifted = False
        self.reseed_count = torch.zeros(1, dtype=torch.int32, device=dev)
        self.graph = bool(graph)
        self._graph = None       # captured frame sequence, and what it was captured for
        self._graph_key = None
        self._graph_frame = None  # the fixed frame buffer the graph reads
        self._marks = None        # (stage, CUDA event) pairs while stage_times runs

    def set_reference_image(self, reference: np.ndarray) -> None:
        """Half-resolution reference for the network (the engine keeps its own),
        and the GPU phase correlation that removes the global translation
        before the first network pass: a 256-pixel window at the centre of the
        half-resolution reference (a 512-pixel region of the frame; the shift
        is resolved to 4 frame pixels, well inside the network's range)."""
        torch = _torch()

        self._drop_graph()
        self._ref_full.copy_(torch.from_numpy(np.ascontiguousarray(reference, dtype=np.uint8)))
        _call(self.lib, "gbdic_reduce_half", _ptr(self._ref_full), self.W, self.H, _ptr(self.ref_half), None)
        self.global_shift.close()
        if self.global_alignment:
            self.global_shift.set_reference_half(self.ref_half.cpu().numpy())
    def propose(self, frame) -> None:
        """Network proposals for device frame `frame` (uint8 H x W) -> self.seeds
        (on self.stream)."""
        torch = _torch()
        net = self.net
        stream = self._handle
        self.stream.wait_stream(torch.cuda.current_stream(net.device))
        with torch.cuda.stream(self.stream):
            self._propose(frame, stream)
        torch.cuda.current_stream(net.device).wait_stream(self.stream)

    def _network_pass(self, out, shift, stream) -> None:
        net = self.inet
        # level-1 pixels per normalised translation unit
        scale = C.c_float(TRANSLATION_SCALE / 2.0)
        for b in range(self.batches):
            s0 = b * net.B
            n = min(net.B, self.lattice - s0)
            _call(self.lib, "gbdic_nn_patches", _ptr(self.ref_ptrs), _ptr(self.tgt_ptrs), None,
                  C.c_void_p(self.centres.data_ptr() + 8 * s0), n, self.W // 2, self.H // 2, _ptr(net.x0),
                  None if shift is None else C.c_void_p(shift.data_ptr() + 4 * OUT_PAD * s0), OUT_PAD, scale, stream)
            net.forward(stream)
            _native_copy(out, s0, net.out, n)  # on the current stream, ordered with `stream`

    def consensus(self, translations: np.ndarray) -> np.ndarray:
        """Host restatement of the device consensus for inspection (see
        fit_consensus)."""
        xy = self._xy.cpu().numpy().astype(np.float64)
        tables = (self._singles.cpu().numpy(), self._triples.cpu().numpy(), self._probes.cpu().numpy())
        return fit_consensus(translations, xy, tables)

    def _consensus_device(self, stream) -> None:
        """self.base (columns 0, 3) <- the fitted field through the totals
        self.base + self.pred, on the device."""
        _call(self.lib, "gbdic_nn_consensus", _ptr(self.pred), _ptr(self.base), OUT_PAD, self.lattice, _ptr(self._xy),
              _ptr(self._singles), int(self._singles.numel()), _ptr(self._triples), int(self._triples.shape[0]),
              _ptr(self._probes), int(self._probes.numel()), self._tolerances.ctypes.data_as(C.c_void_p),
              len(self._tolerances), C.c_float(TRANSLATION_SCALE), stream)

    def _propose(self, frame, stream) -> None:
        # Pass 1 on co-located windows (displaced by the global phase
        # correlation); between passes a robust affine fit of the lattice
        # translations displaces every target window, and the next pass
        # predicts the residual warp around it.  Everything stays on the
        # device, in stream order.
        _call(self.lib, "gbdic_reduce_half", _ptr(frame), self.W, self.H, _ptr(self.tgt_half), stream)
        shift = None
        if self.global_shift.available:
            self.global_shift.write(self.tgt_half.data_ptr(), self.base.data_ptr(), self.lattice, OUT_PAD,
                                    2.0 / TRANSLATION_SCALE, stream)
            shift = self.base
        self._mark("half frame + shift")
        for p in range(self.passes):
            self._network_pass(self.pred, shift, stream)
            self._mark(f"network pass {p + 1}")
            if p == self.passes - 1:
                break
            if shift is None:
                self.base.zero_()
            self._consensus_device(stream)
            self._mark("consensus")
            shift = self.base
        self._shifted = shift is not None
        self._lattice_seeds(stream)
        self._mark("lattice seeds")

    def _lattice_seeds(self, stream) -> None:
        _call(self.lib, "gbdic_nn_lattice_seeds", _ptr(self.pred), _ptr(self.base) if self._shifted else None,
              OUT_PAD, self.lw, self.lh, self.step, self.gw, self.gh, self.engine.subset_stride,
              C.c_float(TRANSLATION_SCALE), C.c_float(GRADIENT_SCALE), _ptr(self.seeds), _ptr(self.active), stream)

    def register_device(self, frame, *, reseed: bool = True, counts: bool = True) -> dict:
        """Learned-seed registration of a device frame into self.state (on
        self.stream; callers synchronise or wait on it).  The number of
        reseeded subsets stays in self.reseed_count (device); with `counts`
        it is also returned (one host synchronisation), else None.

        With `graph`, the first call for a given engine configuration runs
        the sequence once directly, then captures it as a CUDA graph that
        reads the frame from a fixed device buffer; later calls copy the
        frame there and replay the graph.  The graph is captured again when
        the reference (the seeder's or the engine's), the engine's solver
        settings or `reseed` change."""
        torch = _torch()
        self.stream.wait_stream(torch.cuda.current_stream(self.net.device))
        if self.graph:
            key = (bool(reseed), tuple(sorted(self.engine._config.items())), self.engine.solver,
                   self.engine.reference_generation, tuple(frame.shape), frame.dtype)
            if self._graph is None or self._graph_key != key:
                self._capture(frame, bool(reseed), key)
            with torch.cuda.stream(self.stream):
                self._graph_frame.copy_(frame)
                self._graph.replay()
        else:
            with torch.cuda.stream(self.stream):
                self._register(frame, reseed, self._handle)
        torch.cuda.current_stream(self.net.device).wait_stream(self.stream)
        return {"reseeded": int(self.reseed_count.item()) if counts and reseed else (0 if counts else None)}

    def stage_times(self, frame, *, reseed: bool = True) -> dict[str, float]:
        """One frame through the direct sequence with CUDA events between its
        stages (on self.stream); returns milliseconds per stage (half-resolution
        frame and global shift, each network pass, the consensus, the lattice
        seeds, the node solve, the node rows and seeds, the full solve, the
        reseeding) and their total.  Leaves self.state as register_device
        would."""
        torch = _torch()
        self._marks = []
        self.stream.wait_stream(torch.cuda.current_stream(self.net.device))
        with torch.cuda.stream(self.stream):
            self._mark("start")
            self._register(frame, reseed, self._handle)
        marks, self._marks = self._marks, None
        self.stream.synchronize()
        out: dict[str, float] = {}
        for (_, a), (name, b) in zip(marks, marks[1:], strict=False):
            out[name] = out.get(name, 0.0) + a.elapsed_time(b)
        out["total"] = marks[0][1].elapsed_time(marks[-1][1])
        return out

    def _mark(self, name: str) -> None:
        if self._marks is None:
            return
        torch = _torch()
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(self.stream)
        self._marks.append((name, ev))

    def _capture(self, frame, reseed: bool, key) -> None:
        torch = _torch()
        self._drop_graph()
        self._graph_frame = torch.empty_like(frame)
        with torch.cuda.stream(self.stream):
            self._graph_frame.copy_(frame)
            # one direct run: lazy set-up (kernel attributes, occupancy
            # queries, tensor-map entry points) stays out of the capture
            self._register(self._graph_frame, reseed, self._handle)
        self.stream.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=self.stream):
            self._register(self._graph_frame, reseed, self._handle)
        self._graph, self._graph_key = graph, key

    def _drop_graph(self) -> None:
        self._graph = None
        self._graph_key = None

    def _register(self, frame, reseed: bool, stream) -> None:
        eng = self.engine
        cfg = C.byref(eng._cfg(eng._config))
        self._propose(frame, stream)
        if self.refine_nodes:
            # IC-GN on the lattice nodes alone (one subset in step^2) from the
            # network's proposals; their solved warps replace the network rows
            # and the interpolated seeds of every subset come from them.  The
            # full solve then reuses the node solve's B-spline coefficients.
            # The node solve is latency-bound (a few hundred subsets), so its
            # iterations are capped at NODE_ITERATIONS: a node that needs more
            # keeps the network's warp.
            node_cfg = eng._cfg(eng._config)
            node_cfg.iterations = min(int(node_cfg.iterations), NODE_ITERATIONS)
            if self.listed:
                _call_engine(eng, "gbdic_solve_listed_device", _ptr(frame), _ptr(self.seeds), _ptr(self._node_active),
                             _ptr(self._node_list), int(self._node_list.numel()), None, 1, self.list_lanes,
                             C.byref(node_cfg), _ptr(self.state), stream)
            else:
                _call_engine(eng, "gbdic_register_seeded_device", _ptr(frame), _ptr(self.seeds),
                             _ptr(self._node_active), C.byref(node_cfg), _ptr(self.state), stream)
            self._mark("node solve")
            _call(self.lib, "gbdic_nn_node_rows", _ptr(self.state), self.gw, self.gh, self.step, self.lw, self.lh,
                  _ptr(self.pred), _ptr(self.base) if self._shifted else None, OUT_PAD, C.c_float(TRANSLATION_SCALE),
                  C.c_float(GRADIENT_SCALE), stream)
            self._lattice_seeds(stream)
            self._mark("node rows + seeds")
            _call_engine(eng, "gbdic_resolve_seeded_device", _ptr(frame), _ptr(self.seeds), _ptr(self.active), cfg,
                         _ptr(self.state), stream)
        else:
            _call_engine(eng, "gbdic_register_seeded_device", _ptr(frame), _ptr(self.seeds), _ptr(self.active), cfg,
                         _ptr(self.state), stream)
        self._mark("full solve")
        if not reseed:
            return
        # Not converged (0) or converged below the ZNCC threshold (-2): ZNCC
        # search around the current seed, a second solve of those subsets
        # only, and their rows merged back.  Windows pushed off the image (-1)
        # cannot be rescued by a search.  No host round trip: an empty
        # selection costs three near-empty launches.
        count = self.gh * self.gw
        if self.listed:
            _call(self.lib, "gbdic_nn_reseed_select_list", _ptr(self.state), 8, _ptr(self._usable8), count,
                  _ptr(self.mask), _ptr(self.active), _ptr(self.reseed_count), _ptr(self._reseed_list), stream)
            _call_engine(eng, "gbdic_search_seeds_listed_device", _ptr(frame), _ptr(self.seeds), _ptr(self.active),
                         _ptr(self._reseed_list), _ptr(self.reseed_count), self.radius, 1, stream)
            _call_engine(eng, "gbdic_solve_listed_device", _ptr(frame), _ptr(self.seeds), _ptr(self.active),
                         _ptr(self._reseed_list), count, _ptr(self.reseed_count), 0, self.list_lanes, cfg,
                         _ptr(self._retry), stream)
        else:
            _call(self.lib, "gbdic_nn_reseed_select", _ptr(self.state), 8, _ptr(self._usable8), count,
                  _ptr(self.mask), _ptr(self.active), _ptr(self.reseed_count), stream)
            _call_engine(eng, "gbdic_search_seeds_device", _ptr(frame), _ptr(self.seeds), _ptr(self.active),
                         _ptr(self.mask), self.radius, 1, stream)
            _call_engine(eng, "gbdic_resolve_seeded_device", _ptr(frame), _ptr(self.seeds), _ptr(self.active), cfg,
                         _ptr(self._retry), stream)
        _call(self.lib, "gbdic_nn_merge_rows", _ptr(self._retry), _ptr(self.mask), count, 8, _ptr(self.state), stream)
        self._mark("reseeding")


def _native_copy(dst, row0: int, src, n: int) -> None:
    dst[row0:row0 + n].copy_(src[:n])


def _call_engine(engine, name: str, *args) -> None:
    code = getattr(engine._lib, name)(engine._handle, *args)
    engine._check(code)


def timed(fn, *args, repeats: int = 1, **kwargs) -> float:
    torch = _torch()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(repeats):
        fn(*args, **kwargs)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / repeats
