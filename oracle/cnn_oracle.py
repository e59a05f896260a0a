"""CPU oracle of the learned seed network (TEST INFRASTRUCTURE ONLY).

A float64 NumPy restatement of the network in live_dic_gb300/learned.py
(five 3x3 stride-2 pad-1 convolutions with ReLU, channels 32-64-128-128-64,
then a linear layer), forward and backward.  `rounded=True` applies BF16
rounding (round to nearest even) at the points where the GPU path stores
BF16: the input patches, the weights, every post-ReLU activation, the output
gradient, the masked gradients dZ and the gathered / transposed operands;
products are accumulated in float64 instead of the tensor cores' FP32, so the
two agree to accumulation-order error.  `rounded=False` is the exact network,
used to check the backward formulas against central differences.
"""

from __future__ import annotations

import numpy as np

CONV_CHANNELS = ((2, 32), (32, 64), (64, 128), (128, 128), (128, 64))


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def im2col(x: np.ndarray) -> np.ndarray:
    """x (B, H, W, C) -> (B * OH * OW, 9 C), columns ordered (ky, kx, ci)."""
    B, H, W, C = x.shape
    oh, ow = (H + 1) // 2, (W + 1) // 2
    padded = np.zeros((B, H + 2, W + 2, C), x.dtype)
    padded[:, 1:H + 1, 1:W + 1] = x
    cols = []
    for ky in range(3):
        for kx in range(3):
            cols.append(padded[:, ky:ky + 2 * oh:2, kx:kx + 2 * ow:2, :])
    return np.concatenate(cols, axis=-1).reshape(B * oh * ow, 9 * C)


def col2im(cols: np.ndarray, shape) -> np.ndarray:
    """Adjoint of im2col: (B * OH * OW, 9 C) -> (B, H, W, C)."""
    B, H, W, C = shape
    oh, ow = (H + 1) // 2, (W + 1) // 2
    padded = np.zeros((B, H + 2, W + 2, C))
    cols = cols.reshape(B, oh, ow, 9, C)
    for ky in range(3):
        for kx in range(3):
            padded[:, ky:ky + 2 * oh:2, kx:kx + 2 * ow:2, :] += cols[:, :, :, ky * 3 + kx, :]
    return padded[:, 1:H + 1, 1:W + 1]


def forward(x0, weights, biases, w6, b6, *, rounded: bool = True):
    """weights[i]: (Cout, 9 Cin); w6: (6, 256).  Returns (activations, out)."""
    r = bf16 if rounded else (lambda a: np.asarray(a, np.float64))
    x = r(x0)
    acts = [x]
    for w, b in zip(weights, biases, strict=True):
        B, H, W, _ = x.shape
        z = im2col(x) @ r(w).T + b
        y = r(np.maximum(z, 0.0))
        x = y.reshape(B, (H + 1) // 2, (W + 1) // 2, -1)
        acts.append(x)
    out = x.reshape(x.shape[0], -1) @ r(w6).T + b6
    return acts, out


def loss(out: np.ndarray, target: np.ndarray) -> float:
    d = out - target
    return 0.5 * float(np.sum(d * d)) / out.shape[0]


def backward(acts, out, target, weights, w6, *, rounded: bool = True):
    """Gradients (dweights, dbiases, dw6, db6) of loss(out, target)."""
    r = bf16 if rounded else (lambda a: np.asarray(a, np.float64))
    B = out.shape[0]
    dout = (out - target) / B
    db6 = dout.sum(0)
    dout_r = r(dout)
    feats = acts[-1].reshape(B, -1)
    dw6 = dout_r.T @ feats
    dy = (dout_r @ r(w6)).reshape(acts[-1].shape)
    dws, dbs = [], []
    for i in range(len(weights) - 1, -1, -1):
        y = acts[i + 1]
        mask = y > 0
        db = np.where(mask, dy, 0.0).reshape(-1, y.shape[-1]).sum(0)
        dz = r(np.where(mask, dy, 0.0)).reshape(-1, y.shape[-1])
        cols = im2col(acts[i])
        dws.append(dz.T @ cols)
        dbs.append(db)
        if i > 0:
            dy = col2im(dz @ r(weights[i]), acts[i].shape)
    return dws[::-1], dbs[::-1], dw6, db6


def init(seed: int = 0, scale: float = 1.0):
    """Random parameters in the oracle layout (weights (Cout, 9 Cin))."""
    rng = np.random.default_rng(seed)
    weights = [rng.normal(0, scale * np.sqrt(2.0 / (9 * cin)), (cout, 9 * cin)) for cin, cout in CONV_CHANNELS]
    biases = [rng.normal(0, 0.05, cout) for _, cout in CONV_CHANNELS]
    w6 = rng.normal(0, np.sqrt(1.0 / 256), (6, 256))
    b6 = rng.normal(0, 0.05, 6)
    return weights, biases, w6, b6
