"""Checks of the GPU quadratic reference preparation against the float64
restatement of _reference_arrays, shared by the preparation tests.

The reference's GPU-preparation tolerances (test_gpu_reference.py:107-124)
exist for its first-order models only (its GPU preparation rejects the
quadratic model, reference.wgsl:22).  The plane, validity, the first-order
rows and the 12x12 inverse are held to them; the six second-order rows of
J^T f and sum J, whose window weights reach (S-1)^2/4 and whose sums cancel,
are checked stage by stage instead: the binary32 sums against float64 sums
over the same (GPU) plane within 1e-6 of the absolute sum of their terms,
the plane itself against the float64 oracle as above.
"""

from __future__ import annotations

import numpy as np

from live_dic_gb300 import ICGNWGPU
from oracle import reference_prep as rp


def window_weights(size: int, weighting: str, sigma: float | None) -> np.ndarray:
    """The engine's binary32 integration weights of one window."""
    c = np.arange(size) - 0.5 * (size - 1)
    ly, lx = np.meshgrid(c, c, indexing="ij")
    if weighting == "gaussian":
        return np.exp(-0.5 * (lx * lx + ly * ly) / (sigma * sigma)).astype(np.float32)
    return np.ones((size, size), np.float32)


def float64_moments(plane: np.ndarray, width: int, height: int, size: int, stride: int,
                    weights: np.ndarray | None = None):
    """J^T f and sum J of the 12 quadratic Jacobian columns, summed in
    float64 over a given reference plane (f, gx, gy, 0) with the window
    weights, with the absolute sums of their terms."""
    p = plane.reshape(height, width, 4).astype(np.float64)
    gw, gh = 1 + (width - size) // stride, 1 + (height - size) // stride
    w = (np.ones((size, size)) if weights is None else weights.astype(np.float64)).reshape(-1)
    c = np.arange(size) - 0.5 * (size - 1)
    ly, lx = np.meshgrid(c, c, indexing="ij")
    mono = np.stack([np.ones_like(lx), lx, ly, 0.5 * lx * lx, lx * ly, 0.5 * ly * ly]).reshape(6, -1)
    order = [0, 1, 2, 6, 7, 8, 3, 4, 5, 9, 10, 11]   # [gx*m0..2, gy*m0..2, gx*m3..5, gy*m3..5]
    jtf = np.zeros((gh * gw, 12))
    sj = np.zeros_like(jtf)
    jtf_abs = np.zeros_like(jtf)
    sj_abs = np.zeros_like(jtf)
    win = np.lib.stride_tricks.sliding_window_view
    for gy in range(gh):
        rows = win(p[gy * stride: gy * stride + size], (size, size, 4))[0, ::stride, 0][:gw]
        rows = rows.reshape(gw, size * size, 4)
        mean = (rows[..., 0] * w).sum(axis=1, keepdims=True) / w.sum()
        f = rows[..., 0] - mean
        cols = np.concatenate([rows[..., 1:2] * mono.T[None], rows[..., 2:3] * mono.T[None]], -1)[..., order]
        cols = cols * w[None, :, None]
        sl = slice(gy * gw, (gy + 1) * gw)
        jtf[sl] = np.einsum("gpk,gp->gk", cols, f)
        jtf_abs[sl] = np.einsum("gpk,gp->gk", np.abs(cols), np.abs(f))
        sj[sl] = cols.sum(axis=1)
        sj_abs[sl] = np.abs(cols).sum(axis=1)
    return jtf, sj, jtf_abs, sj_abs


def check_quadratic_preparation(image: np.ndarray, size: int, stride: int, weighting: str = "uniform",
                                sigma: float | None = None) -> np.ndarray:
    """Run the engine's quadratic preparation of `image` and check it;
    returns the oracle's validity per window."""
    height, width = image.shape
    plane, inverse, metadata = rp.reference_arrays(image, motion_model="quadratic", subset_size=size,
                                                   subset_stride=stride, spatial_weighting=weighting,
                                                   gaussian_sigma=sigma)
    with ICGNWGPU(motion_model="quadratic", subset_size=size, subset_stride=stride, spatial_weighting=weighting,
                  gaussian_sigma=sigma) as engine:
        engine.set_reference(image)
        g_plane, g_inverse, g_meta = engine.export_reference()
        valid = engine.reference_valid
    n, ms = 12, 28
    err = np.abs(g_plane - plane)
    assert np.all(err <= 3e-4 + 3e-6 * np.abs(plane)), float(err.max())
    meta, gm = metadata.reshape(-1, ms), g_meta.reshape(-1, ms)
    np.testing.assert_array_equal(gm[:, 1], meta[:, 1])
    np.testing.assert_array_equal(valid.ravel(), meta[:, 1] > 0.5)
    ok = meta[:, 1] > 0.5
    second_order = set(range(2 + 6, 2 + n)) | set(range(2 + n + 6, 2 + 2 * n))
    for comp in range(ms):
        if comp in second_order:
            continue
        a, b = gm[ok, comp], meta[ok, comp]
        if 2 <= comp < 2 + n:
            tol = 0.1 + 1e-4 * np.abs(b)
        elif 2 + n <= comp < 2 + 2 * n:
            tol = 0.003 + 1e-4 * np.abs(b)
        else:
            tol = 0.001 + 1e-5 * np.abs(b)
        assert np.all(np.abs(a - b) <= tol), (comp, float(np.abs(a - b).max()))
    jtf, sj, jtf_abs, sj_abs = float64_moments(g_plane, width, height, size, stride,
                                               window_weights(size, weighting, sigma))
    for k in range(6, 12):
        e = np.abs(gm[ok, 2 + k] - jtf[ok, k])
        assert np.all(e <= 1e-6 * jtf_abs[ok, k] + 1e-3), (k, float((e / jtf_abs[ok, k]).max()))
        e = np.abs(gm[ok, 2 + n + k] - sj[ok, k])
        assert np.all(e <= 1e-6 * sj_abs[ok, k] + 1e-3), (k, float((e / sj_abs[ok, k]).max()))
    inv, ginv = inverse.reshape(-1, n * n)[ok], g_inverse.reshape(-1, n * n)[ok]
    scale = np.abs(inv).max(axis=1, keepdims=True)
    assert np.all(np.abs(ginv - inv) <= 5e-9 + 5e-4 * np.maximum(np.abs(inv), 1e-3 * scale))
    return ok
