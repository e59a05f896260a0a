"""GPU reference preparation against the float64 oracle (_reference_arrays).

Tolerances are the reference's own for its GPU preparation twin
(DIC/LucasKanadeICGN/python/tests/test_gpu_reference.py:107-124): plane
3e-4 + 3e-6|b|; metadata J^T f 0.1 + 1e-4|b|, sum J 0.003 + 1e-4|b|, others
0.001 + 1e-5|b|; inverse 5e-9 + 5e-4|b|; identical validity.  The quadratic
12x12 inverse (factorised in binary64 from binary32 moments) is held to the
same relative bound on its well-conditioned entries.
"""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPU, synthetic
from oracle import reference_prep as rp
from quadratic_prep import check_quadratic_preparation

pytestmark = pytest.mark.gpu

W, H = 99, 97


def _texture():
    i = np.arange(W * H)
    return ((i * 7 + i * i + (i // W) * 17) % 251).astype(np.uint8).reshape(H, W)


def _speckle():
    ref, _ = synthetic.reference_image(W, H, seed=33, device="cpu")
    return ref


CASES = [
    ("affine", "bspline", 16, 16),
    ("affine", "bspline", 17, 8),
    ("affine", "linear", 24, 12),
    ("affine", "cubic", 31, 16),
    ("translation", "bspline", 8, 8),
    ("translation", "linear", 10, 5),
    ("translation", "cubic", 15, 15),
    ("affine", "bspline", 33, 33),
]


def _compare(image, model, interp, size, stride, weighting="uniform", sigma=None):
    plane, inverse, metadata = rp.reference_arrays(image, interpolation=interp, motion_model=model,
                                                   subset_size=size, subset_stride=stride,
                                                   spatial_weighting=weighting, gaussian_sigma=sigma)
    with ICGNWGPU(motion_model=model, interpolation=interp, subset_size=size, subset_stride=stride,
                  spatial_weighting=weighting, gaussian_sigma=sigma) as engine:
        info = engine.set_reference(image)
        g_plane, g_inverse, g_meta = engine.export_reference()
        valid = engine.reference_valid
    n = 12 if model == "quadratic" else 6
    ms = 28 if model == "quadratic" else 16
    err = np.abs(g_plane - plane)
    assert np.all(err <= 3e-4 + 3e-6 * np.abs(plane)), float(err.max())
    meta, gm = metadata.reshape(-1, ms), g_meta.reshape(-1, ms)
    np.testing.assert_array_equal(gm[:, 1], meta[:, 1])
    np.testing.assert_array_equal(valid.ravel(), meta[:, 1] > 0.5)
    ok = meta[:, 1] > 0.5
    for comp in range(ms):
        a, b = gm[ok, comp], meta[ok, comp]
        if 2 <= comp < 2 + n:
            tol = 0.1 + 1e-4 * np.abs(b)
        elif 2 + n <= comp < 2 + 2 * n:
            tol = 0.003 + 1e-4 * np.abs(b)
        else:
            tol = 0.001 + 1e-5 * np.abs(b)
        assert np.all(np.abs(a - b) <= tol), (comp, float(np.abs(a - b).max()))
    inv, ginv = inverse.reshape(-1, n * n)[ok], g_inverse.reshape(-1, n * n)[ok]
    scale = np.abs(inv).max(axis=1, keepdims=True)
    assert np.all(np.abs(ginv - inv) <= 5e-9 + 5e-4 * np.maximum(np.abs(inv), 1e-3 * scale))
    assert info.grid == (1 + (W - size) // stride, 1 + (H - size) // stride)


@pytest.mark.parametrize("model,interp,size,stride", CASES)
def test_gpu_preparation_matches_float64_oracle(model, interp, size, stride):
    _compare(_texture(), model, interp, size, stride)


@pytest.mark.parametrize("model", ["affine", "quadratic"])
def test_gpu_preparation_on_speckle(model):
    _compare(_speckle(), model, "bspline", 21, 10)


# Overlapping quadratic windows are prepared by window rows (shared column
# sums; Gaussian weights as the outer product of their axis factors), tiled
# grids by the per-window sums.  Both against the float64 oracle, the
# second-order moments stage by stage.
@pytest.mark.parametrize("size,stride,weighting", [
    (21, 10, "uniform"),    # row path, 8 windows in one row segment
    (25, 4, "uniform"),     # row path, 16 windows per row segment
    (24, 6, "uniform"),     # row path, even size: half-integer window coordinates
    (61, 15, "uniform"),    # row path, 256 columns per CTA (the widest segment)
    (21, 7, "gaussian"),    # row path, weighted
    (24, 6, "gaussian"),    # row path, weighted, even size
    (21, 21, "uniform"),    # per-window path (tiled)
    (21, 21, "gaussian"),   # per-window path (tiled, weighted)
])
def test_gpu_quadratic_preparation_paths(size, stride, weighting):
    ok = check_quadratic_preparation(_speckle(), size, stride, weighting=weighting,
                                     sigma=5.0 if weighting == "gaussian" else None)
    assert ok.mean() > 0.9


def test_gpu_preparation_gaussian_weights():
    _compare(_speckle(), "affine", "bspline", 21, 7, weighting="gaussian", sigma=5.0)


def test_flat_reference_invalid_and_finite():
    flat = np.full((48, 64), 91, dtype=np.uint8)
    with ICGNWGPU(subset_size=13, subset_stride=13) as engine:
        engine.set_reference(flat)
        plane, inverse, metadata = engine.export_reference()
        assert not engine.reference_valid.any()
    assert np.isfinite(plane).all() and np.isfinite(inverse).all() and np.isfinite(metadata).all()
    assert not inverse.any()
