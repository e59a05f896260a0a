"""The float64 moment helper of the quadratic preparation checks
(quadratic_prep.float64_moments) against a direct per-window loop, with
uniform and Gaussian weights, odd and even window sizes (CPU)."""

from __future__ import annotations

import numpy as np
import pytest

from quadratic_prep import float64_moments, window_weights


def _direct(plane, width, height, size, stride, weights):
    p = plane.reshape(height, width, 4).astype(np.float64)
    gw, gh = 1 + (width - size) // stride, 1 + (height - size) // stride
    c = np.arange(size) - 0.5 * (size - 1)
    w = weights.astype(np.float64)
    jtf = np.zeros((gh * gw, 12))
    sj = np.zeros_like(jtf)
    for gy in range(gh):
        for gx in range(gw):
            win = p[gy * stride: gy * stride + size, gx * stride: gx * stride + size]
            f = win[..., 0] - (win[..., 0] * w).sum() / w.sum()
            k = gy * gw + gx
            y, x = np.meshgrid(c, c, indexing="ij")
            monomials = [np.ones_like(x), x, y, 0.5 * x * x, x * y, 0.5 * y * y]
            for q in range(12):
                # columns [gx m0..2, gy m0..2, gx m3..5, gy m3..5]
                grad = win[..., 1] if q in (0, 1, 2, 6, 7, 8) else win[..., 2]
                mono = monomials[(0, 1, 2, 0, 1, 2, 3, 4, 5, 3, 4, 5)[q]]
                col = grad * mono * w
                jtf[k, q] = (col * f).sum()
                sj[k, q] = col.sum()
    return jtf, sj


@pytest.mark.parametrize("size,stride,weighting", [(9, 4, "uniform"), (8, 3, "uniform"), (9, 2, "gaussian")])
def test_float64_moments_match_direct_sums(size, stride, weighting):
    rng = np.random.default_rng(size * 10 + stride)
    width, height = 29, 23
    plane = np.zeros((height, width, 4), np.float32)
    plane[..., 0] = rng.uniform(0, 255, (height, width))
    plane[..., 1:3] = rng.normal(0, 20, (height, width, 2))
    weights = window_weights(size, weighting, 2.5)
    jtf, sj, jtf_abs, sj_abs = float64_moments(plane, width, height, size, stride, weights)
    ejtf, esj = _direct(plane, width, height, size, stride, weights)
    np.testing.assert_allclose(jtf, ejtf, rtol=1e-10, atol=1e-8 * np.abs(ejtf).max())
    np.testing.assert_allclose(sj, esj, rtol=1e-10, atol=1e-8 * np.abs(esj).max())
    assert np.all(jtf_abs >= np.abs(jtf) - 1e-6) and np.all(sj_abs >= np.abs(sj) - 1e-6)
