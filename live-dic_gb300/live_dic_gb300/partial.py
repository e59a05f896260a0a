"""Partial-support reference preparation (host, float64).

Restates prepare_partial_reference (partial.py:26-121): for every ROI window
cut by the mask, the weighted mean, centred intensities, Jacobian sums,
Hessian, its inverse and the admission test (full numerical rank, normalised
condition number <= 1e8, weighted contrast >= 1 grey level, more supported
pixels than parameters) are recomputed over the window's support pixels only,
from the gradients the GPU stored in the reference plane.  The rows are then
uploaded over the full-window rows; validity -4 marks a partial window that
only the partial solver handles.  Complete windows are untouched.
"""

from __future__ import annotations

from dataclasses import replace

import numpy as np

from . import _native
from .roi import PARTIAL_MAX_NORMALIZED_CONDITION, PARTIAL_MIN_WEIGHTED_CONTRAST, RoiPlan, immutable, unpack_support


def prepare_partial_reference(plane: np.ndarray, inverse: np.ndarray, metadata: np.ndarray, roi: RoiPlan, *,
                              width: int, height: int, size: int, stride: int, motion_model: str, weighting: str,
                              sigma: float) -> RoiPlan:
    """Updates `metadata` (grid x 16) and `inverse` (grid x 36) in place for
    the partial windows of `roi`; returns the plan with the per-window
    condition, rank and contrast."""
    pixels = plane.reshape(height, width, 4)
    rows = metadata.reshape(-1, 16)
    inverses = inverse.reshape(-1, 6, 6)
    grid_w = roi.selected.shape[1]
    yy, xx = np.indices((size, size), dtype=np.float64)
    xx = xx.ravel() - (size - 1) / 2
    yy = yy.ravel() - (size - 1) / 2
    spatial = np.exp(-0.5 * (xx ** 2 + yy ** 2) / sigma ** 2) if weighting == "gaussian" else np.ones(size * size)
    active = [0, 3] if motion_model == "translation" else list(range(6))
    scale = np.array([1, 1 / size, 1 / size, 1, 1 / size, 1 / size])[active]
    conditions = np.zeros(roi.selected.shape)
    ranks = np.zeros(roi.selected.shape, np.uint32)
    contrasts = np.zeros(roi.selected.shape)
    for ordinal, index in enumerate(roi.partial_indices):
        gy, gx = divmod(int(index), grid_w)
        support = unpack_support(roi.support_words[ordinal], size).ravel()
        w = spatial * support
        wsum = w.sum(dtype=np.float64)
        tile = pixels[gy * stride: gy * stride + size, gx * stride: gx * stride + size].reshape(-1, 4).astype(np.float64)
        mean = np.dot(w, tile[:, 0]) / wsum
        f = tile[:, 0] - mean
        gxv, gyv = tile[:, 1], tile[:, 2]
        jac = np.stack((gxv, gxv * xx, gxv * yy, gyv, gyv * xx, gyv * yy), axis=1)
        j = jac[:, active]
        hessian = j.T @ (w[:, None] * j)
        eig = np.linalg.eigvalsh(hessian * scale[:, None] * scale[None, :])
        largest = float(eig[-1])
        rank = int(np.count_nonzero(eig > np.finfo(np.float64).eps * len(active) * max(largest, 0.0)))
        contrast = float(np.sqrt(np.dot(w, f * f) / wsum))
        condition = largest / eig[0] if eig[0] > 0 else 0.0
        conditions[gy, gx] = condition if np.isfinite(condition) else 0.0
        ranks[gy, gx] = rank
        contrasts[gy, gx] = contrast
        valid = (rank == len(active) and condition <= PARTIAL_MAX_NORMALIZED_CONDITION
                 and contrast >= PARTIAL_MIN_WEIGHTED_CONTRAST and support.sum() > len(active))
        inv = np.zeros((6, 6))
        if valid:
            if motion_model == "translation":
                det = hessian[0, 0] * hessian[1, 1] - hessian[0, 1] ** 2
                block = np.array([[hessian[1, 1], -hessian[0, 1]], [-hessian[0, 1], hessian[0, 0]]]) / det
            else:
                block = np.linalg.inv(hessian)
            valid = bool(np.isfinite(block).all() and np.max(np.abs(block)) <= np.finfo(np.float32).max)
            if valid:
                inv[np.ix_(active, active)] = block
        inverses[index] = inv
        rows[index] = 0
        rows[index, 0] = np.sqrt(np.dot(w, f * f))
        rows[index, 1] = -4.0 if valid else 0.0
        rows[index, 2:8] = jac.T @ (w * f)
        rows[index, 8:14] = jac.T @ w
        rows[index, 14] = mean
        rows[index, 15] = wsum
    return replace(roi, support_condition=immutable(conditions), support_rank=immutable(ranks),
                   support_contrast=immutable(contrasts))


def install_partial_reference(roi: RoiPlan, export, upload, *, width: int, height: int, size: int, stride: int,
                              motion_model: str, weighting: str, sigma: float) -> RoiPlan:
    """Reads one level's GPU-prepared plane, inverse and metadata through
    `export(what, dtype, shape)`, prepares the partial windows of `roi` and
    hands the tables and replacement rows to `upload(count, indices, words,
    words_per_window, boxes, metadata_rows, inverse_rows)` (a
    gbdic_set_partial_support-shaped C entry)."""
    count = roi.selected.size
    plane = export(_native.EXPORT_PLANE, np.float32, (height * width * 4,))
    inverse = export(_native.EXPORT_INVERSE, np.float32, (count * 36,)).astype(np.float64)
    metadata = export(_native.EXPORT_METADATA, np.float32, (count * 16,)).astype(np.float64)
    roi = prepare_partial_reference(plane, inverse, metadata, roi, width=width, height=height, size=size,
                                    stride=stride, motion_model=motion_model, weighting=weighting, sigma=sigma)
    idx = np.ascontiguousarray(roi.partial_indices, dtype=np.int32)
    rows = np.ascontiguousarray(metadata.reshape(-1, 16)[idx], dtype=np.float32)
    inv_rows = np.ascontiguousarray(inverse.reshape(-1, 36)[idx], dtype=np.float32)
    words = np.ascontiguousarray(roi.support_words, dtype=np.uint32)
    boxes = np.ascontiguousarray(roi.support_boxes, dtype=np.float32)
    upload(int(idx.size), _native.ptr(idx), _native.ptr(words), int(words.shape[1]), _native.ptr(boxes),
           _native.ptr(rows), _native.ptr(inv_rows))
    return roi
