"""Host-side checks of the plate-with-hole fixture window (no GPU): the
stored mask is the analytic hole of plate_hole_reference.hole_mask() on the
window, and the ROI planner admits the same 24 partial windows the
reference's regression counts on the full frame (test_plate_hole.py:97)."""

from __future__ import annotations

from pathlib import Path

import numpy as np

from live_dic_gb300 import roi

FIXTURE = Path(__file__).resolve().parent / "golden" / "plate_hole_crop.npz"


def test_window_mask_and_partial_plan():
    with np.load(FIXTURE) as g:
        mask, (ox, oy), (hx, hy), radius = g["mask"], g["origin"], g["centre"], float(g["radius"])
        partial_count = int(g["full_partial_count"])
        truth = g["truth"]
    y, x = np.ogrid[: mask.shape[0], : mask.shape[1]]
    np.testing.assert_array_equal(mask, (x + ox - hx) ** 2 + (y + oy - hy) ** 2 >= radius ** 2)
    plan = roi.prepare_roi(mask, 16, 16, policy="partial")
    assert plan.partial_indices.size == partial_count
    full = roi.prepare_roi(mask, 16, 16, policy="full")
    assert truth.shape[:2] == full.selected.shape
    # the partial windows are exactly the windows cut by the hole boundary
    cut = ~full.selected.ravel() & plan.selected.ravel()
    assert set(np.flatnonzero(cut)) <= set(plan.partial_indices.tolist())
