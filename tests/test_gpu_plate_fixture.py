"""The reference's UHD plate-with-hole regression on its own fixture.

Follows UHDPlateRegressionTests (test_plate_hole.py:69-99): the full
pyramid with motion_model="affine" and outlier_policy="median", the hole
excluded by the boolean ROI mask under roi_policy "full" and "partial"; on
the predeclared far-field population (radius >= 288 px from the hole centre,
32 px from the border) at least 90 % of the subsets accepted and a
displacement RMSE below 0.05 px against the Kirsch solution at 250 MPa;
under "partial" the 24 partial windows are all admitted and accepted.  The
images are a 768 x 768 window around the hole of assets/uhd_plate_hole
(reference.png, frame_095.png), cut on the 16-px subset grid with the truth
at its subset centres (tests/golden/make_uhd_fixtures.py); the border
margin applies to that window.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPUFullPyramid

pytestmark = pytest.mark.gpu
FIXTURE = Path(__file__).resolve().parent / "golden" / "plate_hole_crop.npz"


@pytest.mark.parametrize("policy", ["full", "partial"])
def test_plate_hole_fixture_gates(policy):
    with np.load(FIXTURE) as g:
        reference, target, mask, truth = g["reference"], g["target"], g["mask"], g["truth"]
        (ox, oy), (hx, hy) = g["origin"], g["centre"]
        partial_count = int(g["full_partial_count"])
    side = reference.shape[0]
    gy, gx = np.indices(truth.shape[:2])
    x, y = gx * 16 + 7.5, gy * 16 + 7.5
    radius = np.hypot(x + ox - hx, y + oy - hy)
    population = (radius >= 288) & (x >= 32) & (x < side - 32) & (y >= 32) & (y < side - 32)
    with ICGNWGPUFullPyramid(motion_model="affine", outlier_policy="median") as engine:
        info = engine.set_reference(reference, roi_mask=mask, roi_policy=policy)
        result = engine.register(target)
        assert (result.height, result.width) == reference.shape
        assert result.status.shape == truth.shape[:2]
        assert np.isfinite(result.parameters).all()
        assert np.all(result.status[~info.roi_selected] == -3)
        accepted = result.accepted_mask[population]
        assert accepted.mean() >= 0.9, accepted.mean()
        error = result.displacement[population][accepted] - truth[population][accepted]
        rmse = float(np.sqrt(np.mean(np.sum(error ** 2, axis=-1))))
        assert rmse < 0.05, rmse
        if policy == "partial":
            assert info.roi.partial_indices.size == partial_count
            assert np.all(result.accepted_mask.ravel()[info.roi.partial_indices])
