"""The reference's UHD tensile regressions on a window of its own fixture.

Follows UHDRegistrationRegressionTests (test_uhd_fixtures.py:86-128, 316-437):
frame_040.png registered against reference.png under the uniform stretch of
machine_truth.csv frame 40 about the frame centre, with the limits of the
fixture's manifest (regression_limits): S16/s16 affine B-spline with UOD
disabled and median (median repair leaves statuses and accepted parameters
unchanged), median filters 5 and 9 at the default subset, and the identity
recovered on the archived images; large fractional rigid motion (16.35,
-8.2) px captured by a 4-level pyramid and (128.35, -64.2) px by the Fourier
initialisation (interior margin 192 px).  The images are a 768 x 768 window of the
native UHD pair on the 16-px grid (tests/golden/make_uhd_fixtures.py); the
interior margin applies to the window.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPUFullPyramid

pytestmark = pytest.mark.gpu
FIXTURE = Path(__file__).resolve().parent / "golden" / "tensile_crop.npz"


def _fixture():
    with np.load(FIXTURE) as g:
        limits = dict(zip(g["limit_names"].tolist(), g["limit_values"].tolist(), strict=True))
        return (g["reference"], g["target"], tuple(g["origin"]), tuple(g["centre"]), tuple(g["stretch"] - 1.0),
                limits)


def _interior(result, margin):
    gy, gx = np.indices(result.status.shape)
    x = gx * result.subset_stride + (result.subset_size - 1) / 2
    y = gy * result.subset_stride + (result.subset_size - 1) / 2
    valid = (x >= margin) & (x < result.width - margin) & (y >= margin) & (y < result.height - margin)
    return valid, x, y


def _truth(x, y, origin, centre, strain):
    return np.stack((strain[0] * (x + origin[0] - centre[0]), strain[1] * (y + origin[1] - centre[1])), axis=-1)


def test_affine_frame_040_median_repair_preserves_accepted_results():
    reference, target, origin, centre, strain, limits = _fixture()
    raw = None
    for policy in ("disabled", "median"):
        with ICGNWGPUFullPyramid(motion_model="affine", subset_size=16, subset_stride=16, interpolation="bspline",
                                 outlier_policy=policy) as engine:
            engine.set_reference(reference)
            result = engine.register(target)
        assert np.isfinite(result.parameters).all()
        assert result.parameters.shape == (48, 48, 6)
        interior, x, y = _interior(result, limits["interior_margin_px"])
        mask = interior & result.accepted_mask
        assert mask.sum() / interior.sum() >= limits["affine_frame_040_minimum_accepted_fraction"]
        distance = np.linalg.norm(result.parameters[..., (0, 3)][mask] - _truth(x, y, origin, centre, strain)[mask],
                                  axis=-1)
        assert float(np.sqrt(np.mean(distance ** 2))) < limits["affine_frame_040_displacement_rmse_px"]
        assert float(np.percentile(distance, 95)) < limits["affine_frame_040_displacement_p95_px"]
        if policy == "disabled":
            raw = (result.parameters.copy(), result.status.copy())
        else:
            np.testing.assert_array_equal(result.status, raw[1])
            np.testing.assert_array_equal(result.parameters[result.accepted_mask], raw[0][result.accepted_mask])


@pytest.mark.parametrize("filter_size", [5, 9])
def test_wider_median_repair_preserves_displacement_bounds(filter_size):
    reference, target, origin, centre, strain, limits = _fixture()
    with ICGNWGPUFullPyramid(motion_model="affine", interpolation="bspline", outlier_policy="median",
                             median_filter_size=filter_size) as engine:
        engine.set_reference(reference)
        result = engine.register(target)
    assert result.config["medianFilterSize"] == filter_size
    assert np.isfinite(result.parameters).all()
    interior, x, y = _interior(result, limits["interior_margin_px"])
    accepted = interior & result.accepted_mask
    assert accepted.sum() / interior.sum() >= 0.90
    distance = np.linalg.norm(result.displacement[accepted] - _truth(x, y, origin, centre, strain)[accepted], axis=-1)
    assert float(np.sqrt(np.mean(distance ** 2))) < 0.05
    assert float(np.percentile(distance, 95)) < 0.10


def test_archived_images_recover_identity():
    reference, target, _, _, _, limits = _fixture()
    with ICGNWGPUFullPyramid(motion_model="translation", subset_size=16, subset_stride=16, interpolation="bspline",
                             outlier_policy="median") as engine:
        for image in (reference, target):
            engine.set_reference(image)
            result = engine.register(image)
            assert result.parameters.shape == (48, 48, 6)
            assert np.isfinite(result.parameters).all()
            interior, _, _ = _interior(result, limits["interior_margin_px"])
            mask = result.accepted_mask & interior
            assert mask.sum() / interior.sum() >= limits["identity_minimum_accepted_fraction"]
            displacement = result.parameters[..., (0, 3)][mask]
            assert float(np.sqrt(np.mean(np.sum(displacement ** 2, axis=-1)))) < limits["identity_displacement_rmse_px"]
            np.testing.assert_array_equal(result.parameters[..., (1, 2, 4, 5)], 0)


def _motion_case(key):
    with np.load(FIXTURE) as g:
        return g["reference"], g[f"shift_{key}"], tuple(float(v) for v in g[f"motion_{key}"])


@pytest.mark.parametrize("model", ["translation", "affine"])
def test_four_level_pyramid_captures_large_fractional_rigid_motion(model):
    reference, target, truth = _motion_case("pyramid")
    with ICGNWGPUFullPyramid(pyramid_levels=4, motion_model=model, outlier_policy="disabled") as engine:
        engine.set_reference(reference)
        result = engine.register(target)
    interior, _, _ = _interior(result, 192)
    accepted = interior & result.accepted_mask
    distance = np.linalg.norm(result.displacement[accepted] - truth, axis=-1)
    assert result.config["pyramidLevels"] == 4
    assert np.isfinite(result.parameters).all()
    assert accepted.sum() / interior.sum() >= 0.90
    assert float(np.sqrt(np.mean(distance ** 2))) < 0.05
    assert float(np.percentile(distance, 95)) < 0.10


@pytest.mark.parametrize("model", ["translation", "affine"])
def test_fourier_initialization_refines_large_fractional_motion(model):
    reference, target, truth = _motion_case("fourier")
    with ICGNWGPUFullPyramid(initialization="fourier", motion_model=model, outlier_policy="disabled") as engine:
        engine.set_reference(reference)
        result = engine.register(target)
    interior, _, _ = _interior(result, 192)
    accepted = interior & result.accepted_mask
    distance = np.linalg.norm(result.displacement[accepted] - truth, axis=-1)
    assert np.isfinite(result.parameters).all()
    assert accepted.sum() / interior.sum() >= 0.90
    assert float(np.sqrt(np.mean(distance ** 2))) < 0.05
    assert float(np.percentile(distance, 95)) < 0.10
    assert abs(result.config["globalTranslation"]["dx"] - truth[0]) <= 2
