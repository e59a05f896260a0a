"""Partial-support ROI windows on the GPU (roi_policy="partial").

The partial solver is compared bit for bit with the oracle's partial solve
(icgn.wgsl solve_partial, restated in oracle/icgn_oracle.c) on the arrays the
engine holds after the partial preparation; the host preparation itself is
pinned to the reference's outputs by the CPU tests.  At engine level the
windows cut by a hole recover the imposed field over their support.
"""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNError, ICGNWGPU, synthetic
from oracle import oracle as oracle_c

pytestmark = pytest.mark.gpu

W, H = 256, 224
FIELD = (0.37, 1e-3, 0.0, -0.21, 0.0, -5e-4)


@pytest.fixture(scope="module")
def pair():
    ref, sp = synthetic.reference_image(W, H, seed=301, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(*FIELD), noise_seed=302, device="cpu")
    return ref, tgt


def _packed(result):
    return np.concatenate([result.parameters, result.status[..., None], result.iterations[..., None]], -1)


@pytest.mark.parametrize("model,interp", [("affine", "bspline"), ("translation", "cubic"),
                                          ("affine", "linear")])
@pytest.mark.parametrize("lanes", [32, 64])
def test_partial_solver_bit_exact(pair, model, interp, lanes):
    ref, tgt = pair
    mask = synthetic.hole_mask(W, H, 45.0)
    with ICGNWGPU(subset_size=21, subset_stride=10, motion_model=model, interpolation=interp,
                  outlier_policy="disabled", solver_workgroup_size=lanes) as engine:
        info = engine.set_reference(ref, roi_mask=mask, roi_policy="partial")
        result = engine.register(tgt)
        plane, inverse, metadata = engine.export_reference()
        coef = engine.export_coefficients() if interp == "bspline" else None
    plan = info.roi
    assert plan.partial_indices.size > 0
    state = oracle_c.solve(tgt, coef, plane, metadata, inverse, subset_size=21, subset_stride=10, model=model,
                           interpolation=interp, lanes=lanes, roi_enabled=True)
    state = oracle_c.solve(tgt, coef, plane, metadata, inverse, subset_size=21, subset_stride=10, model=model,
                           interpolation=interp, lanes=lanes, roi_enabled=True, state=state,
                           partial=(plan.partial_indices, plan.support_words, plan.support_boxes))
    got = _packed(result)
    expected = state.reshape(got.shape[0], got.shape[1], -1)[..., : got.shape[-1]]
    np.testing.assert_array_equal(got, expected)
    flat = got.reshape(-1, got.shape[-1])
    admitted = metadata.reshape(-1, 16)[plan.partial_indices, 1] == -4.0
    assert admitted.sum() > 0
    assert (flat[plan.partial_indices[admitted], 6] == 1).mean() > 0.8


def test_partial_windows_recover_field_under_hole(pair):
    ref, tgt = pair
    mask = synthetic.hole_mask(W, H, 45.0)
    with ICGNWGPU(subset_size=21, subset_stride=10, outlier_policy="disabled") as engine:
        full = engine.set_reference(ref, roi_mask=mask)
        plain = engine.register(tgt)
        info = engine.set_reference(ref, roi_mask=mask, roi_policy="partial")
        result = engine.register(tgt)
        again = engine.register(tgt)
    plan = info.roi
    cut = np.zeros(plan.selected.shape, bool)
    cut.ravel()[plan.partial_indices] = True
    assert (plain.status[cut] == -3).all()
    ok = (result.status == 1) & cut
    assert ok.sum() >= 0.8 * cut.sum()
    cx, cy = synthetic.subset_centres(W, H, 21, 10)
    truth = synthetic.affine_truth(FIELD, cx, cy)
    err = result.displacement[ok] - truth[ok]
    assert float(np.sqrt(np.mean(np.sum(err * err, axis=1)))) < 0.03
    # complete windows are solved exactly as under roi_policy="full"
    complete = full.roi.selected & ~cut
    np.testing.assert_array_equal(result.parameters[complete], plain.parameters[complete])
    np.testing.assert_array_equal(again.parameters, result.parameters)


def test_partial_policy_rejects_quadratic(pair):
    ref, _ = pair
    mask = synthetic.hole_mask(W, H, 45.0)
    with ICGNWGPU(subset_size=21, subset_stride=10, motion_model="quadratic") as engine:
        with pytest.raises((ICGNError, ValueError)):
            engine.set_reference(ref, roi_mask=mask, roi_policy="partial")


@pytest.mark.parametrize("levels", [2, 3])
def test_full_pyramid_partial_windows(pair, levels):
    from live_dic_gb300 import ICGNWGPUFullPyramid

    ref, tgt = pair
    mask = synthetic.hole_mask(W, H, 45.0)
    with ICGNWGPUFullPyramid(pyramid_levels=levels, subset_size=21, subset_stride=10) as engine:
        info = engine.set_reference(ref, roi_mask=mask, roi_policy="partial")
        result = engine.register(tgt)
        streamed = list(engine.register_stream([tgt, tgt], pipeline_depth=2))
    plan = info.roi
    cut = np.zeros(plan.selected.shape, bool)
    cut.ravel()[plan.partial_indices] = True
    assert cut.sum() > 0
    ok = result.status == 1
    assert ok[cut].mean() > 0.8
    assert ok[plan.selected].mean() > 0.85  # the image-edge row is lost at the coarse scales, as without a mask
    cx, cy = synthetic.subset_centres(W, H, 21, 10)
    truth = synthetic.affine_truth(FIELD, cx, cy)
    err = result.displacement[ok] - truth[ok]
    assert float(np.sqrt(np.mean(np.sum(err * err, axis=1)))) < 0.03
    for r in streamed:
        np.testing.assert_array_equal(r.parameters, result.parameters)


def test_selective_recovery_keeps_partial_policy(pair):
    ref, tgt = pair
    mask = synthetic.hole_mask(W, H, 45.0)
    with ICGNWGPU(subset_size=21, subset_stride=10, pyramid_levels=2) as engine:
        info = engine.set_reference(ref, roi_mask=mask, roi_policy="partial")
        result = engine.register(tgt)
    cut = np.zeros(info.roi.selected.shape, bool)
    cut.ravel()[info.roi.partial_indices] = True
    assert (result.status[cut] == 1).mean() > 0.8
