"""End-to-end behaviour of the drop-in engines on the GPU.

Parity against the oracle pipeline on identical inputs (the oracle solves
with the float64 reference preparation, the engine with its own GPU
preparation): identical statuses except for documented threshold
borderline cases, displacement within 1e-3 px and displacement gradients
within 1e-5 at a 1e-4 px convergence tolerance; accuracy against the FP64
imposed field; stream/register equivalence; full-pyramid behaviour.
"""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNError, ICGNWGPU, ICGNWGPUFullPyramid, synthetic
from oracle import oracle as oracle_c
from oracle import reference_prep as rp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c0_pair():
    """Config-0 workload: 512^2 speckle, u = 0.37 + 1e-3 x, v = -0.21 - 5e-4 y."""
    ref, sp = synthetic.reference_image(512, 512, seed=2024, device="cpu")
    field = synthetic.affine_field(0.37, 1e-3, 0.0, -0.21, 0.0, -5e-4)
    tgt = synthetic.deformed_image(sp, field, noise_seed=2025, device="cpu")
    return ref, tgt


def _packed(result):
    return np.concatenate([result.parameters, result.status[..., None], result.iterations[..., None]], -1)


def test_c0_parity_with_oracle_and_truth(c0_pair):
    ref, tgt = c0_pair
    S, s = 21, 10
    with ICGNWGPU(subset_size=S, subset_stride=s, outlier_policy="disabled") as engine:
        engine.set_reference(ref, tolerance=1e-4)
        result = engine.register(tgt)
    plane, inverse, metadata = rp.reference_arrays(ref, subset_size=S, subset_stride=s)
    coef = oracle_c.prefilter(tgt, rp.runtime_fir_taps())
    expected = oracle_c.solve(tgt, coef, plane, metadata, inverse, subset_size=S, subset_stride=s, lanes=16,
                              tolerance=1e-4).reshape(_packed(result).shape)
    status, estatus = result.status, expected[..., 6]
    both = (status == 1) & (estatus == 1)
    mismatch = status != estatus
    assert mismatch.sum() <= max(1, int(0.002 * status.size)), int(mismatch.sum())
    d = np.abs(result.parameters[both] - expected[..., :6][both])
    assert d[:, [0, 3]].max() <= 1e-3
    assert d[:, [1, 2, 4, 5]].max() <= 1e-5
    cx, cy = synthetic.subset_centres(512, 512, S, s)
    truth = synthetic.affine_truth((0.37, 1e-3, 0.0, -0.21, 0.0, -5e-4), cx, cy)
    err = result.displacement[status == 1] - truth[status == 1]
    rmse = float(np.sqrt(np.mean(np.sum(err * err, axis=1))))
    assert rmse <= 0.01, rmse
    assert (status == 1).mean() > 0.9


def test_autotuner_selects_a_validated_variant(c0_pair):
    ref, tgt = c0_pair
    with ICGNWGPU(subset_size=21, subset_stride=10, autotune=True) as engine:
        engine.set_reference(ref)
        chosen = engine.solver
        result = engine.register(tgt)
    assert chosen in engine.solver_tuning_ms
    assert engine.solver_validation[chosen]["valid"]
    assert len(engine.solver_validation) == 18  # 8 exact, 4 fast, 4 staged, 2 staged-wide
    assert (result.status == 1).mean() > 0.9


def test_stream_matches_register(c0_pair):
    ref, tgt = c0_pair
    with ICGNWGPU(subset_size=21, subset_stride=10, pipeline_slots=3) as engine:
        engine.set_reference(ref)
        single = engine.register(tgt)
        streamed = list(engine.register_stream([tgt, ref, tgt, tgt], pipeline_depth=3))
    assert len(streamed) == 4
    np.testing.assert_array_equal(streamed[0].parameters, single.parameters)
    np.testing.assert_array_equal(streamed[2].status, single.status)
    np.testing.assert_array_equal(streamed[3].parameters, single.parameters)
    assert np.abs(streamed[1].displacement[streamed[1].status == 1]).max() < 0.05


def test_lock_rejects_concurrent_use(c0_pair):
    ref, tgt = c0_pair
    with ICGNWGPU(subset_size=21, subset_stride=10) as engine:
        engine.set_reference(ref)
        stream = engine.register_stream([tgt, tgt])
        next(stream)
        with pytest.raises(ICGNError, match="Another registration"):
            engine.register(tgt)
        list(stream)
        engine.register(tgt)


def test_register_before_reference_and_closed_engine():
    engine = ICGNWGPU(subset_size=21, subset_stride=10)
    with pytest.raises(ICGNError, match="set_reference"):
        engine.register(np.zeros((64, 64), np.uint8))
    engine.close()
    engine.close()
    with pytest.raises(ICGNError, match="closed"):
        engine.set_reference(np.zeros((64, 64), np.uint8))


def test_roi_excludes_windows_and_keeps_status(c0_pair):
    ref, tgt = c0_pair
    mask = synthetic.hole_mask(512, 512, 60.0)
    with ICGNWGPU(subset_size=21, subset_stride=10) as engine:
        info = engine.set_reference(ref, roi_mask=mask)
        result = engine.register(tgt)
    excluded = ~info.roi.selected
    assert excluded.sum() > 0
    assert (result.status[excluded] == -3).all()
    assert (result.status[~excluded] == 1).mean() > 0.9
    assert result.populations["roiExcluded"] == int(excluded.sum())


@pytest.mark.parametrize("levels", [1, 2, 3])
def test_full_pyramid_recovers_field(c0_pair, levels):
    ref, tgt = c0_pair
    with ICGNWGPUFullPyramid(pyramid_levels=levels, subset_size=21, subset_stride=10) as engine:
        engine.set_reference(ref)
        result = engine.register(tgt)
    cx, cy = synthetic.subset_centres(512, 512, 21, 10)
    truth = synthetic.affine_truth((0.37, 1e-3, 0.0, -0.21, 0.0, -5e-4), cx, cy)
    ok = result.status >= 1
    err = result.displacement[ok] - truth[ok]
    assert ok.mean() > 0.85
    assert float(np.sqrt(np.mean(np.sum(err * err, axis=1)))) < 0.02


def test_full_pyramid_large_shift_needs_levels():
    ref, sp = synthetic.reference_image(384, 320, seed=71, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(6.3, 0.0, 0.0, -5.2, 0.0, 0.0), noise_seed=72,
                                   device="cpu")
    with ICGNWGPUFullPyramid(pyramid_levels=3, subset_size=31, subset_stride=8) as engine:
        engine.set_reference(ref)
        result = engine.register(tgt)
    ok = result.status >= 1
    assert ok.mean() > 0.8
    np.testing.assert_allclose(np.median(result.displacement[ok], axis=0), [6.3, -5.2], atol=0.02)


def test_temporal_stream_tracks_ramp_and_counts():
    ref, sp = synthetic.reference_image(256, 256, seed=81, device="cpu")
    frames = [
        synthetic.deformed_image(sp, synthetic.affine_field(0.8 * k, 0.0, 0.0, -0.6 * k, 0.0, 0.0),
                                 noise_seed=90 + k, device="cpu")
        for k in range(1, 5)
    ]
    with ICGNWGPUFullPyramid(pyramid_levels=2, subset_size=21, subset_stride=10, initialization="temporal",
                             temporal_prediction="velocity") as engine:
        engine.set_reference(ref)
        results = list(engine.register_stream(frames, pipeline_depth=1))
        engine.reset_temporal_state()
        again = engine.register(frames[0])
    for k, r in enumerate(results, start=1):
        ok = r.status >= 1
        assert ok.mean() > 0.85
        np.testing.assert_allclose(np.median(r.displacement[ok], axis=0), [0.8 * k, -0.6 * k], atol=0.02)
    assert results[0].timing["temporallySeededCoarseSubsets"] == 0
    assert results[1].timing["temporallySeededCoarseSubsets"] > 0
    assert results[2].timing["velocityPredictedSubsets"] > 0
    assert again.timing["temporallySeededCoarseSubsets"] == 0


def test_selective_pyramid_recovery_of_failed_subsets():
    ref, sp = synthetic.reference_image(384, 320, seed=71, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(6.3, 0.0, 0.0, -5.2, 0.0, 0.0), noise_seed=72,
                                   device="cpu")
    mask = synthetic.hole_mask(384, 320, 50.0)
    with ICGNWGPU(subset_size=31, subset_stride=8) as single:
        single.set_reference(ref, roi_mask=mask)
        plain = single.register(tgt)
    with ICGNWGPU(subset_size=31, subset_stride=8, pyramid_levels=3) as engine:
        info = engine.set_reference(ref, roi_mask=mask)
        result = engine.register(tgt)
        # the coarser targets were reduced on the device, bit for bit as
        # the reference's _reduce_half (restated in pyramid_recovery)
        from live_dic_gb300 import _native
        from live_dic_gb300.pyramid_recovery import reduce_half

        expected = tgt
        for child in engine._pyramid_engines:
            expected = reduce_half(expected)
            got = child._export(_native.EXPORT_FRAME, np.uint8, expected.shape)
            np.testing.assert_array_equal(got, expected)
        streamed = list(engine.register_stream([tgt, tgt], pipeline_depth=2))
    inside = info.roi.selected
    assert (result.status[~inside] == -3).all()
    assert result.timing["pyramidFailedBefore"] > 0 and result.timing["pyramidRecovered"] > 0
    ok, ok_plain = result.status >= 1, plain.status >= 1
    assert ok[inside].mean() > ok_plain[inside].mean() + 0.3
    assert ok[inside].mean() > 0.75  # the outer ring and windows pushed off the image stay unrecoverable
    np.testing.assert_allclose(np.median(result.displacement[ok], axis=0), [6.3, -5.2], atol=0.02)
    # subsets the fine level solved are kept as they were
    kept = ok_plain
    np.testing.assert_array_equal(result.parameters[kept], plain.parameters[kept])
    for r in streamed:
        np.testing.assert_array_equal(r.status, result.status)
        np.testing.assert_array_equal(r.parameters, result.parameters)


def test_register_pair_one_shot(c0_pair):
    from live_dic_gb300 import register_pair

    ref, tgt = c0_pair
    one = register_pair(ref, tgt, subset_size=21, subset_stride=10, pyramid_levels=2)
    with ICGNWGPUFullPyramid(pyramid_levels=2, subset_size=21, subset_stride=10) as engine:
        engine.set_reference(ref)
        expected = engine.register(tgt)
    np.testing.assert_array_equal(one.parameters, expected.parameters)
    np.testing.assert_array_equal(one.status, expected.status)
    assert (one.status >= 1).mean() > 0.9
