"""Spatial seed propagation on the GPU (spatial_seed.wgsl): the affine
frontier and the translation-hypothesis scoring are bit-exact against the
oracle, and the frontier feeds the seeded solver as in the reference's
test_affine_frontier.py:44-68."""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPU, synthetic
from oracle import oracle as oracle_c

pytestmark = pytest.mark.gpu


def _snapshot(values, accepted):
    packed = np.zeros((*accepted.shape, 8), np.float32)
    packed[..., :6] = values
    packed[..., 6] = accepted
    return packed


def test_frontier_bit_exact_with_roi():
    ref, sp = synthetic.reference_image(240, 200, seed=31, device="cpu")
    mask = synthetic.hole_mask(240, 200, 40.0)
    rng = np.random.default_rng(3)
    with ICGNWGPU(subset_size=21, subset_stride=10) as engine:
        engine.set_reference(ref, roi_mask=mask)
        shape = (engine.grid_height, engine.grid_width)
        values = rng.normal(0, 0.05, (*shape, 6)).astype(np.float32)
        values[..., 0] += 1.5
        values[..., 3] -= 0.5
        accepted = rng.uniform(size=shape) < 0.4
        seeds, active = engine.affine_frontier_seeds(values, accepted)
        valid, permissions = engine._spatial_permissions()
    usable = accepted & valid
    expected, expected_active = oracle_c.affine_frontier(
        _snapshot(np.where(usable[..., None], values, 0), usable), permissions, subset_stride=10)
    np.testing.assert_array_equal(active, expected_active)
    np.testing.assert_array_equal(seeds, expected[..., :6])
    assert active.any() and not (active & usable).any()


def test_public_frontier_feeds_seeded_solver():
    image = np.random.default_rng(46).integers(0, 256, (128, 128), dtype=np.uint8)
    with ICGNWGPU(subset_size=16, subset_stride=16, interpolation="linear", outlier_policy="disabled") as engine:
        engine.set_reference(image, zncc_min=0.65)
        shape = (engine.grid_height, engine.grid_width)
        params = np.zeros((*shape, 6), np.float32)
        accepted = np.zeros(shape, bool)
        accepted[3, 3] = True
        seeds, active = engine.affine_frontier_seeds(params, accepted)
        assert int(active.sum()) == 8 and not active[3, 3]
        result = engine.register_seeded(image, seeds, active, include_zncc=True)
        assert int(np.count_nonzero(result.status == 1)) == 8
        np.testing.assert_allclose(result.zncc[active], 1, atol=1e-5)
        _, empty = engine.affine_frontier_seeds(params, np.zeros(shape, bool))
        assert not empty.any()
        with pytest.raises(ValueError, match="Boolean"):
            engine.affine_frontier_seeds(params, accepted.astype(np.uint8))


@pytest.mark.parametrize("mode,step,failed_only", [("neighbours", 1, False), ("median", 3, False),
                                                   ("neighbours+median", 2, True)])
def test_choose_bit_exact(mode, step, failed_only):
    ref, sp = synthetic.reference_image(256, 224, seed=41, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(6.4, 0.0, 0.0, -4.3, 0.0, 0.0), noise_seed=42,
                                   device="cpu")
    with ICGNWGPU(subset_size=21, subset_stride=10) as engine:
        engine.set_reference(ref)
        first = engine.register(tgt)
        values = np.array(first.parameters)
        accepted = np.asarray(first.status >= 1)
        rng = np.random.default_rng(9)
        prior = np.zeros_like(values)
        prior[..., 0], prior[..., 3] = rng.uniform(-8, 8, accepted.shape), rng.uniform(-8, 8, accepted.shape)
        seeds, improved, scores = engine.spatial_seed_candidates(
            values, accepted, prior=prior, sample_step=step, min_gain=0.01, min_displacement=0.5,
            failed_only=failed_only, candidate_mode=mode)
        _, permissions = engine._spatial_permissions()
    codes = {"neighbours": 0, "median": 1, "neighbours+median": 2}
    prior_packed = np.zeros((*accepted.shape, 8), np.float32)
    prior_packed[..., :6] = prior
    e_seeds, e_active, e_scores = oracle_c.spatial_choose(
        ref, tgt, _snapshot(values, accepted), permissions, subset_size=21, subset_stride=10, prior=prior_packed,
        sample_step=step, min_gain=0.01, min_displacement=0.5, failed_only=failed_only, candidate_mode=codes[mode])
    np.testing.assert_array_equal(improved, e_active)
    np.testing.assert_array_equal(seeds, e_seeds[..., :6])
    np.testing.assert_array_equal(scores, e_scores[..., :2])


def test_choose_recovers_failed_subsets():
    ref, sp = synthetic.reference_image(256, 224, seed=43, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(7.2, 0.0, 0.0, -5.6, 0.0, 0.0), noise_seed=44,
                                   device="cpu")
    with ICGNWGPU(subset_size=21, subset_stride=10) as engine:
        engine.set_reference(ref)
        zero = engine.register(tgt)
        assert (zero.status == 1).mean() < 0.5  # 9 px is beyond the zero-seed capture range
        # one correct island at the centre; every other subset starts from zero
        values = np.zeros((*zero.status.shape, 6), np.float32)
        recovered = np.zeros(zero.status.shape, bool)
        centre = (zero.status.shape[0] // 2, zero.status.shape[1] // 2)
        values[centre] = [7.2, 0.0, 0.0, -5.6, 0.0, 0.0]
        recovered[centre] = True
        for _ in range(40):
            seeds, improved, _ = engine.spatial_seed_candidates(values, recovered, min_gain=0.05,
                                                                min_displacement=0.5, failed_only=True)
            if not improved.any():
                break
            out = engine.register_seeded(tgt, seeds, improved)
            ok = improved & (out.status == 1)
            values[ok] = out.parameters[ok]
            recovered |= ok
    assert recovered.mean() > 0.8
    err = values[recovered][:, [0, 3]] - [7.2, -5.6]
    assert float(np.sqrt(np.mean(np.sum(err * err, -1)))) < 0.02
    assert np.abs(err).max() < 0.25
