"""ZNCC integer seed search: bit-exact against the oracle, and the capture
range it adds to the pyramid."""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPUFullPyramid, _native, synthetic
from oracle import oracle as oracle_c

pytestmark = pytest.mark.gpu


def _inside(width, height, size, stride, shift, margin=4):
    """Windows whose displaced footprint stays inside the image support."""
    gw, gh = 1 + (width - size) // stride, 1 + (height - size) // stride
    y, x = np.indices((gh, gw)) * stride
    return ((x + shift[0] >= 2 + margin) & (x + size - 1 + shift[0] <= width - 3 - margin)
            & (y + shift[1] >= 2 + margin) & (y + size - 1 + shift[1] <= height - 3 - margin))


def _shifted(width, height, shift, seed):
    ref, sp = synthetic.reference_image(width, height, seed=seed, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(shift[0], 0.0, 0.0, shift[1], 0.0, 0.0),
                                   noise_seed=seed + 1, device="cpu")
    return ref, tgt


@pytest.mark.parametrize("radius", [3, 8])
def test_search_bit_exact_single_level(radius):
    ref, tgt = _shifted(200, 176, (5.0, -4.0), 51)
    with ICGNWGPUFullPyramid(pyramid_levels=1, subset_size=21, subset_stride=10, initialization="zncc",
                             seed_search_radius=radius) as engine:
        engine.set_reference(ref)
        engine.register(tgt)
        gw, gh = engine.level_grid(0)
        seed = engine.export_level(0, _native.EXPORT_SEED, np.float32, (gw * gh, 8))
        active = engine.export_level(0, _native.EXPORT_ACTIVE, np.uint32, (gw * gh,))
    expected, expected_active, score = oracle_c.seed_search(ref, tgt, subset_size=21, subset_stride=10,
                                                            radius=radius)
    np.testing.assert_array_equal(seed, expected)
    np.testing.assert_array_equal(active, expected_active)
    if radius == 8:
        interior = score > 0.8
        assert interior.sum() > 0.5 * interior.size
        np.testing.assert_array_equal(seed[interior][:, [0, 3]], np.tile([5.0, -4.0], (int(interior.sum()), 1)))


def test_search_extends_capture_range():
    ref, tgt = _shifted(384, 320, (23.4, -17.7), 61)
    truth = np.array([23.4, -17.7])
    common = dict(pyramid_levels=3, subset_size=31, subset_stride=8)
    with ICGNWGPUFullPyramid(initialization="zero", **common) as engine:
        engine.set_reference(ref)
        plain = engine.register(tgt)
    with ICGNWGPUFullPyramid(initialization="zncc", seed_search_radius=8, **common) as engine:
        engine.set_reference(ref)
        searched = engine.register(tgt)
    # Coarse windows pushed off the image fail with status 0, and the seed
    # transfer interpolates every status > -0.5 (full_pyramid.wgsl:272), so a
    # band about one coarse window wide along the leading edges inherits those
    # seeds; capture is measured inside it.
    inside = _inside(384, 320, 31, 8, truth, margin=48)
    ok = searched.status >= 1
    assert ok.mean() > 0.6
    assert ok[inside].mean() > 0.95
    np.testing.assert_allclose(np.median(searched.displacement[ok], axis=0), truth, atol=0.02)
    good_plain = (plain.status >= 1) & (np.abs(plain.displacement - truth).max(axis=-1) < 0.1)
    assert good_plain[inside].mean() < 0.5 * ok[inside].mean()


def test_temporal_with_search_seeds_first_frame_only():
    ref, sp = synthetic.reference_image(256, 256, seed=71, device="cpu")
    frames = [
        synthetic.deformed_image(sp, synthetic.affine_field(12.0 + 0.5 * k, 0.0, 0.0, -9.0 - 0.3 * k, 0.0, 0.0),
                                 noise_seed=80 + k, device="cpu")
        for k in range(3)
    ]
    with ICGNWGPUFullPyramid(pyramid_levels=2, subset_size=21, subset_stride=10, initialization="temporal",
                             seed_search_radius=8) as engine:
        engine.set_reference(ref)
        results = list(engine.register_stream(frames, pipeline_depth=1))
    for k, r in enumerate(results):
        ok = r.status >= 1
        assert ok[_inside(256, 256, 21, 10, (12.0 + 0.5 * k, -9.0 - 0.3 * k))].mean() > 0.9
        np.testing.assert_allclose(np.median(r.displacement[ok], axis=0), [12.0 + 0.5 * k, -9.0 - 0.3 * k],
                                   atol=0.02)
    assert results[0].timing["temporallySeededCoarseSubsets"] == 0
    assert results[1].timing["temporallySeededCoarseSubsets"] > 0
