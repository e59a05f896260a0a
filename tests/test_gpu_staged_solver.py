"""The IC-GN solver on TMA-staged coefficient tiles ("staged" and
"staged-wide" solver modes) against the exact loop.

The staged modes change only where the B-spline coefficients are read from
(a per-warp shared-memory tile loaded by cp.async.bulk.tensor, reloaded when
a footprint leaves it, global loads for footprints that do not fit); the
samples and their arithmetic are the exact loop's, so every field, status
and iteration count must be bit-identical to it, whatever the tiles do:
reuse across iterations, reloads, footprints too large for the tile, and
widths the tensor map cannot take (the exact loop runs)."""

from __future__ import annotations

import math

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPU, ICGNWGPUFullPyramid, synthetic

pytestmark = pytest.mark.gpu


def _packed(result):
    return np.concatenate([result.parameters, result.status[..., None], result.iterations[..., None]], -1)


@pytest.fixture(scope="module")
def c0_pair():
    ref, sp = synthetic.reference_image(512, 512, seed=2024, device="cuda")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(0.37, 1e-3, 0.0, -0.21, 0.0, -5e-4), noise_seed=2025,
                                   device="cuda")
    return ref, tgt


def _register(ref, tgt, mode, *, size=21, stride=10, **kw):
    roi = kw.pop("roi_mask", None)
    with ICGNWGPU(subset_size=size, subset_stride=stride, outlier_policy="disabled", solver_mode=mode, **kw) as e:
        e.set_reference(ref, tolerance=1e-4, roi_mask=roi)
        assert e.solver_mode == mode
        return _packed(e.register(tgt))


@pytest.mark.parametrize("mode", ["staged", "staged-wide"])
@pytest.mark.parametrize("lanes,persistent", [(16, False), (32, False), (16, True), (32, True)])
def test_staged_tiles_are_bit_identical_to_the_exact_loop(c0_pair, mode, lanes, persistent):
    ref, tgt = c0_pair
    exact = _register(ref, tgt, "exact", solver_workgroup_size=lanes, persistent=persistent)
    staged = _register(ref, tgt, mode, solver_workgroup_size=lanes, persistent=persistent)
    np.testing.assert_array_equal(staged, exact)
    assert (exact[..., 6] == 1).mean() > 0.9


@pytest.mark.parametrize("case", ["translation", "gaussian", "roi"])
def test_staged_tile_variants(c0_pair, case):
    ref, tgt = c0_pair
    kw: dict = {}
    if case == "translation":
        kw = {"motion_model": "translation"}
    elif case == "gaussian":
        kw = {"spatial_weighting": "gaussian"}
    elif case == "roi":
        yy, xx = np.ogrid[:512, :512]
        kw = {"roi_mask": (xx - 250) ** 2 + (yy - 260) ** 2 >= 90 ** 2}
    exact = _register(ref, tgt, "exact", **dict(kw))
    staged = _register(ref, tgt, "staged", **dict(kw))
    np.testing.assert_array_equal(staged, exact)


def test_footprints_beyond_the_tile_and_rotations():
    """A rotated and stretched target: footprints grow with the warp, the
    union of a warp's two windows stops fitting, and S 41 / stride 20 windows
    do not fit the compact tile at all (global loads) but fit the wide one;
    the fields stay bit-identical, failures included."""
    ref, sp = synthetic.reference_image(512, 512, seed=77, device="cuda")
    th = math.radians(3.0)
    c = 255.5

    def field(X, Y):
        dx, dy = X - c, Y - c
        return (math.cos(th) - 1.0) * dx - math.sin(th) * dy + 0.02 * dx, math.sin(th) * dx + (math.cos(th) - 1.0) * dy

    tgt = synthetic.deformed_image(sp, field, noise_seed=78, device="cuda")
    for size, stride in ((21, 10), (31, 8), (41, 20), (15, 7)):
        exact = _register(ref, tgt, "exact", size=size, stride=stride)
        for mode in ("staged", "staged-wide"):
            np.testing.assert_array_equal(_register(ref, tgt, mode, size=size, stride=stride), exact)


def test_widths_the_tensor_map_cannot_take_keep_the_exact_loop():
    """W % 4 != 0 (row pitch not a multiple of 16 bytes) and unsupported
    configurations run the exact loop under the staged modes."""
    ref, sp = synthetic.reference_image(510, 300, seed=91, device="cuda")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(0.3, 2e-3, 0.0, -0.4, 0.0, 1e-3), noise_seed=92,
                                   device="cuda")
    np.testing.assert_array_equal(_register(ref, tgt, "staged"), _register(ref, tgt, "exact"))
    ref2, sp2 = synthetic.reference_image(256, 256, seed=93, device="cuda")
    tgt2 = synthetic.deformed_image(sp2, synthetic.affine_field(0.3, 2e-3, 0.0, -0.4, 0.0, 1e-3), noise_seed=94,
                                    device="cuda")
    for kw in ({"motion_model": "quadratic"}, {"interpolation": "linear"}, {"solver_workgroup_size": 64}):
        np.testing.assert_array_equal(_register(ref2, tgt2, "staged", **dict(kw)),
                                      _register(ref2, tgt2, "exact", **dict(kw)))


def test_staged_pyramid_sequence_is_bit_identical():
    """Config-1 geometry on a 1024 x 768 crop: 3 levels, S31 / s8, ROI hole,
    ZNCC search on the first frame, temporal + velocity seeding, UOD
    replace; every level's solve on staged tiles."""
    W, H = 1024, 768
    ref, sp = synthetic.reference_image(W, H, seed=1201, device="cuda")
    field = synthetic.KirschField(W, H, 150.0, peak=2.0)
    mask = synthetic.hole_mask(W, H, 150.0)
    frames = [synthetic.deformed_image(sp, field.torch_field(k / 5), noise_seed=1300 + k, device="cuda")
              for k in range(1, 6)]
    seq = {}
    for mode in ("exact", "staged"):
        with ICGNWGPUFullPyramid(pyramid_levels=3, subset_size=31, subset_stride=8, initialization="temporal",
                                 temporal_prediction="velocity", seed_search_radius=4, solver_mode=mode) as e:
            e.set_reference(ref, roi_mask=mask)
            seq[mode] = [_packed(e.register(f)) for f in frames]
    for a, b in zip(seq["staged"], seq["exact"], strict=True):
        np.testing.assert_array_equal(a, b)
