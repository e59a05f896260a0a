"""The sliding-window ("fast") IC-GN pixel loop against the exact one.

The exact loop keeps the reference's pixel-to-lane order and is bit-exact
against the oracle (test_gpu_kernels.py); the fast loop walks column runs and
sums in another order, so it is held to the parity tolerances instead:
statuses identical except threshold-borderline windows (at most 0.2 % of the
grid), and on windows both accept with the same iteration count
|du| <= 1e-3 px and |grad u| <= 1e-5.  A window whose iteration count
differs (its last update straddled the convergence tolerance) may differ by
up to that tolerance; the field's accuracy against the imposed FP64 field
must be the same.
"""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPU, ICGNWGPUFullPyramid, synthetic

pytestmark = pytest.mark.gpu


def _packed(result):
    return np.concatenate([result.parameters, result.status[..., None], result.iterations[..., None]], -1)


def _check_parity(fast, exact, n=6, tolerance=1e-3):
    sf, se = fast[..., n], exact[..., n]
    assert int((sf != se).sum()) <= max(1, int(0.002 * sf.size)), int((sf != se).sum())
    both = (sf >= 1) & (se >= 1)
    assert both.sum() > 0
    same = both & (fast[..., n + 1] == exact[..., n + 1])
    # At a tight convergence tolerance on small windows the last update is
    # near the noise floor, and a few per cent of windows stop one iteration
    # earlier or later under the other summation order.
    assert same.sum() >= 0.9 * both.sum()
    d = np.abs(fast[..., :n][same] - exact[..., :n][same])
    assert d[:, [0, 3]].max() <= 1e-3, float(d[:, [0, 3]].max())
    assert d[:, [1, 2, 4, 5]].max() <= 1e-5, float(d[:, [1, 2, 4, 5]].max())
    d = np.abs(fast[..., :n][both] - exact[..., :n][both])
    assert d[:, [0, 3]].max() <= tolerance, float(d[:, [0, 3]].max())


@pytest.fixture(scope="module")
def c0_pair():
    ref, sp = synthetic.reference_image(512, 512, seed=2024, device="cuda")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(0.37, 1e-3, 0.0, -0.21, 0.0, -5e-4), noise_seed=2025,
                                   device="cuda")
    return ref, tgt


def _register(ref, tgt, mode, **kw):
    tolerance = kw.pop("tolerance", 1e-4)
    roi = kw.pop("roi_mask", None)
    with ICGNWGPU(subset_size=21, subset_stride=10, outlier_policy="disabled", solver_mode=mode, **kw) as engine:
        engine.set_reference(ref, tolerance=tolerance, roi_mask=roi)
        assert engine.solver_mode == mode
        return _packed(engine.register(tgt))


@pytest.mark.parametrize("lanes,persistent", [(16, False), (32, False), (16, True)])
def test_fast_loop_parity_and_accuracy(c0_pair, lanes, persistent):
    ref, tgt = c0_pair
    exact = _register(ref, tgt, "exact", solver_workgroup_size=lanes, persistent=persistent)
    fast = _register(ref, tgt, "fast", solver_workgroup_size=lanes, persistent=persistent)
    _check_parity(fast, exact)
    cx, cy = synthetic.subset_centres(512, 512, 21, 10)
    truth = synthetic.affine_truth((0.37, 1e-3, 0.0, -0.21, 0.0, -5e-4), cx, cy)
    ok = fast[..., 6] == 1
    err = fast[..., [0, 3]][ok] - truth[ok]
    assert float(np.sqrt(np.mean(np.sum(err * err, 1)))) <= 0.01
    assert ok.mean() > 0.9


@pytest.mark.parametrize("case", ["translation", "gaussian", "roi"])
def test_fast_loop_variants(c0_pair, case):
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
    fast = _register(ref, tgt, "fast", **dict(kw))
    _check_parity(fast, exact)
    if case == "roi":
        assert (fast[..., 6] == -3).sum() > 0
        np.testing.assert_array_equal(fast[..., 6] == -3, exact[..., 6] == -3)


def test_fast_loop_other_subset_sizes(c0_pair):
    """Run partitions of other window sizes (several row segments per column,
    idle slots in the last phase)."""
    ref, tgt = c0_pair
    for size, stride in ((15, 7), (41, 20), (16, 16)):
        res = {}
        for mode in ("exact", "fast"):
            with ICGNWGPU(subset_size=size, subset_stride=stride, outlier_policy="disabled", solver_mode=mode) as e:
                e.set_reference(ref, tolerance=1e-4)
                res[mode] = _packed(e.register(tgt))
        _check_parity(res["fast"], res["exact"])


def test_unsupported_configurations_keep_the_exact_loop(c0_pair):
    """Quadratic windows and the direct interpolants run the exact loop even
    when the fast one is selected: the fields are bit-identical."""
    ref, tgt = c0_pair
    for kw in ({"motion_model": "quadratic"}, {"interpolation": "linear"}, {"solver_workgroup_size": 64}):
        a = _register(ref, tgt, "exact", **dict(kw))
        b = _register(ref, tgt, "fast", **dict(kw))
        np.testing.assert_array_equal(a, b)


def test_fast_loop_on_the_plate_with_hole_sequence():
    """The headline workload's pipeline on a 1024x768 crop: S31/s8, 3 levels,
    ROI hole, ZNCC search on the first frame, temporal + velocity seeding,
    UOD replace, at the engine's per-level schedule (finest tolerance
    5e-3 px)."""
    W, H = 1024, 768
    ref, sp = synthetic.reference_image(W, H, seed=1201, device="cuda")
    field = synthetic.KirschField(W, H, 150.0, peak=2.0)
    mask = synthetic.hole_mask(W, H, 150.0)
    frames = [synthetic.deformed_image(sp, field.torch_field(k / 6), noise_seed=1300 + k, device="cuda")
              for k in range(1, 7)]
    seq = {}
    for mode in ("exact", "fast"):
        with ICGNWGPUFullPyramid(pyramid_levels=3, subset_size=31, subset_stride=8, initialization="temporal",
                                 temporal_prediction="velocity", seed_search_radius=4, solver_mode=mode) as e:
            e.set_reference(ref, roi_mask=mask)
            seq[mode] = [_packed(e.register(f)) for f in frames]
    cx, cy = synthetic.subset_centres(W, H, 31, 8)
    for k in range(6):
        _check_parity(seq["fast"][k], seq["exact"][k], tolerance=5e-3)
        truth = field.truth(cx, cy, load=(k + 1) / 6)
        rmse = {}
        for mode in ("exact", "fast"):
            v = seq[mode][k]
            ok = v[..., 6] >= 1
            err = v[..., [0, 3]][ok] - truth[ok]
            rmse[mode] = float(np.sqrt(np.mean(np.sum(err * err, 1))))
        assert abs(rmse["fast"] - rmse["exact"]) <= 1e-4, rmse
        assert rmse["fast"] < 0.02
