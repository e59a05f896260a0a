"""Parity at the geometry of the headline workloads.

* UHD plate-with-hole sequence (subset 31 / step 8, 3-level pyramid, a
  circular ROI hole, ZNCC integer search on the first frame, temporal
  seeding with velocity prediction afterwards, UOD replace): a 1024x768
  crop with a hole of radius 150 px and the Kirsch field ramped to a 2 px
  peak over 6 frames, every frame bit for bit against the pipeline oracle
  (oracle/pyramid_oracle.py) fed the engine's per-level reference arrays
  and the host ROI tables.
* Quadratic consecutive pairs (subset 41 / step 10, GPU reference
  preparation every pair): the 12x12 preparation against the float64
  restatement of _reference_arrays (the reference's own GPU-preparation
  tolerances, test_gpu_reference.py:107-124, for every first-order
  quantity; the second-order moments stage by stage), then the engine's GPU
  preparation + GPU solve against float64 preparation + oracle solve at
  the parity tolerances (identical statuses except threshold borderline
  windows, |du| <= 1e-3 px, |grad u| <= 1e-5), and the reference's accuracy
  gate for the quadratic model against the imposed sinusoid field
  (test_gpu_regressions.py:730-793: displacement RMSE < 0.02 px, curvature
  RMSE < 2e-4).
"""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPU, ICGNWGPUFullPyramid, _native, synthetic
from oracle import oracle as oracle_c
from oracle import reference_prep as rp
from oracle.pyramid_oracle import LevelArrays, PyramidOracle, roi_tables
from quadratic_prep import check_quadratic_preparation

pytestmark = pytest.mark.gpu


def _packed(result):
    return np.concatenate([result.parameters, result.status[..., None], result.iterations[..., None]], -1)


# ------------------------------------------------------------------ plate-with-hole sequence
PW, PH, HOLE, S1, ST1, LEVELS, RADIUS = 1024, 768, 150.0, 31, 8, 3, 4


def test_plate_with_hole_sequence_bit_exact():
    ref, sp = synthetic.reference_image(PW, PH, seed=1201, device="cuda")
    field = synthetic.KirschField(PW, PH, HOLE, peak=2.0)
    mask = synthetic.hole_mask(PW, PH, HOLE)
    count = 6
    frames = [synthetic.deformed_image(sp, field.torch_field(k / count), noise_seed=1300 + k, device="cuda")
              for k in range(1, count + 1)]
    plans, rois, temporal = roi_tables(mask, subset_size=S1, subset_stride=ST1, levels=LEVELS)
    refs = [ref]
    for _ in range(1, LEVELS):
        refs.append(oracle_c.reduce(refs[-1]))
    with ICGNWGPUFullPyramid(pyramid_levels=LEVELS, subset_size=S1, subset_stride=ST1, initialization="temporal",
                             temporal_prediction="velocity", seed_search_radius=RADIUS) as engine:
        info = engine.set_reference(ref, roi_mask=mask)
        np.testing.assert_array_equal(info.roi.selected, plans[0].selected)
        levels = []
        for level in range(LEVELS):
            gw, gh = engine.level_grid(level)
            w, h = PW >> level, PH >> level
            levels.append(LevelArrays(
                w, h, gw, gh,
                engine.export_level(level, _native.EXPORT_PLANE, np.float32, (h * w * 4,)),
                engine.export_level(level, _native.EXPORT_METADATA, np.float32, (gw * gh * 16,)),
                engine.export_level(level, _native.EXPORT_INVERSE, np.float32, (gw * gh * 36,))))
        oracle = PyramidOracle(levels, subset_size=S1, subset_stride=ST1, iterations=engine.iterations_per_level,
                               tolerances=engine.tolerance_per_level, outlier_policy=engine.outlier_policy,
                               lanes=engine.solver_workgroup_size, temporal=True, velocity=True, rois=rois,
                               temporal_links=temporal, search_radius=RADIUS, reference_levels=refs)
        selected = plans[0].selected
        cx, cy = synthetic.subset_centres(PW, PH, S1, ST1)
        for k, frame in enumerate(frames):
            result = engine.register(frame)
            state, counters = oracle.register(frame)
            got = _packed(result)
            np.testing.assert_array_equal(got, state.reshape(got.shape), err_msg=f"frame {k}")
            assert result.timing["temporallySeededCoarseSubsets"] == counters[0]
            assert result.timing["temporalAcceptedUpdates"] == counters[1]
            assert result.timing["velocityPredictedSubsets"] == counters[2]
            assert np.all(result.status[~selected] == -3)
            ok = result.status >= 1
            assert ok[selected].mean() > 0.95, (k, ok[selected].mean())
            truth = field.truth(cx, cy, load=(k + 1) / count)
            err = result.displacement[ok] - truth[ok]
            rmse = float(np.sqrt(np.mean(np.sum(err * err, axis=1))))
            assert rmse < 0.02, (k, rmse)
        assert counters[0] > 0 and counters[2] > 0


# ------------------------------------------------------------------ quadratic pairs
QW, QH, S2, ST2 = 640, 480, 41, 10


@pytest.fixture(scope="module")
def quadratic_pair():
    ref, sp = synthetic.reference_image(QW, QH, seed=1401, device="cuda")
    field = synthetic.sinusoid_field()
    tgt = synthetic.deformed_image(sp, field, noise_seed=1402, device="cuda")
    return ref, tgt, field


def _sinusoid_parameters(cx, cy):
    """u = 2 sin(kx x) cos(ky y), v = 1.5 cos(kv x): the 12 quadratic
    parameters [u, ux, uy, v, vx, vy, uxx, uxy, uyy, vxx, vxy, vyy]."""
    kx, ky, kv = 2 * np.pi / 400.0, 2 * np.pi / 600.0, 2 * np.pi / 500.0
    sx, cxx = np.sin(kx * cx), np.cos(kx * cx)
    sy, cyy = np.sin(ky * cy), np.cos(ky * cy)
    sv, cv = np.sin(kv * cx), np.cos(kv * cx)
    zero = np.zeros_like(cx)
    return np.stack([
        2 * sx * cyy, 2 * kx * cxx * cyy, -2 * ky * sx * sy,
        1.5 * cv, -1.5 * kv * sv, zero,
        -2 * kx * kx * sx * cyy, -2 * kx * ky * cxx * sy, -2 * ky * ky * sx * cyy,
        -1.5 * kv * kv * cv, zero, zero], -1)


def test_quadratic_preparation_matches_float64_oracle(quadratic_pair):
    """The reference's GPU-preparation tolerances for every first-order
    quantity, the second-order moments stage by stage
    (quadratic_prep.check_quadratic_preparation)."""
    ref, _, _ = quadratic_pair
    ok = check_quadratic_preparation(ref, S2, ST2)
    assert ok.all()


def test_quadratic_pair_parity_and_curvature_accuracy(quadratic_pair):
    ref, tgt, _ = quadratic_pair
    with ICGNWGPU(motion_model="quadratic", subset_size=S2, subset_stride=ST2, outlier_policy="disabled") as engine:
        engine.set_reference(ref, tolerance=1e-4)
        result = engine.register(tgt)
    plane, inverse, metadata = rp.reference_arrays(ref, motion_model="quadratic", subset_size=S2, subset_stride=ST2)
    coef = oracle_c.prefilter(tgt, rp.runtime_fir_taps())
    expected = oracle_c.solve(tgt, coef, plane, metadata, inverse, subset_size=S2, subset_stride=ST2,
                              model="quadratic", lanes=16, tolerance=1e-4)
    expected = expected.reshape(result.parameters.shape[:2] + (16,))
    status, estatus = result.status, expected[..., 12]
    mismatch = status != estatus
    assert mismatch.sum() <= max(1, int(0.002 * status.size)), int(mismatch.sum())
    both = (status == 1) & (estatus == 1)
    assert both.mean() > 0.95
    d = np.abs(result.parameters[both] - expected[..., :12][both])
    assert d[:, [0, 3]].max() <= 1e-3, float(d[:, [0, 3]].max())
    assert d[:, [1, 2, 4, 5]].max() <= 1e-5, float(d[:, [1, 2, 4, 5]].max())
    # the curvature terms: the gradient bound over half a subset
    assert d[:, 6:].max() <= 1e-5 / ((S2 - 1) / 2), float(d[:, 6:].max())
    cx, cy = synthetic.subset_centres(QW, QH, S2, ST2)
    truth = _sinusoid_parameters(cx, cy)
    ok = status == 1
    error = result.parameters.astype(np.float64) - truth
    displacement_rmse = float(np.sqrt(np.mean(np.sum(error[..., (0, 3)][ok] ** 2, axis=1))))
    curvature_rmse = float(np.sqrt(np.mean(error[..., 6:][ok] ** 2)))
    assert displacement_rmse < 0.02, displacement_rmse
    assert curvature_rmse < 2e-4, curvature_rmse


# ------------------------------------------------------------------ large motion, Fourier-seeded search
def test_fourier_seeded_search_pyramid_bit_exact():
    """The plain comparator of the learned seeding at its geometry (subset 31
    / step 8, 3 levels) on a 1024x768 crop: rigid translations of 20-30 px
    plus strain and shear of 1-2 %.  The Fourier initialization's global
    translation seeds the coarsest level and the integer ZNCC search,
    centred on it, absorbs the strain's residual; every frame is compared bit
    for bit with the pipeline oracle given the engine's translation
    estimate."""
    W, H, radius = 1024, 768, 6
    ref, sp = synthetic.reference_image(W, H, seed=1501, device="cuda")
    c = (0.5 * (W - 1), 0.5 * (H - 1))
    cases = [((24.3, -17.6), (0.02, -0.015, 0.01)), ((-28.1, 9.4), (-0.018, 0.02, -0.012))]
    refs = [ref]
    for _ in range(2):
        refs.append(oracle_c.reduce(refs[-1]))
    cx, cy = synthetic.subset_centres(W, H, S1, ST1)
    with ICGNWGPUFullPyramid(pyramid_levels=3, subset_size=S1, subset_stride=ST1, initialization="fourier",
                             seed_search_radius=radius) as engine:
        engine.set_reference(ref)
        levels = []
        for level in range(3):
            gw, gh = engine.level_grid(level)
            w, h = W >> level, H >> level
            levels.append(LevelArrays(
                w, h, gw, gh,
                engine.export_level(level, _native.EXPORT_PLANE, np.float32, (h * w * 4,)),
                engine.export_level(level, _native.EXPORT_METADATA, np.float32, (gw * gh * 16,)),
                engine.export_level(level, _native.EXPORT_INVERSE, np.float32, (gw * gh * 36,))))
        oracle = PyramidOracle(levels, subset_size=S1, subset_stride=ST1, iterations=engine.iterations_per_level,
                               tolerances=engine.tolerance_per_level, outlier_policy=engine.outlier_policy,
                               lanes=engine.solver_workgroup_size, search_radius=radius, reference_levels=refs,
                               global_shift=True)
        for k, (t, e) in enumerate(cases):
            def field(X, Y, t=t, e=e):
                return (t[0] + e[0] * (X - c[0]) + e[2] * (Y - c[1]), t[1] + e[2] * (X - c[0]) + e[1] * (Y - c[1]))

            frame = synthetic.deformed_image(sp, field, noise_seed=1510 + k, device="cuda")
            result = engine.register(frame)
            shift = result.config["globalTranslation"]
            assert abs(shift["dx"] - t[0]) <= 2.0 and abs(shift["dy"] - t[1]) <= 2.0
            state, _ = oracle.register(frame, shift=(shift["dx"], shift["dy"]))
            got = _packed(result)
            np.testing.assert_array_equal(got, state.reshape(got.shape), err_msg=f"frame {k}")
            u, v = field(cx, cy)
            # Coarse windows pushed off the image fail, and the transfer
            # hands their seeds to a band about one coarse window wide
            # (31 x 4 px) along the leading edges; accuracy is measured
            # inside it.
            m = 2 * S1
            inside = (cx - 15 + u > m) & (cx + 15 + u < W - m) & (cy - 15 + v > m) & (cy + 15 + v < H - m)
            ok = result.status >= 1
            assert ok[inside].mean() > 0.95, ok[inside].mean()
            err = np.hypot(result.displacement[..., 0] - u, result.displacement[..., 1] - v)[ok & inside]
            assert float(np.sqrt(np.mean(err ** 2))) < 0.02
