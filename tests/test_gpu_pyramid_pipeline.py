"""Whole full-pyramid frames against the oracle, bit for bit.

The oracle composes its restatements of the reduction, prefilter, seeded
IC-GN, UOD, coarse-to-fine transfer, temporal projection, velocity
prediction, temporal fine correction and history merges in the reference's
order (oracle/pyramid_oracle.py) on the reference arrays the engine prepared;
over a sequence of frames every state, status, iteration count and counter of
every frame must match, which also pins the temporal history the engine
carries from frame to frame.  The adaptive policy's level decision is
checked against the reference's rule.
"""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPUFullPyramid, _native, synthetic
from oracle.pyramid_oracle import LevelArrays, PyramidOracle

pytestmark = pytest.mark.gpu

W, H = 256, 224


def _frames(pattern: str):
    ref, sp = synthetic.reference_image(W, H, seed=401, device="cpu")
    frames = []
    for k in range(1, 8):
        if pattern == "dropout" and k in (4, 5):
            rng = np.random.default_rng(500 + k)
            frames.append(rng.integers(0, 256, size=(H, W), dtype=np.uint8))
            continue
        field = synthetic.affine_field(0.45 * k, 2e-4 * k, 0.0, -0.3 * k, 0.0, -1e-4 * k)
        frames.append(synthetic.deformed_image(sp, field, noise_seed=410 + k, device="cpu"))
    return ref, frames


def _oracle(engine: ICGNWGPUFullPyramid, **kw) -> PyramidOracle:
    levels = []
    for level in range(engine.pyramid_levels):
        gw, gh = engine.level_grid(level)
        w, h = W >> level, H >> level
        levels.append(LevelArrays(
            w, h, gw, gh,
            engine.export_level(level, _native.EXPORT_PLANE, np.float32, (h * w * 4,)),
            engine.export_level(level, _native.EXPORT_METADATA, np.float32, (gw * gh * 16,)),
            engine.export_level(level, _native.EXPORT_INVERSE, np.float32, (gw * gh * 36,))))
    return PyramidOracle(levels, subset_size=engine.subset_size, subset_stride=engine.subset_stride,
                         iterations=engine.iterations_per_level, tolerances=engine.tolerance_per_level,
                         outlier_policy=engine.outlier_policy, lanes=engine.solver_workgroup_size, temporal=True,
                         **kw)


def _packed(result):
    return np.concatenate([result.parameters, result.status[..., None], result.iterations[..., None]], -1)


@pytest.mark.parametrize("prediction,fine,policy,pattern", [
    ("none", False, "fixed", "ramp"),
    ("velocity", False, "fixed", "dropout"),
    ("none", True, "fixed", "ramp"),
    ("velocity", True, "fixed", "dropout"),
    ("none", False, "adaptive", "dropout"),
    ("velocity", True, "adaptive", "dropout"),
])
def test_temporal_pyramid_frames_bit_exact(prediction, fine, policy, pattern):
    ref, frames = _frames(pattern)
    max_age = 1
    with ICGNWGPUFullPyramid(pyramid_levels=2, subset_size=21, subset_stride=10, initialization="temporal",
                             temporal_prediction=prediction, temporal_fine_correction=fine, pyramid_policy=policy,
                             adaptive_acceptance=0.8, temporal_max_age=max_age) as engine:
        engine.set_reference(ref)
        oracle = _oracle(engine, velocity=prediction == "velocity", fine_correction=fine,
                         adaptive=policy == "adaptive", max_age=max_age)
        population = int(engine.reference_valid.sum())
        expected_levels = 2
        used = []
        for k, frame in enumerate(frames):
            result = engine.register(frame)
            levels = int(result.timing["pyramidLevels"])
            used.append(levels)
            assert levels == expected_levels, k
            state, counters = oracle.register(frame, levels)
            got = _packed(result)
            np.testing.assert_array_equal(got, state.reshape(got.shape[0], got.shape[1], -1)[..., : got.shape[-1]],
                                          err_msg=f"frame {k}")
            assert result.timing["temporallySeededCoarseSubsets"] == counters[0]
            assert result.timing["temporalAcceptedUpdates"] == counters[1]
            if prediction == "velocity":
                assert result.timing["velocityPredictedSubsets"] == counters[2]
            if policy == "adaptive":
                assert result.timing["temporalExpiredSubsets"] == counters[3]
                expected_levels = 1 if counters[1] / population >= 0.8 and not counters[3] else 2
                assert result.config["pyramidLevelsUsed"] == levels
    if policy == "adaptive":
        assert 1 in used and used[0] == 2
    if pattern == "dropout":
        assert used[4] == 2 or policy == "fixed"


def test_fine_correction_keeps_fine_detail_over_frames():
    ref, frames = _frames("ramp")
    with ICGNWGPUFullPyramid(pyramid_levels=2, subset_size=21, subset_stride=10, initialization="temporal",
                             temporal_fine_correction=True) as engine:
        engine.set_reference(ref)
        results = list(engine.register_stream(frames, pipeline_depth=2))
        assert engine._config_echo()["temporalFineCorrection"] is True
    for k, r in enumerate(results, start=1):
        ok = r.status >= 1
        assert ok.mean() > 0.85
        np.testing.assert_allclose(np.median(r.displacement[ok], axis=0), [0.45 * k + 2e-4 * k * (W / 2),
                                                                          -0.3 * k - 1e-4 * k * (H / 2)], atol=0.05)


def test_resident_graph_replay_equals_direct_launches():
    """Resident registrations replay the slot's CUDA graph (between two
    device copies) unless solver profiling is on, when the launches are
    issued directly; over a temporal sequence both give the same states."""
    torch = pytest.importorskip("torch")
    ref, frames = _frames("ramp")
    dev = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in frames]
    out = {}
    for mode in ("graph", "direct"):
        with ICGNWGPUFullPyramid(pyramid_levels=2, subset_size=21, subset_stride=10, initialization="temporal",
                                 temporal_prediction="velocity") as engine:
            info = engine.set_reference(ref)
            gw, gh = info.grid
            engine.set_profiling(mode == "direct")
            state = torch.zeros(gw * gh * 8, dtype=torch.float32, device="cuda")
            seq = []
            for f in dev:
                engine.register_device(f.data_ptr(), state.data_ptr())
                torch.cuda.synchronize()
                seq.append(state.view(gh, gw, 8).cpu().numpy().copy())
            out[mode] = seq
    assert len(out["graph"]) == len(frames)
    for a, b in zip(out["graph"], out["direct"], strict=True):
        np.testing.assert_array_equal(a, b)
