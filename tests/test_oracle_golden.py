"""The oracle is pinned to the reference's own outputs before it is trusted.

Golden vectors come from the reference's NumPy code (tests/golden/
make_golden.py); the IC-GN restatement is pinned to the accuracy gates the
reference's GPU regression tests assert on analytic fixtures
(DIC/LucasKanadeICGN/python/tests/test_gpu_regressions.py:191-241, 730-793).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as oracle_c
from oracle import reference_prep as rp


def test_fir_weights_bit_identical(golden):
    np.testing.assert_array_equal(rp.fir_weights(), golden["fir_weights"])
    assert rp.runtime_fir_taps().shape == (25,)


def test_prefilter_matches_reference_float32_fir(golden):
    # test_gpu_regressions.py:832-858 accepts the GPU FIR at rtol 2e-6, atol 2e-5
    coef = oracle_c.prefilter(golden["prefilter_image"], rp.runtime_fir_taps())
    np.testing.assert_allclose(coef, golden["prefilter_expected"], rtol=2e-6, atol=2e-5)


@pytest.mark.parametrize("k", range(4))
def test_reduce_half_exact(golden, k):
    src = golden[f"reduce_{k}_in"]
    np.testing.assert_array_equal(rp.reduce_half(src), golden[f"reduce_{k}_half"])
    np.testing.assert_array_equal(oracle_c.reduce(src), golden[f"reduce_{k}_int"])
    np.testing.assert_array_equal(golden[f"reduce_{k}_half"], golden[f"reduce_{k}_int"])


def test_reference_arrays_bit_identical(golden):
    image = golden["prep_image"]
    for index, case in enumerate(str(c) for c in golden["prep_cases"]):
        model, interp, size, stride, weighting, sigma = case.split("|")
        plane, inverse, metadata = rp.reference_arrays(
            image,
            interpolation=interp,
            motion_model=model,
            subset_size=int(size),
            subset_stride=int(stride),
            spatial_weighting=weighting,
            gaussian_sigma=float(sigma) if sigma else None,
        )
        np.testing.assert_array_equal(plane, golden[f"prep_{index}_plane"], err_msg=case)
        np.testing.assert_array_equal(inverse, golden[f"prep_{index}_inverse"], err_msg=case)
        np.testing.assert_array_equal(metadata, golden[f"prep_{index}_metadata"], err_msg=case)


def test_flat_reference_is_invalid_and_finite(golden):
    flat = np.full((40, 40), 91, dtype=np.uint8)
    _, inverse, metadata = rp.reference_arrays(flat, subset_size=13, subset_stride=13)
    np.testing.assert_array_equal(inverse, golden["flat_inverse"])
    # a constant image has gradients of pure round-off (~1e-13): compare those absolutely
    np.testing.assert_allclose(metadata, golden["flat_metadata"], rtol=0, atol=1e-8)
    np.testing.assert_array_equal(metadata.reshape(-1, 16)[:, 1], golden["flat_metadata"].reshape(-1, 16)[:, 1])
    assert not metadata.reshape(-1, 16)[:, 1].any()
    assert np.isfinite(inverse).all()


@pytest.mark.parametrize("model", ["affine", "quadratic"])
def test_cpu_seed_transfer_matches_reference(golden, model):
    params = golden[f"transfer_{model}_params"]
    seeds, active = rp.transfer_seed_cpu(
        params,
        golden[f"transfer_{model}_status"],
        source_available=golden[f"transfer_{model}_available"],
        source_scale=2,
        destination_scale=1,
        destination_grid=(17, 13),
        requested=golden[f"transfer_{model}_requested"],
        subset_size=21,
        subset_stride=10,
        motion_model=model,
    )
    np.testing.assert_allclose(seeds, golden[f"transfer_{model}_seeds"], rtol=1e-6, atol=1e-7)
    np.testing.assert_array_equal(active, golden[f"transfer_{model}_active"])


def _texture(x, y):
    v = (
        127.0
        + 34.0 * np.sin(0.173 * x + 0.071 * y)
        + 29.0 * np.cos(0.043 * x - 0.191 * y)
        + 23.0 * np.sin(0.311 * x - 0.137 * y + 0.4)
        + 17.0 * np.cos(0.229 * x + 0.257 * y - 0.8)
    )
    return np.clip(np.rint(v), 0, 255).astype(np.uint8)


@pytest.mark.parametrize("model", ["translation", "affine"])
@pytest.mark.parametrize("lanes", [16, 128])
def test_oracle_solver_fractional_translation_gate(model, lanes):
    """Reference gate: fractional (0.5, -0.375) shift, RMSE < 0.03 px."""
    y, x = np.mgrid[:128, :128].astype(np.float64)
    truth = (0.5, -0.375)
    ref, tgt = _texture(x, y), _texture(x - truth[0], y - truth[1])
    plane, inverse, metadata = rp.reference_arrays(ref, motion_model=model, subset_size=16, subset_stride=16)
    coef = oracle_c.prefilter(tgt, rp.runtime_fir_taps())
    state = oracle_c.solve(tgt, coef, plane, metadata, inverse, subset_size=16, subset_stride=16,
                           model=model, lanes=lanes).reshape(-1, 8)
    accepted = state[:, 6] > 0.5
    assert accepted.sum() > 0
    err = state[accepted][:, [0, 3]] - np.array(truth)
    assert np.sqrt(np.mean(np.sum(err * err, axis=1))) < 0.03


def test_oracle_quadratic_gate():
    """Reference gate (730-793): quadratic warp, displacement RMSE < 0.02 px,
    curvature RMSE < 2e-4, more than 30 accepted (Keys cubic, S = 32)."""
    w = h = 256
    p = np.array([0.4, 0.002, -0.001, -0.3, 0.001, 0.003, 2e-4, -1e-4, 1.5e-4, -2e-4, 1e-4, 2.5e-4])
    ty, tx = np.mgrid[:h, :w].astype(np.float64)
    ox, oy = 0.5 * (w - 1), 0.5 * (h - 1)
    rx, ry = tx.copy(), ty.copy()
    for _ in range(20):
        X, Y = rx - ox, ry - oy
        u = p[0] + p[1] * X + p[2] * Y + 0.5 * p[6] * X * X + p[7] * X * Y + 0.5 * p[8] * Y * Y
        v = p[3] + p[4] * X + p[5] * Y + 0.5 * p[9] * X * X + p[10] * X * Y + 0.5 * p[11] * Y * Y
        j11 = 1 + p[1] + p[6] * X + p[7] * Y
        j12 = p[2] + p[7] * X + p[8] * Y
        j21 = p[4] + p[9] * X + p[10] * Y
        j22 = 1 + p[5] + p[10] * X + p[11] * Y
        rxr, ryr = rx + u - tx, ry + v - ty
        det = j11 * j22 - j12 * j21
        rx -= (j22 * rxr - j12 * ryr) / det
        ry -= (-j21 * rxr + j11 * ryr) / det
    ref, tgt = _texture(tx, ty), _texture(rx, ry)
    plane, inverse, metadata = rp.reference_arrays(ref, motion_model="quadratic", interpolation="cubic",
                                                   subset_size=32, subset_stride=16)
    state = oracle_c.solve(tgt, None, plane, metadata, inverse, subset_size=32, subset_stride=16,
                           model="quadratic", interpolation="cubic", lanes=32).reshape(-1, 16)
    gw = 1 + (w - 32) // 16
    gy, gx = np.divmod(np.arange(state.shape[0]), gw)
    cx, cy = gx * 16 + 15.5 - ox, gy * 16 + 15.5 - oy
    accepted = state[:, 12] > 0.5
    assert accepted.sum() > 30
    u = p[0] + p[1] * cx + p[2] * cy + 0.5 * p[6] * cx * cx + p[7] * cx * cy + 0.5 * p[8] * cy * cy
    v = p[3] + p[4] * cx + p[5] * cy + 0.5 * p[9] * cx * cx + p[10] * cx * cy + 0.5 * p[11] * cy * cy
    err = np.stack([state[:, 0] - u, state[:, 3] - v], 1)[accepted]
    assert np.sqrt(np.mean(np.sum(err * err, 1))) < 0.02
    curv = state[accepted][:, 6:12] - p[6:12]
    assert np.sqrt(np.mean(curv * curv)) < 2e-4


def test_oracle_seed_search_finds_integer_shift():
    rng = np.random.default_rng(3)
    ref = rng.integers(0, 256, size=(90, 100), dtype=np.uint8)
    tgt = np.roll(ref, shift=(-2, 3), axis=(0, 1))  # target(x) = ref(x - 3, y + 2)
    seeds, active, score = oracle_c.seed_search(ref, tgt, subset_size=21, subset_stride=10, radius=5)
    gw = 1 + (100 - 21) // 10
    interior = score > 0.999
    assert interior.sum() > 10 and active.all()
    np.testing.assert_array_equal(seeds[interior][:, 0], 3.0)
    np.testing.assert_array_equal(seeds[interior][:, 3], -2.0)
    assert seeds.shape == (gw * (1 + (90 - 21) // 10), 8)


def test_oracle_uod_flags_a_planted_outlier():
    """A planted translation spike in a smooth field is flagged (status 2)
    and, under 'replace', takes the neighbour medians (icgn.wgsl:1484-1592)."""
    gw, gh = 7, 6
    state = np.zeros((gh * gw, 8), np.float32)
    state[:, 0] = 0.25
    state[:, 3] = -0.1
    state[:, 6] = 1.0
    state[:, 7] = 3.0
    spike = 3 * gw + 3
    state[spike, 0] = 2.0
    meta = np.zeros((gh * gw, 16), np.float32)
    meta[:, 1] = 1.0
    out = oracle_c.uod(state, meta, grid=(gw, gh), subset_stride=10, policy="replace")
    assert out[spike, 6] == 2.0
    assert out[spike, 0] == np.float32(0.25)
    flagged = oracle_c.uod(state, meta, grid=(gw, gh), subset_stride=10, policy="flag")
    assert flagged[spike, 6] == 2.0 and flagged[spike, 0] == 2.0
    others = np.delete(np.arange(gh * gw), spike)
    np.testing.assert_array_equal(out[others], state[others])
