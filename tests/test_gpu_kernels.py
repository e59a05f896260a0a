"""Bit-exact parity of the CUDA kernels with the CPU oracle.

The solver is fed the same prepared reference arrays as the oracle (the
reference's own layout, via set_reference_arrays), so the FIR prefilter,
IC-GN iterations, statuses and the UOD pass can be compared bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPU, synthetic
from oracle import oracle as oracle_c
from oracle import reference_prep as rp

pytestmark = pytest.mark.gpu

W, H = 160, 144


@pytest.fixture(scope="module")
def pair():
    ref, sp = synthetic.reference_image(W, H, seed=101, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(0.37, 1e-3, 0.0, -0.21, 0.0, -5e-4), noise_seed=102,
                                   device="cpu")
    return ref, tgt


def _packed(result):
    return np.concatenate([result.parameters, result.status[..., None], result.iterations[..., None]], -1)


def _solve_both(ref, tgt, *, model, interp, lanes, size=21, stride=10, tolerance=1e-3, weighting="uniform",
                sigma=None, persistent=False):
    plane, inverse, metadata = rp.reference_arrays(ref, interpolation=interp, motion_model=model, subset_size=size,
                                                   subset_stride=stride, spatial_weighting=weighting,
                                                   gaussian_sigma=sigma)
    with ICGNWGPU(subset_size=size, subset_stride=stride, motion_model=model, interpolation=interp,
                  outlier_policy="disabled", solver_workgroup_size=lanes, spatial_weighting=weighting,
                  gaussian_sigma=sigma, persistent=persistent) as engine:
        engine.set_reference_arrays(W, H, plane, metadata, inverse, tolerance=tolerance)
        result = engine.register(tgt)
        weights = engine.export_weights() if weighting == "gaussian" else None
        coef = engine.export_coefficients() if interp == "bspline" else None
    expected_coef = oracle_c.prefilter(tgt, rp.runtime_fir_taps()) if interp == "bspline" else None
    if coef is not None:
        np.testing.assert_array_equal(coef, expected_coef)
    expected = oracle_c.solve(tgt, expected_coef, plane, metadata, inverse, subset_size=size, subset_stride=stride,
                              model=model, interpolation=interp, lanes=lanes, tolerance=tolerance,
                              weights=weights)
    got = _packed(result)
    return got, expected.reshape(got.shape[0], got.shape[1], -1)[..., : got.shape[-1]]


def test_prefilter_bit_exact(pair):
    _, tgt = pair
    got, expected = _solve_both(*pair, model="affine", interp="bspline", lanes=32)
    np.testing.assert_array_equal(got, expected)


@pytest.mark.parametrize("model", ["affine", "translation", "quadratic"])
@pytest.mark.parametrize("interp", ["bspline", "linear", "cubic"])
def test_solver_bit_exact_models_and_interpolants(pair, model, interp):
    got, expected = _solve_both(*pair, model=model, interp=interp, lanes=32)
    np.testing.assert_array_equal(got, expected)
    assert (got[..., -2] > 0.5).sum() > 0


@pytest.mark.parametrize("lanes", [16, 32, 64, 128])
def test_solver_bit_exact_every_lane_count(pair, lanes):
    got, expected = _solve_both(*pair, model="affine", interp="bspline", lanes=lanes, tolerance=1e-4)
    np.testing.assert_array_equal(got, expected)


@pytest.mark.parametrize("lanes", [32, 128])
def test_persistent_queue_matches_grid_launch(pair, lanes):
    got, expected = _solve_both(*pair, model="affine", interp="bspline", lanes=lanes, persistent=True)
    np.testing.assert_array_equal(got, expected)


def test_gaussian_weighting_bit_exact(pair):
    got, expected = _solve_both(*pair, model="affine", interp="bspline", lanes=32, size=21, stride=7,
                                weighting="gaussian", sigma=5.0)
    np.testing.assert_array_equal(got, expected)


def test_tiled_grid_and_quadratic_lanes(pair):
    got, expected = _solve_both(*pair, model="quadratic", interp="bspline", lanes=64, size=31, stride=31)
    np.testing.assert_array_equal(got, expected)


def test_seeded_and_retry_bit_exact(pair):
    ref, tgt = pair
    plane, inverse, metadata = rp.reference_arrays(ref, subset_size=21, subset_stride=10)
    gw, gh = 1 + (W - 21) // 10, 1 + (H - 21) // 10
    rng = np.random.default_rng(5)
    seeds = np.zeros((gh, gw, 6), np.float32)
    seeds[..., 0] = 0.3 + rng.normal(0, 0.2, (gh, gw))
    seeds[..., 3] = -0.2 + rng.normal(0, 0.2, (gh, gw))
    active = rng.random((gh, gw)) > 0.3
    with ICGNWGPU(subset_size=21, subset_stride=10, outlier_policy="disabled") as engine:
        engine.set_reference_arrays(W, H, plane, metadata, inverse)
        result = engine.register_seeded(tgt, seeds, active, iterations=12)
    coef = oracle_c.prefilter(tgt, rp.runtime_fir_taps())
    packed_seeds = np.zeros((gh * gw, 8), np.float32)
    packed_seeds[:, :6] = np.where(active.reshape(-1, 1), seeds.reshape(-1, 6), 0)
    expected = oracle_c.solve(tgt, coef, plane, metadata, inverse, subset_size=21, subset_stride=10, lanes=16,
                              iterations=12, seed_state=packed_seeds, active=active.ravel().astype(np.uint32))
    np.testing.assert_array_equal(_packed(result), expected.reshape(gh, gw, 8))
    assert (result.status[~active] == -1).all()


@pytest.mark.parametrize("policy", ["replace", "flag", "median"])
def test_uod_bit_exact_on_planted_outliers(pair, policy):
    ref, tgt = pair
    plane, inverse, metadata = rp.reference_arrays(ref, subset_size=21, subset_stride=10)
    gw, gh = 1 + (W - 21) // 10, 1 + (H - 21) // 10
    rng = np.random.default_rng(9)
    state = np.zeros((gh, gw, 8), np.float32)
    state[..., 0] = 0.3 + rng.normal(0, 0.02, (gh, gw))
    state[..., 3] = -0.2 + rng.normal(0, 0.02, (gh, gw))
    state[..., 1:3] = rng.normal(0, 1e-3, (gh, gw, 2))
    state[..., 4:6] = rng.normal(0, 1e-3, (gh, gw, 2))
    state[..., 6] = rng.choice(np.array([1.0] * 10 + [0.0, -1.0, -2.0], np.float32), (gh, gw))
    state[..., 7] = 4.0
    spikes = rng.random((gh, gw)) < 0.08
    state[spikes, 0] += 3.0
    with ICGNWGPU(subset_size=21, subset_stride=10, outlier_policy=policy) as engine:
        engine.set_reference_arrays(W, H, plane, metadata, inverse)
        got = engine.apply_outlier_filter(state)
        seeded = engine.apply_outlier_filter(state, seed_mode=True) if policy == "median" else None
    expected = oracle_c.uod(state.reshape(-1, 8), metadata, grid=(gw, gh), subset_stride=10, policy=policy)
    np.testing.assert_array_equal(got.reshape(-1, 8), expected)
    if policy != "median":
        assert (got[..., 6] == 2.0).sum() > 0
    if seeded is not None:
        expected_seeded = oracle_c.uod(state.reshape(-1, 8), metadata, grid=(gw, gh), subset_stride=10,
                                       policy=policy, seed_mode=True)
        np.testing.assert_array_equal(seeded.reshape(-1, 8), expected_seeded)


@pytest.mark.parametrize("size", [5, 9])
def test_wide_median_bit_exact(pair, size):
    ref, _ = pair
    plane, inverse, metadata = rp.reference_arrays(ref, subset_size=21, subset_stride=10)
    gw, gh = 1 + (W - 21) // 10, 1 + (H - 21) // 10
    rng = np.random.default_rng(10 + size)
    state = np.zeros((gh, gw, 8), np.float32)
    state[..., :6] = rng.normal(0, 0.1, (gh, gw, 6))
    state[..., 6] = rng.choice(np.array([1.0, 0.0, -1.0], np.float32), (gh, gw))
    with ICGNWGPU(subset_size=21, subset_stride=10, outlier_policy="median", median_filter_size=size,
                  median_filter_scope="all") as engine:
        engine.set_reference_arrays(W, H, plane, metadata, inverse)
        got = engine.apply_outlier_filter(state)
    expected = oracle_c.uod(state.reshape(-1, 8), metadata, grid=(gw, gh), subset_stride=10, policy="median",
                            median_size=size, scope_all=True)
    np.testing.assert_array_equal(got.reshape(-1, 8), expected)


def test_register_with_uod_matches_oracle_pipeline(pair):
    ref, tgt = pair
    plane, inverse, metadata = rp.reference_arrays(ref, subset_size=21, subset_stride=10)
    gw, gh = 1 + (W - 21) // 10, 1 + (H - 21) // 10
    with ICGNWGPU(subset_size=21, subset_stride=10) as engine:
        engine.set_reference_arrays(W, H, plane, metadata, inverse)
        result = engine.register(tgt)
    coef = oracle_c.prefilter(tgt, rp.runtime_fir_taps())
    raw = oracle_c.solve(tgt, coef, plane, metadata, inverse, subset_size=21, subset_stride=10, lanes=16)
    expected = oracle_c.uod(raw, metadata, grid=(gw, gh), subset_stride=10, policy="replace")
    np.testing.assert_array_equal(_packed(result), expected.reshape(gh, gw, 8))


def test_final_zncc_matches_oracle(pair):
    ref, tgt = pair
    plane, inverse, metadata = rp.reference_arrays(ref, subset_size=21, subset_stride=10)
    gw, gh = 1 + (W - 21) // 10, 1 + (H - 21) // 10
    with ICGNWGPU(subset_size=21, subset_stride=10) as engine:
        engine.set_reference_arrays(W, H, plane, metadata, inverse)
        result = engine.register(tgt, include_zncc=True)
    coef = oracle_c.prefilter(tgt, rp.runtime_fir_taps())
    state = _packed(result).reshape(-1, 8)
    expected = oracle_c.final_zncc(tgt, coef, plane, state, subset_size=21, subset_stride=10, lanes=64)
    expected[expected < -1.0] = np.nan
    np.testing.assert_array_equal(result.zncc.ravel(), expected)
    assert np.nanmin(result.zncc[result.status == 1]) > 0.8


@pytest.mark.parametrize("width,height", [(3840, 2160), (1920, 1080), (161, 143), (64, 18), (130, 35)])
def test_reduce_half_bit_exact(width, height):
    """Pyramid reduction (full_pyramid.wgsl reduce_fused, exact integer 5x5 / 256)."""
    import torch

    from live_dic_gb300 import _native

    rng = np.random.default_rng(width * 7 + height)
    img = rng.integers(0, 256, size=(height, width), dtype=np.uint8)
    src = torch.from_numpy(img).cuda()
    dst = torch.empty((height // 2, width // 2), dtype=torch.uint8, device="cuda")
    lib = _native.load()
    _native.check(lib.gbdic_reduce_half(src.data_ptr(), width, height, dst.data_ptr(), None),
                  lib.gbdic_last_error(None))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dst.cpu().numpy(), oracle_c.reduce(img))
