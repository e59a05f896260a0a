"""Host-side behaviour that needs no GPU: the C ABI surface, argument
validation before any device work (as the reference's portable tests pin,
DIC/LucasKanadeICGN/python/tests/test_wgpu_backend.py:57-231), input
normalisation and ROI planning against the reference's golden vectors,
result views, and the multi-process replica aggregation of bench.py."""

from __future__ import annotations

import ctypes
import os
import re
from pathlib import Path

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPU, ICGNWGPUFullPyramid, _native, roi
from live_dic_gb300.engine import _as_uint8_gray, result_from_packed

ROOT = Path(__file__).resolve().parents[1]


def test_library_exports_every_declared_symbol():
    header = (ROOT / "include" / "gbdic.h").read_text()
    declared = set(re.findall(r"^(?:int|void|const char \*)\s*\**\s*(gbdic_\w+)\(", header, flags=re.M))
    assert len(declared) >= 30
    lib = ctypes.CDLL(str(_native.LIBRARY_PATH))
    for name in sorted(declared):
        assert hasattr(lib, name), name
    assert declared == set(_native.EXPORTED_SYMBOLS)
    assert _native.load().gbdic_abi_version() == 2


@pytest.mark.parametrize(
    "kwargs,message",
    [
        ({"motion_model": "spline"}, "motion_model"),
        ({"interpolation": "nearest"}, "interpolation"),
        ({"outlier_policy": "drop"}, "outlier_policy"),
        ({"median_filter_size": 4}, "median_filter_size"),
        ({"median_filter_scope": "all"}, "median_filter_scope"),
        ({"median_filter_size": 5}, "median_filter_size"),
        ({"subset_size": 3}, "subset_size"),
        ({"subset_size": 46341}, "subset_size"),
        ({"subset_size": 16, "subset_stride": 17}, "subset_stride"),
        ({"subset_stride": True}, "subset_stride"),
        ({"spatial_weighting": "triangle"}, "spatial_weighting"),
        ({"spatial_weighting": "gaussian", "gaussian_sigma": 0.0}, "gaussian_sigma"),
        ({"solver_workgroup_size": 48}, "solver_workgroup_size"),
        ({"pyramid_levels": 4}, "pyramid_levels"),
        ({"pyramid_levels": True}, "pyramid_levels"),
        ({"device_type": "tpu"}, "device_type"),
        ({"power_preference": "max"}, "power_preference"),
        ({"prefer_subgroups": True, "subset_size": 32}, "prefer_subgroups"),
        ({"solver_mode": "tiled"}, "solver_mode"),
        ({"solver_mode": 2}, "solver_mode"),
    ],
)
def test_engine_validation_before_device_work(kwargs, message):
    with pytest.raises(ValueError, match=message):
        ICGNWGPU(**kwargs)


@pytest.mark.parametrize(
    "kwargs,message",
    [
        ({"pyramid_levels": 5}, "pyramid_levels"),
        ({"iterations_per_level": (8,)}, "iterations_per_level"),
        ({"iterations_per_level": (0, 16)}, "iterations"),
        ({"tolerance_per_level": (1e-2, -1.0)}, "tolerance"),
        ({"initialization": "random"}, "initialization"),
        ({"temporal_prediction": "velocity"}, "temporal_prediction"),
        ({"temporal_max_age": -1}, "temporal_max_age"),
        ({"pyramid_policy": "adaptive"}, "adaptive"),
        ({"adaptive_acceptance": 1.5}, "adaptive_acceptance"),
        ({"seed_search_radius": 0, "initialization": "zncc"}, "seed_search_radius"),
        ({"seed_search_radius": 4}, "seed_search_radius"),
        ({"divergence_patience": 31}, "divergence_patience"),
    ],
)
def test_full_pyramid_validation_before_device_work(kwargs, message):
    with pytest.raises(ValueError, match=message):
        ICGNWGPUFullPyramid(**kwargs)


def test_input_normalisation_matches_reference(golden):
    np.testing.assert_array_equal(_as_uint8_gray(golden["gray_float_in"]), golden["gray_float_out"])
    np.testing.assert_array_equal(_as_uint8_gray(golden["gray_wide_in"]), golden["gray_wide_out"])
    with pytest.raises(ValueError, match="at least 16"):
        _as_uint8_gray(np.zeros((8, 32), np.uint8))
    with pytest.raises(ValueError, match=r"\[0, 255\]"):
        _as_uint8_gray(np.full((20, 20), 300, np.int32))
    rgb = np.random.default_rng(0).integers(0, 256, (20, 20, 3), dtype=np.uint8)
    luma = _as_uint8_gray(rgb)
    assert luma.shape == (20, 20) and luma.dtype == np.uint8


def test_roi_planning_matches_reference(golden):
    mask = golden["roi_mask"]
    plan = roi.prepare_roi(mask, 21, 10)
    np.testing.assert_array_equal(plan.selected, golden["roi_selected"])
    np.testing.assert_array_equal(plan.neighbour_bits, golden["roi_neighbour_bits"])
    np.testing.assert_array_equal(roi.prepare_roi(mask, 21, 10, median_filter_size=9).median_neighbour_words,
                                  golden["roi_median_words"])
    coarse_mask = roi.reduce_mask(mask)
    np.testing.assert_array_equal(coarse_mask, golden["roi_reduced_mask"])
    coarse = roi.prepare_roi(coarse_mask, 21, 10)
    np.testing.assert_array_equal(coarse.selected, golden["roi_coarse_selected"])
    np.testing.assert_array_equal(
        roi.seed_permissions(coarse, plan, source_scale=2, destination_scale=1, size=21, stride=10,
                             reference_mask=mask),
        golden["roi_seed_permissions"],
    )
    np.testing.assert_array_equal(
        roi.seed_permissions(plan, coarse, source_scale=1, destination_scale=2, size=21, stride=10,
                             reference_mask=mask),
        golden["roi_temporal_permissions"],
    )
    with pytest.raises(TypeError):
        roi.validate_roi(mask.astype(np.uint8), "full", mask.shape, "affine")
    with pytest.raises(ValueError, match="translation and affine"):
        roi.validate_roi(mask, "full", mask.shape, "quadratic")


def test_result_views_statistics_and_archive(tmp_path):
    packed = np.zeros((3, 4, 8), np.float32)
    packed[..., 0] = 0.5
    packed[..., 3] = -0.25
    packed[..., 6] = 1.0
    packed[..., 7] = 3.0
    packed[0, 0, 6] = 2.0
    packed[2, 3, 6] = -1.0
    result = result_from_packed(packed, motion_model="affine", timing={"totalWallMs": 1.0},
                                config={"motionModel": "affine"}, width=64, height=48, subset_size=16,
                                subset_stride=16)
    assert result.accepted == 11 and result.replaced == 1
    assert result.mean_translation == (0.5, -0.25)
    result.displacement[1, 1, 0] = 7.0  # zero-copy view of the packed field
    assert packed[1, 1, 0] == 7.0
    assert result.rmse((0.5, -0.25)) > 0
    assert result.populations["accepted"] == 11
    path = tmp_path / "field.npz"
    result.save_npz(path)
    with np.load(path) as archive:
        assert archive["parameters"].shape == (3, 4, 6)
        assert tuple(archive["parameter_order"]) == result.parameter_order


def test_autotune_acceptance_rule():
    from live_dic_gb300.autotune import compare_solver_outputs

    rng = np.random.default_rng(1)
    base = np.zeros((20, 30, 8), np.float32)
    base[..., :6] = rng.normal(0, 0.1, (20, 30, 6))
    base[..., 6] = 1.0
    ok = compare_solver_outputs(base, base + np.float32(1e-5) * (np.arange(8) < 6))
    assert ok["valid"] and ok["parameter_max_abs"] < 2e-5
    far = base.copy()
    far[..., 0] += 0.05
    assert compare_solver_outputs(base, far)["reason"] == "parameters disagree"
    flipped = base.copy()
    flipped[:5, :, 6] = 0.0
    assert compare_solver_outputs(base, flipped)["reason"] == "accepted subset masks disagree"
    nan = base.copy()
    nan[0, 0, 0] = np.nan
    assert compare_solver_outputs(base, nan)["reason"] == "non-finite solver output"


def _replica_worker(rank, world, port, out):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    value = bench.job_throughput(steps=10, local_ms=100.0 * (rank + 1), world=world, dist=dist, device="cpu")
    out[rank] = value
    dist.destroy_process_group()
    del torch


def test_bench_replica_throughput_two_gloo_ranks():
    import torch.multiprocessing as mp

    manager = mp.Manager()
    out = manager.dict()
    port = 29500 + (os.getpid() % 1000)
    mp.spawn(_replica_worker, args=(2, port, out), nprocs=2, join=True)
    # both ranks see the slowest rank's time: 2 replicas x 10 frames / 0.2 s
    assert out[0] == pytest.approx(100.0) and out[1] == pytest.approx(100.0)


@pytest.mark.parametrize(
    "kwargs,message",
    [
        ({"solver_workgroup_size": 48}, "solver_workgroup_size"),
        ({"solver_workgroup_size": True}, "solver_workgroup_size"),
        ({"mode": "sequential"}, "mode"),
        ({"ctas_per_sm": 33}, "ctas_per_sm"),
    ],
)
def test_batch_validation_before_device_work(kwargs, message):
    from live_dic_gb300 import ICGNBatch

    with pytest.raises(ValueError, match=message):
        ICGNBatch(**kwargs)


def test_uneven_workload_generator():
    from live_dic_gb300 import synthetic

    pairs = synthetic.uneven_workload(4, count=5, sizes=((96, 80), (128, 96)), subsets=(15, 21), device="cpu")
    assert len(pairs) == 5
    for p in pairs:
        h, w = p["reference"].shape
        assert p["target"].shape == (h, w) and p["target"].dtype == np.uint8
        assert p["subset_stride"] == p["subset_size"] // 3
        assert (p["roi_mask"] is None) == (p["motion_model"] == "quadratic")
        gy, gx = np.mgrid[0:h:8, 0:w:8].astype(np.float64)
        u, v = p["field"](gx, gy)
        assert np.sqrt(u * u + v * v).max() == pytest.approx(p["field_params"]["peak"], rel=1e-9)
        assert 0.5 <= p["field_params"]["peak"] <= 3.0


@pytest.mark.parametrize("k", range(4))
def test_recovery_reduction_matches_reference(golden, k):
    from live_dic_gb300.pyramid_recovery import reduce_half

    np.testing.assert_array_equal(reduce_half(golden[f"reduce_{k}_in"]), golden[f"reduce_{k}_half"])


@pytest.mark.parametrize("model", ["affine", "quadratic"])
def test_recovery_seed_transfer_matches_reference(golden, model):
    from live_dic_gb300.pyramid_recovery import pyramid_dependency_mask, transfer_pyramid_seed

    requested = golden[f"transfer_{model}_requested"]
    seeds, active = transfer_pyramid_seed(
        golden[f"transfer_{model}_params"], golden[f"transfer_{model}_status"], motion_model=model,
        source_available=golden[f"transfer_{model}_available"], source_scale=2, destination_scale=1,
        destination_grid=(17, 13), requested=requested, subset_size=21, subset_stride=10)
    np.testing.assert_allclose(seeds, golden[f"transfer_{model}_seeds"], rtol=1e-6, atol=1e-7)
    np.testing.assert_array_equal(active, golden[f"transfer_{model}_active"])
    status = golden[f"transfer_{model}_status"]
    closure = pyramid_dependency_mask(source_grid=(status.shape[1], status.shape[0]), source_scale=2,
                                      destination_scale=1, requested=requested, subset_size=21, subset_stride=10)
    assert closure.shape == status.shape and closure.any()


@pytest.mark.parametrize("truncation", ["none", "visibility"])
def test_partial_roi_planning_matches_reference(truncation):
    g = np.load(ROOT / "tests" / "golden" / "partial_vectors.npz")
    plan = roi.prepare_roi(g["partial_mask"], 21, 10, policy="partial", truncation=truncation)
    np.testing.assert_array_equal(plan.selected, g[f"partial_{truncation}_selected"])
    np.testing.assert_array_equal(plan.partial_indices, g[f"partial_{truncation}_indices"])
    np.testing.assert_array_equal(plan.support_words, g[f"partial_{truncation}_words"])
    np.testing.assert_array_equal(plan.support_boxes, g[f"partial_{truncation}_boxes"])
    np.testing.assert_array_equal(plan.neighbour_bits, g[f"partial_{truncation}_bits"])


def test_partial_reference_preparation_matches_reference():
    from live_dic_gb300.partial import prepare_partial_reference

    g = np.load(ROOT / "tests" / "golden" / "partial_vectors.npz")
    plan = roi.prepare_roi(g["partial_mask"], 21, 10, policy="partial")
    metadata = g["partial_metadata_in"].copy()
    inverse = g["partial_inverse_in"].copy()
    updated = prepare_partial_reference(g["partial_plane"], inverse, metadata, plan, width=170, height=150, size=21,
                                        stride=10, motion_model="affine", weighting="uniform", sigma=5.25)
    np.testing.assert_array_equal(metadata, g["partial_metadata_out"])
    np.testing.assert_array_equal(inverse, g["partial_inverse_out"])
    np.testing.assert_array_equal(updated.support_rank, g["partial_rank"])
    np.testing.assert_allclose(updated.support_condition, g["partial_condition"], rtol=1e-12)


@pytest.mark.parametrize("model", ["affine", "quadratic"])
def test_result_summary_matches_numpy_selection(model):
    """RegistrationResult counts and FP64 means (engine.py:106-327) from the
    library's one-pass summary equal the boolean-selection formulas."""
    from live_dic_gb300.engine import result_from_packed

    rng = np.random.default_rng(17)
    stride, n = (16, 12) if model == "quadratic" else (8, 6)
    packed = rng.normal(size=(37, 53, stride)).astype(np.float32)
    packed[..., n] = rng.choice([2.0, 1.0, 0.0, -1.0, -3.0, np.nan], size=(37, 53),
                                p=[0.05, 0.8, 0.05, 0.04, 0.04, 0.02]).astype(np.float32)
    r = result_from_packed(packed, motion_model=model, timing={}, config={}, width=600, height=400,
                           subset_size=21, subset_stride=10)
    mask = packed[..., n] > 0.5
    assert r.accepted == int(mask.sum())
    assert r.replaced == int((packed[..., n] > 1.5).sum())
    assert r.mean_translation == (float(np.mean(packed[..., 0][mask], dtype=np.float64)),
                                  float(np.mean(packed[..., 3][mask], dtype=np.float64)))
    assert r.mean_iterations == float(np.mean(packed[..., n + 1][mask], dtype=np.float64))
    assert np.shares_memory(r.parameters, packed)


def test_package_exports_cover_the_reference_api():
    """live_dic.__all__ (__init__.py:21-41) without the headless-browser engine."""
    import live_dic_gb300

    expected = {"BenchmarkResult", "AFFINE_PARAMETER_ORDER", "DEFAULT_IN_FLIGHT_FRAMES", "DEFAULT_FULL_PYRAMID_LEVELS",
                "DEFAULT_PYRAMID_LEVELS", "EngineInfo", "ImageInput", "ICGNError", "ICGNWGPU",
                "ICGNWGPUFullPyramid", "MOTION_MODELS", "OUTLIER_POLICIES", "PARAMETER_ORDER",
                "QUADRATIC_PARAMETER_ORDER", "ReferenceInfo", "RegistrationResult", "SEEDED_SOLVE_API_VERSION",
                "register_pair"}
    assert expected <= set(live_dic_gb300.__all__)
    assert live_dic_gb300.SEEDED_SOLVE_API_VERSION == 1


def test_register_pair_argument_errors():
    from live_dic_gb300 import ICGNError, register_pair

    image = np.zeros((64, 64), np.uint8)
    with pytest.raises(ValueError, match="ROI requires"):
        register_pair(image, image, roi_mask=np.ones((64, 64), bool))
    with pytest.raises(ValueError, match="ROI requires"):
        register_pair(image, image, roi_policy="partial")
    with pytest.raises(ICGNError, match="CUDA engine"):
        register_pair(image, image, backend="regl")


@pytest.mark.parametrize("case", [0, 1, 2])
def test_roi_planning_matches_reference_on_harder_masks(case):
    """Several holes and cut edges, odd and even windows, overlapping and
    tiled grids: selection, 3x3 bits, every median lattice, the mask hash,
    both partial truncations, the reduced mask and the seed permissions in
    both directions, against the reference's own outputs."""
    g = np.load(ROOT / "tests" / "golden" / "roi_vectors.npz")
    k = f"roi{case}"
    mask = g[f"{k}_mask"]
    size, stride = (int(v) for v in g[f"{k}_geometry"])
    plan = roi.prepare_roi(mask, size, stride)
    np.testing.assert_array_equal(plan.selected, g[f"{k}_selected"])
    np.testing.assert_array_equal(plan.neighbour_bits, g[f"{k}_bits"])
    assert plan.mask_hash == bytes(g[f"{k}_hash"]).decode()
    for median in (5, 7, 9):
        np.testing.assert_array_equal(roi.prepare_roi(mask, size, stride, median_filter_size=median)
                                      .median_neighbour_words, g[f"{k}_median{median}"])
    for truncation in ("none", "visibility"):
        partial = roi.prepare_roi(mask, size, stride, policy="partial", truncation=truncation)
        for name in ("selected", "partial_indices", "support_words", "support_boxes", "coverage", "neighbour_bits"):
            got, want = getattr(partial, name), g[f"{k}_partial_{truncation}_{name}"]
            assert got.dtype == want.dtype, name
            np.testing.assert_array_equal(got, want, err_msg=name)
    coarse_mask = roi.reduce_mask(mask)
    np.testing.assert_array_equal(coarse_mask, g[f"{k}_reduced"])
    coarse = roi.prepare_roi(coarse_mask, size, stride)
    np.testing.assert_array_equal(roi.seed_permissions(coarse, plan, source_scale=2, destination_scale=1, size=size,
                                                       stride=stride, reference_mask=mask), g[f"{k}_down"])
    np.testing.assert_array_equal(roi.seed_permissions(plan, coarse, source_scale=1, destination_scale=2, size=size,
                                                       stride=stride, reference_mask=mask), g[f"{k}_up"])


def test_solver_modes_and_autotuner_axes():
    """Pixel-loop modes accepted by the engines and the autotuner's axes:
    lanes, work distribution, and the staging axis (L1, register window,
    TMA-staged tile) with its two tile shapes."""
    from live_dic_gb300 import autotune
    from live_dic_gb300.native_backend import normalize_solver_mode

    for mode in ("exact", "fast", "staged", "staged-wide"):
        assert normalize_solver_mode(mode) == mode
        assert _native.SOLVER_MODES[mode] in (0, 1, 2, 3)
    modes = {m for _, _, m in autotune.CANDIDATES}
    assert modes == {"exact", "fast", "staged", "staged-wide"}
    assert len(autotune.CANDIDATES) == len(set(autotune.CANDIDATES)) == 18
    assert {(lanes, persistent) for lanes, persistent, m in autotune.CANDIDATES if m == "staged"} == {
        (16, False), (32, False), (16, True), (32, True)}
    assert autotune.variant_name(16, False, "staged-wide") == "16-lane grid staged-wide"


def test_batch_modes_and_split_k_choice():
    """The batch step modes (single persistent launch by default) and the
    inference network's split-K choice: the smallest divisor of the K
    blocks that fills one wave of output tiles, 1 when the tiles do."""
    from live_dic_gb300 import batch, learned

    assert batch._MODES == {"persistent": _native.BATCH_PERSISTENT, "per-job": _native.BATCH_PER_JOB,
                            "single": _native.BATCH_SINGLE}
    C = learned._Conv
    # (cin, cout, H, OH, kp, kp_rows, kt, M, Min) at batch 512: conv4 and conv5
    conv4 = C(128, 128, 8, 4, 1152, 1152, 1152, 512 * 16, 512 * 64)
    conv5 = C(128, 64, 4, 2, 1152, 1152, 576, 512 * 4, 512 * 16)
    conv2 = C(32, 64, 32, 16, 320, 384, 576, 512 * 256, 512 * 1024)
    assert learned.SeedNet._forward_splits(conv4) == 3   # 64 tiles -> 192
    assert learned.SeedNet._forward_splits(conv5) == 18  # 16 tiles -> 288
    assert learned.SeedNet._forward_splits(conv2) == 1   # 1024 tiles fill the GPU
