"""ctypes front end of the C oracle (icgn_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, by __graft_entry__.smoke() as the
checker and by bench.py's CPU-baseline leg.  The product package never
imports it.  `build()` compiles oracle/_build/liboracle.so with the
committed Makefile (gcc, OpenMP, -ffp-contract=off).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
MODELS = {"affine": 0, "translation": 1, "quadratic": 2}
INTERPOLATIONS = {"bspline": 0, "linear": 1, "cubic": 2}
POLICIES = {"flag": 0, "replace": 1, "median": 3}

_lib = None


def build(force: bool = False) -> Path:
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < (HERE / "icgn_oracle.c").stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


class SolveCfg(C.Structure):
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int),
        ("grid_w", C.c_int), ("grid_h", C.c_int),
        ("subset_size", C.c_int), ("subset_stride", C.c_int),
        ("model", C.c_int), ("interp", C.c_int), ("lanes", C.c_int),
        ("iterations", C.c_int),
        ("tolerance", C.c_float), ("zncc_min", C.c_float),
        ("roi_enabled", C.c_int),
        ("divergence_patience", C.c_int), ("divergence_min_iterations", C.c_int),
        ("weights", C.POINTER(C.c_float)),
        ("weight_sum", C.c_float),
    ]


class UodCfg(C.Structure):
    _fields_ = [
        ("grid_w", C.c_int), ("grid_h", C.c_int),
        ("subset_stride", C.c_int),
        ("model", C.c_int), ("policy", C.c_int),
        ("median_size", C.c_int), ("scope_all", C.c_int), ("seed_mode", C.c_int),
        ("roi_enabled", C.c_int),
        ("permissions", C.POINTER(C.c_float)),
        ("meta", C.POINTER(C.c_float)),
    ]


class SeedCfg(C.Structure):
    _fields_ = [
        ("src_grid_w", C.c_int), ("src_grid_h", C.c_int),
        ("dst_grid_w", C.c_int), ("dst_grid_h", C.c_int),
        ("src_scale", C.c_float), ("dst_scale", C.c_float),
        ("subset_size", C.c_float), ("subset_stride", C.c_float),
        ("model", C.c_int), ("track_availability", C.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB_PATH))
    return _lib


def _p(array, ctype=C.c_float):
    if array is None:
        return None
    return array.ctypes.data_as(C.POINTER(ctype))


def set_threads(count: int) -> None:
    os.environ["OMP_NUM_THREADS"] = str(count)


def prefilter(image: np.ndarray, taps25: np.ndarray) -> np.ndarray:
    img = np.ascontiguousarray(image, dtype=np.uint8)
    h, w = img.shape
    coef = np.empty((h, w), np.float32)
    scratch = np.empty((h, w), np.float32)
    taps = np.ascontiguousarray(taps25, dtype=np.float32)
    lib().oracle_prefilter(_p(img, C.c_uint8), w, h, _p(taps), _p(coef), _p(scratch))
    return coef


def solve(
    image: np.ndarray,
    coef: np.ndarray | None,
    plane: np.ndarray,
    metadata: np.ndarray,
    inverse: np.ndarray,
    *,
    subset_size: int,
    subset_stride: int,
    model: str = "affine",
    interpolation: str = "bspline",
    lanes: int = 32,
    iterations: int = 30,
    tolerance: float = 1e-3,
    zncc_min: float = 0.8,
    roi_enabled: bool = False,
    weights: np.ndarray | None = None,
    seed_state: np.ndarray | None = None,
    active: np.ndarray | None = None,
    preserve_disabled: bool = False,
    state: np.ndarray | None = None,
    subsets: np.ndarray | None = None,
    divergence_patience: int = 0,
    divergence_min_iterations: int = 4,
    partial: tuple | None = None,
) -> np.ndarray:
    """`partial` = (indices, support words, boxes): solve only those partial
    windows with their supports (into `state`)."""
    img = np.ascontiguousarray(image, dtype=np.uint8)
    h, w = img.shape
    gw = 1 + (w - subset_size) // subset_stride
    gh = 1 + (h - subset_size) // subset_stride
    stride = 16 if model == "quadratic" else 8
    if state is None:
        state = np.zeros((gh * gw, stride), np.float32)
    cfg = SolveCfg()
    cfg.width, cfg.height, cfg.grid_w, cfg.grid_h = w, h, gw, gh
    cfg.subset_size, cfg.subset_stride = subset_size, subset_stride
    cfg.model, cfg.interp, cfg.lanes = MODELS[model], INTERPOLATIONS[interpolation], lanes
    cfg.iterations, cfg.tolerance, cfg.zncc_min = iterations, tolerance, zncc_min
    cfg.roi_enabled = int(roi_enabled)
    cfg.divergence_patience = divergence_patience
    cfg.divergence_min_iterations = divergence_min_iterations
    meta = np.ascontiguousarray(metadata, dtype=np.float32).ravel()
    wts = None
    if weights is not None:
        wts = np.ascontiguousarray(weights, dtype=np.float32).ravel()
        cfg.weights = _p(wts)
        n = 12 if model == "quadratic" else 6
        cfg.weight_sum = float(meta.reshape(gh * gw, -1)[0, 3 + 2 * n])
    coef_arr = None if coef is None else np.ascontiguousarray(coef, dtype=np.float32)
    pl = np.ascontiguousarray(plane, dtype=np.float32).ravel()
    inv = np.ascontiguousarray(inverse, dtype=np.float32).ravel()
    seed = None if seed_state is None else np.ascontiguousarray(seed_state, dtype=np.float32).reshape(-1)
    act = None if active is None else np.ascontiguousarray(active, dtype=np.uint32).ravel()
    sub = None if subsets is None else np.ascontiguousarray(subsets, dtype=np.int32)
    if partial is not None:
        indices, words, boxes = partial
        idx = np.ascontiguousarray(indices, dtype=np.int32)
        wds = np.ascontiguousarray(words, dtype=np.uint32)
        bxs = np.ascontiguousarray(boxes, dtype=np.float32)
        lib().oracle_solve_partial(
            C.byref(cfg), _p(img, C.c_uint8), _p(coef_arr), _p(pl), _p(meta), _p(inv), _p(seed),
            _p(act, C.c_uint32), _p(idx, C.c_int32), int(idx.size), _p(wds, C.c_uint32),
            int(wds.shape[1]) if wds.ndim == 2 else 0, _p(bxs), _p(state))
        return state
    lib().oracle_solve(
        C.byref(cfg), _p(img, C.c_uint8), _p(coef_arr), _p(pl), _p(meta), _p(inv),
        _p(seed), _p(act, C.c_uint32), int(preserve_disabled),
        _p(sub, C.c_int32), 0 if sub is None else int(sub.size), _p(state),
    )
    return state


def uod(
    state: np.ndarray,
    metadata: np.ndarray,
    *,
    grid: tuple[int, int],
    subset_stride: int,
    model: str = "affine",
    policy: str = "replace",
    median_size: int = 3,
    scope_all: bool = False,
    seed_mode: bool = False,
    permissions: np.ndarray | None = None,
) -> np.ndarray:
    gw, gh = grid
    src = np.ascontiguousarray(state, dtype=np.float32)
    out = np.empty_like(src)
    cfg = UodCfg()
    cfg.grid_w, cfg.grid_h, cfg.subset_stride = gw, gh, subset_stride
    cfg.model, cfg.policy = MODELS[model], POLICIES[policy]
    cfg.median_size, cfg.scope_all, cfg.seed_mode = median_size, int(scope_all), int(seed_mode)
    perm = None
    if permissions is not None:
        perm = np.ascontiguousarray(permissions, dtype=np.float32).reshape(-1)
        cfg.roi_enabled = 1
        cfg.permissions = _p(perm)
    meta = np.ascontiguousarray(metadata, dtype=np.float32).ravel()
    cfg.meta = _p(meta)
    lib().oracle_uod(C.byref(cfg), _p(src), _p(out))
    return out


def reduce(image: np.ndarray) -> np.ndarray:
    img = np.ascontiguousarray(image, dtype=np.uint8)
    h, w = img.shape
    out = np.empty((h // 2, w // 2), np.uint8)
    lib().oracle_reduce(_p(img, C.c_uint8), w, h, _p(out, C.c_uint8))
    return out


def transfer_seed(
    source_state: np.ndarray,
    *,
    source_grid: tuple[int, int],
    destination_grid: tuple[int, int],
    source_scale: float,
    destination_scale: float,
    subset_size: int,
    subset_stride: int,
    model: str = "affine",
    permissions: np.ndarray | None = None,
    track_availability: bool = False,
    return_weights: bool = False,
):
    """Seeds and activity of the destination grid (and, with
    `return_weights`, each destination's interpolation weight sum)."""
    cfg = SeedCfg()
    cfg.src_grid_w, cfg.src_grid_h = source_grid
    cfg.dst_grid_w, cfg.dst_grid_h = destination_grid
    cfg.src_scale, cfg.dst_scale = source_scale, destination_scale
    cfg.subset_size, cfg.subset_stride = subset_size, subset_stride
    cfg.model, cfg.track_availability = MODELS[model], int(track_availability)
    stride = 16 if model == "quadratic" else 8
    count = destination_grid[0] * destination_grid[1]
    seeds = np.zeros((count, stride), np.float32)
    active = np.zeros(count, np.uint32)
    src = np.ascontiguousarray(source_state, dtype=np.float32)
    perm = None if permissions is None else np.ascontiguousarray(permissions, dtype=np.uint32).ravel()
    weights = np.zeros(count, np.float32)
    lib().oracle_transfer_seed(C.byref(cfg), _p(src), _p(perm, C.c_uint32), _p(seeds), _p(active, C.c_uint32),
                               _p(weights))
    return (seeds, active, weights) if return_weights else (seeds, active)


def _seed_cfg(source_grid, destination_grid, source_scale, destination_scale, subset_size, subset_stride, model,
              track_availability=False) -> SeedCfg:
    cfg = SeedCfg()
    cfg.src_grid_w, cfg.src_grid_h = source_grid
    cfg.dst_grid_w, cfg.dst_grid_h = destination_grid
    cfg.src_scale, cfg.dst_scale = source_scale, destination_scale
    cfg.subset_size, cfg.subset_stride = subset_size, subset_stride
    cfg.model, cfg.track_availability = MODELS[model], int(track_availability)
    return cfg


def refine_temporal_seed(seeds: np.ndarray, active: np.ndarray, coarse_history: np.ndarray, coarse_ages: np.ndarray,
                         history: np.ndarray, ages: np.ndarray, *, source_grid, destination_grid, source_scale: float,
                         subset_size: int, subset_stride: int, model: str = "affine", max_age: int = 0xFFFFFFFE,
                         permissions: np.ndarray | None = None) -> np.ndarray:
    """full_pyramid.wgsl refine_temporal_seed on a copy of `seeds`."""
    cfg = _seed_cfg(source_grid, destination_grid, source_scale, 1.0, subset_size, subset_stride, model, True)
    out = np.ascontiguousarray(seeds, dtype=np.float32).copy()
    perm = None if permissions is None else np.ascontiguousarray(permissions, dtype=np.uint32).ravel()
    lib().oracle_refine_temporal_seed(
        C.byref(cfg), _p(np.ascontiguousarray(coarse_history, np.float32)),
        _p(np.ascontiguousarray(coarse_ages, np.uint32), C.c_uint32), _p(perm, C.c_uint32),
        _p(np.ascontiguousarray(history, np.float32)), _p(np.ascontiguousarray(ages, np.uint32), C.c_uint32),
        C.c_uint32(max_age), _p(out), _p(np.ascontiguousarray(active, np.uint32), C.c_uint32))
    return out


def temporal_merge(history: np.ndarray, ages: np.ndarray, raw: np.ndarray, output: np.ndarray, *, model: str,
                   max_age: int, use_filtered: bool) -> tuple[int, int]:
    """In place on `history` / `ages`; returns (accepted updates, expired)."""
    acc, exp = C.c_uint32(), C.c_uint32()
    lib().oracle_temporal_merge(int(ages.size), MODELS[model], C.c_uint32(max_age), int(use_filtered), _p(history),
                                _p(ages, C.c_uint32), _p(np.ascontiguousarray(raw, np.float32)),
                                _p(np.ascontiguousarray(output, np.float32)), C.byref(acc), C.byref(exp))
    return acc.value, exp.value


def temporal_predict(history: np.ndarray, previous: np.ndarray, ages: np.ndarray, previous_ages: np.ndarray, *,
                     model: str) -> tuple[np.ndarray, int]:
    out = np.empty_like(history)
    lib().oracle_temporal_predict.restype = C.c_uint32
    n = lib().oracle_temporal_predict(int(ages.size), MODELS[model], _p(history), _p(previous), _p(ages, C.c_uint32),
                                      _p(previous_ages, C.c_uint32), _p(out))
    return out, int(n)


def temporal_save_previous(history: np.ndarray, ages: np.ndarray, raw: np.ndarray, output: np.ndarray,
                           previous: np.ndarray, previous_ages: np.ndarray, *, model: str) -> None:
    lib().oracle_temporal_save_previous(int(ages.size), MODELS[model], _p(history), _p(ages, C.c_uint32),
                                        _p(np.ascontiguousarray(raw, np.float32)),
                                        _p(np.ascontiguousarray(output, np.float32)), _p(previous),
                                        _p(previous_ages, C.c_uint32))


def seed_search(reference: np.ndarray, target: np.ndarray, *, subset_size: int, subset_stride: int, radius: int,
                model: str = "affine", seed: np.ndarray | None = None, only_missing: bool = False,
                selected: np.ndarray | None = None, centered: bool = False,
                mask: np.ndarray | None = None,
                active: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Exhaustive integer ZNCC search; returns (seed states, activity, best scores).
    `active` (or all ones) is the activity that subsets left unsearched keep."""
    ref = np.ascontiguousarray(reference, dtype=np.uint8)
    tgt = np.ascontiguousarray(target, dtype=np.uint8)
    h, w = ref.shape
    gw = 1 + (w - subset_size) // subset_stride
    gh = 1 + (h - subset_size) // subset_stride
    stride = 16 if model == "quadratic" else 8
    seeds = np.zeros((gh * gw, stride), np.float32) if seed is None else np.ascontiguousarray(seed, np.float32).copy()
    active = np.ones(gh * gw, np.uint32) if active is None else np.ascontiguousarray(active, np.uint32).ravel().copy()
    score = np.full(gh * gw, -3.0, np.float32)
    sel = None if selected is None else np.ascontiguousarray(selected, dtype=np.uint8).ravel()
    msk = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8).ravel()
    lib().oracle_seed_search_ex(
        _p(ref, C.c_uint8), _p(tgt, C.c_uint8), w, h, gw, gh, subset_size, subset_stride, radius, MODELS[model],
        int(only_missing), _p(sel, C.c_uint8), _p(seeds), _p(active, C.c_uint32), _p(score), int(centered),
        _p(msk, C.c_uint8),
    )
    return seeds, active, score


def final_zncc(image, coef, plane, state, *, subset_size, subset_stride, interpolation="bspline", lanes=64):
    img = np.ascontiguousarray(image, dtype=np.uint8)
    h, w = img.shape
    gw = 1 + (w - subset_size) // subset_stride
    gh = 1 + (h - subset_size) // subset_stride
    out = np.empty(gw * gh, np.float32)
    coef_arr = None if coef is None else np.ascontiguousarray(coef, dtype=np.float32)
    lib().oracle_final_zncc(
        w, h, gw, gh, subset_size, subset_stride, INTERPOLATIONS[interpolation], lanes,
        _p(img, C.c_uint8), _p(coef_arr), _p(np.ascontiguousarray(plane, dtype=np.float32)),
        _p(np.ascontiguousarray(state, dtype=np.float32)), _p(out),
    )
    return out


def affine_frontier(states: np.ndarray, permissions: np.ndarray, *, subset_stride: int) -> tuple[np.ndarray, np.ndarray]:
    """spatial_seed.wgsl affine_frontier on a (gh, gw, 8) snapshot; returns
    (seeds (gh, gw, 8), activity (gh, gw) bool)."""
    snap = np.ascontiguousarray(states, dtype=np.float32)
    gh, gw = snap.shape[:2]
    perms = np.ascontiguousarray(permissions, dtype=np.uint32)
    seeds = np.zeros((gh, gw, 8), np.float32)
    active = np.zeros((gh, gw), np.uint32)
    lib().oracle_affine_frontier(gh * gw, gw, subset_stride, _p(snap), _p(perms, C.c_uint32), _p(seeds),
                                 _p(active, C.c_uint32))
    return seeds, active.astype(bool)


def spatial_choose(reference: np.ndarray, target: np.ndarray, states: np.ndarray, permissions: np.ndarray, *,
                   subset_size: int, subset_stride: int, prior: np.ndarray | None = None, sample_step: int = 1,
                   min_gain: float = 0.0, min_displacement: float = 0.0, failed_only: bool = False,
                   candidate_mode: int = 0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """spatial_seed.wgsl choose; returns (seeds (gh, gw, 8), activity, scores (gh, gw, 4))."""
    ref = np.ascontiguousarray(reference, dtype=np.uint8)
    tgt = np.ascontiguousarray(target, dtype=np.uint8)
    h, w = ref.shape
    snap = np.ascontiguousarray(states, dtype=np.float32)
    gh, gw = snap.shape[:2]
    perms = np.ascontiguousarray(permissions, dtype=np.uint32)
    pri = None if prior is None else np.ascontiguousarray(prior, dtype=np.float32)
    seeds = np.zeros((gh, gw, 8), np.float32)
    scores = np.zeros((gh, gw, 4), np.float32)
    active = np.zeros((gh, gw), np.uint32)
    lib().oracle_spatial_choose(
        _p(ref, C.c_uint8), _p(tgt, C.c_uint8), w, h, gw, gh * gw, subset_size, subset_stride, sample_step,
        C.c_float(min_gain), C.c_float(min_displacement), int(failed_only), candidate_mode, _p(snap), _p(pri),
        _p(perms, C.c_uint32), _p(seeds), _p(scores), _p(active, C.c_uint32))
    return seeds, active.astype(bool), scores
