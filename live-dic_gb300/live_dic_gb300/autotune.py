"""Solver autotuner: picks lanes per subset, the work distribution and the
pixel loop.

Follows the reference's _autotune_solver (wgpu_backend.py:2213-2296): run the
baseline variant and every candidate on one representative target (the
reference shifted by (-1, +2) pixels), reject candidates whose field disagrees
with the baseline under the reference's acceptance rule
(_compare_solver_outputs, 222-299: accepted-mask mismatch <= 0.5 % of the
grid, parameter RMSE <= 2e-3, max |difference| <= 2e-2), time the rest and
keep the fastest.  Candidates: 16, 32, 64 or 128 lanes per subset with the
exact pixel loop (the reference's pixel-to-lane order), and 16 or 32 lanes
with the sliding-window loop (column runs sharing B-spline taps in
registers) or with the exact loop on TMA-staged shared-memory tiles of the
coefficient plane (staging axis; tile shape 56 x 44 or, "staged-wide",
72 x 56 floats per warp); the engine runs the last two for B-spline
translation / affine windows and falls back to the exact loop elsewhere.
Each runs as a grid launch or as a persistent grid over the work queue
(the wide tile as a grid launch only).
"""

from __future__ import annotations

import math
from collections.abc import Callable
from statistics import median

import numpy as np

CANDIDATES = tuple((lanes, persistent, "exact") for persistent in (False, True) for lanes in (16, 32, 64, 128)) + \
    tuple((lanes, persistent, "fast") for persistent in (False, True) for lanes in (16, 32)) + \
    tuple((lanes, persistent, "staged") for persistent in (False, True) for lanes in (16, 32)) + \
    tuple((lanes, False, "staged-wide") for lanes in (16, 32))


def compare_solver_outputs(portable: np.ndarray, candidate: np.ndarray) -> dict:
    """Acceptance rule of the reference for a candidate solver's field."""
    p = np.asarray(portable, dtype=np.float32).reshape(-1, portable.shape[-1])
    c = np.asarray(candidate, dtype=np.float32).reshape(-1, candidate.shape[-1])
    n_params = 12 if p.shape[1] >= 14 else 6
    status = n_params
    out = {"valid": False, "reason": "invalid result size", "accepted_portable": 0, "accepted_candidate": 0,
           "accepted_mismatch": int(p.shape[0]), "parameter_rmse": None, "parameter_max_abs": None}
    if p.shape != c.shape:
        return out
    if not (np.isfinite(p).all() and np.isfinite(c).all()):
        out["reason"] = "non-finite solver output"
        return out
    pa, ca = p[:, status] > 0.5, c[:, status] > 0.5
    mismatch = int(np.count_nonzero(pa != ca))
    out.update(accepted_portable=int(pa.sum()), accepted_candidate=int(ca.sum()), accepted_mismatch=mismatch)
    limit = max(1, int(math.ceil(p.shape[0] * 0.005)))
    if pa.sum() == 0:
        if mismatch:
            out["reason"] = "accepted subset masks disagree"
            return out
        out.update(valid=True, reason="compatible with no accepted subsets", parameter_rmse=0.0, parameter_max_abs=0.0)
        return out
    if mismatch > limit:
        out["reason"] = "accepted subset masks disagree"
        return out
    common = pa & ca
    if common.sum() == 0 or common.sum() < pa.sum() - limit:
        out["reason"] = "insufficient common accepted subsets"
        return out
    diff = c[common, :n_params].astype(np.float64) - p[common, :n_params]
    rmse = float(np.sqrt(np.mean(diff * diff)))
    mx = float(np.max(np.abs(diff)))
    out.update(parameter_rmse=rmse, parameter_max_abs=mx)
    if rmse > 2e-3 or mx > 2e-2:
        out["reason"] = "parameters disagree"
        return out
    out.update(valid=True, reason="compatible")
    return out


def variant_name(lanes: int, persistent: bool, mode: str = "exact") -> str:
    name = f"{lanes}-lane {'persistent-queue' if persistent else 'grid'}"
    return name if mode == "exact" else f"{name} {mode}"


def autotune(
    set_variant: Callable[[int, bool, str], None],
    run: Callable[[], tuple[np.ndarray, float]],
    *,
    baseline: tuple[int, bool, str] = (32, False, "exact"),
    candidates=CANDIDATES,
    repeats: int = 3,
) -> tuple[tuple[int, bool, str], dict[str, float], dict[str, dict]]:
    """Returns (best variant, median device ms per variant, validation per variant).
    A variant is (lanes, persistent, pixel loop).  `run()` registers the
    tuning target and returns (packed field, device ms)."""
    set_variant(*baseline)
    run()
    reference_field, _ = run()
    timings: dict[str, list[float]] = {}
    validation: dict[str, dict] = {}
    valid = []
    for variant in candidates:
        name = variant_name(*variant)
        set_variant(*variant)
        field, _ = run()
        check = compare_solver_outputs(reference_field, field)
        validation[name] = check
        if check["valid"]:
            valid.append(variant)
    if baseline not in valid:
        valid.insert(0, baseline)
    for repetition in range(repeats):
        order = valid if repetition % 2 == 0 else list(reversed(valid))
        for variant in order:
            set_variant(*variant)
            _, ms = run()
            timings.setdefault(variant_name(*variant), []).append(ms)
    tuning = {name: float(median(values)) for name, values in timings.items()}
    best = min(valid, key=lambda v: tuning[variant_name(*v)])
    set_variant(*best)
    return best, tuning, validation
