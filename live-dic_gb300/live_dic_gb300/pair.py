"""One-shot registration and the browser-engine record types, for callers of
live_dic's package-level API (engine.py:61-79, 331-362, 1522-1574).

The reference's register_pair drives its headless-browser engine; here the
pair runs on the CUDA full-pyramid engine with the same arguments.  The
browser-only settings (repo_root, chromium, backend, global_affine_levels)
have no effect on the CUDA path: a non-default backend or affine level count
raises ICGNError instead of silently running a different solver.  ROI
arguments raise the reference's ValueError.
"""

from __future__ import annotations

import os
from collections.abc import Iterable
from dataclasses import dataclass

import numpy as np

from .engine import ICGNError, ImageInput, RegistrationResult
from .full_pyramid_backend import DEFAULT_FULL_PYRAMID_LEVELS, ICGNWGPUFullPyramid


@dataclass(frozen=True, slots=True)
class EngineInfo:
    """Properties of an engine runtime (the reference's browser engine record)."""

    width: int
    height: int
    grid: tuple[int, int]
    subset_size: int
    subset_stride: int
    device: str
    timer_query: bool
    solver: str = "unknown"
    subgroup_width: int = 0
    subgroup_probe_width: int = 0
    subgroup_solver_width: int = 0
    subgroup_validation: str = "unavailable"
    motion_model: str = "affine"
    outlier_policy: str = "replace"
    median_filter_scope: str = "rejected"


@dataclass(frozen=True, slots=True)
class BenchmarkResult:
    """Timing distribution and final registration of a benchmark run."""

    repeats: int
    warmups: int
    gpu_times_ms: np.ndarray
    wall_times_ms: np.ndarray
    gpu_median_ms: float | None
    gpu_p95_ms: float | None
    wall_median_ms: float
    wall_p95_ms: float
    device: str
    registration: RegistrationResult


def register_pair(
    reference: ImageInput,
    target: ImageInput,
    *,
    repo_root: str | os.PathLike[str] | None = None,
    chromium: str | os.PathLike[str] | None = None,
    backend: str = "three-tsl",
    pyramid_levels: int | None = None,
    iterations_per_level: Iterable[int] | None = None,
    tolerance_per_level: Iterable[float] | None = None,
    interpolation: str = "bspline",
    motion_model: str = "affine",
    outlier_policy: str = "replace",
    median_filter_size: int = 3,
    subset_size: int = 31,
    subset_stride: int | None = None,
    initialization: str = "zero",
    global_affine_levels: int = 5,
    iterations: int | None = None,
    tolerance: float | None = None,
    zncc_min: float | None = None,
    roi_mask: np.ndarray | None = None,
    roi_policy: str = "full",
    roi_truncation: str = "none",
) -> RegistrationResult:
    """Run a one-shot registration and release the engine afterward."""
    if roi_mask is not None or roi_policy != "full" or roi_truncation != "none":
        raise ValueError("ROI requires ICGNWGPU or ICGNWGPUFullPyramid")
    if backend not in ("three-tsl", "webgpu-wgsl") or global_affine_levels != 5:
        raise ICGNError("register_pair runs on the CUDA engine; browser backends and global_affine_levels are "
                        "not available in this build")
    levels = DEFAULT_FULL_PYRAMID_LEVELS if pyramid_levels is None else pyramid_levels
    if iterations is not None and iterations_per_level is None:
        iterations_per_level = (int(iterations),) * int(levels)
    if tolerance is not None and tolerance_per_level is None:
        tolerance_per_level = (float(tolerance),) * int(levels)
    with ICGNWGPUFullPyramid(
        pyramid_levels=levels,
        iterations_per_level=None if iterations_per_level is None else tuple(iterations_per_level),
        tolerance_per_level=None if tolerance_per_level is None else tuple(tolerance_per_level),
        interpolation=interpolation,
        motion_model=motion_model,
        outlier_policy=outlier_policy,
        median_filter_size=median_filter_size,
        subset_size=subset_size,
        subset_stride=subset_stride,
        initialization=initialization,
        pipeline_slots=1,
    ) as engine:
        engine.set_reference(reference, zncc_min=0.8 if zncc_min is None else float(zncc_min))
        return engine.register(target)
