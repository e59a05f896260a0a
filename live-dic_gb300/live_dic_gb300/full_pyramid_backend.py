"""GPU-resident coarse-to-fine IC-GN engine (drop-in for ICGNWGPUFullPyramid).

Mirrors live_dic/full_pyramid_backend.py (158-1926): every target pyramid
level is built on the GPU, each level is solved from the transferred coarse
field, and only the finest target is uploaded and the finest field read
back.  In libgbdic.so the whole per-frame sequence is one CUDA graph per
pipeline slot.  ``initialization='temporal'`` seeds the coarsest level from
the last accepted fine field (optionally extrapolated with
``temporal_prediction='velocity'``).
"""

from __future__ import annotations

import ctypes as C
import operator
import threading
import time
from collections import deque
from collections.abc import Iterable, Iterator, Mapping
from typing import Any

import numpy as np

from . import _native
from . import autotune as _tuning
from .engine import ICGNError, ImageInput, ReferenceInfo, RegistrationResult, _as_uint8_gray, result_from_packed
from .fourier import FourierInitializer
from .interpolation import normalize_interpolation
from .motion import normalize_motion_model, parameter_count, state_float_count
from .native_backend import (DEFAULT_IN_FLIGHT_FRAMES, _normalize_device_type, _normalize_solver_workgroup_size,
                             _validated_config, native_options, normalize_solver_mode)
from .outlier import normalize_median_filter_scope, normalize_median_filter_size, normalize_outlier_policy
from .roi import immutable, integral, prepare_roi, reduce_mask, seed_permissions, validate_roi
from .subset import DEFAULT_SUBSET_SIZE, normalize_subset_size, normalize_subset_stride, subset_grid_shape
from .weighting import normalize_gaussian_sigma, normalize_spatial_weighting

DEFAULT_FULL_PYRAMID_LEVELS = 2
# Per-level iteration ceilings and tolerances, coarsest level first
# (full_pyramid_backend.py:51-62).
_DEFAULT_ITERATION_SCHEDULES = {1: (30,), 2: (8, 16), 3: (6, 8, 16), 4: (12, 8, 8, 16)}
_DEFAULT_TOLERANCES = (1e-2, 5e-3, 5e-3)
_FOUR_LEVEL_TOLERANCES = (1e-2, *_DEFAULT_TOLERANCES)
_INITIALIZATIONS = ("zero", "temporal", "fourier", "wgpu-matching", "zncc")


def _level_count(value: int) -> int:
    try:
        count = operator.index(value)
    except TypeError as error:
        raise ValueError("pyramid_levels must be an integer from 1 to 4") from error
    if isinstance(value, bool) or not 1 <= count <= 4:
        raise ValueError("pyramid_levels must be an integer from 1 to 4")
    return count


def _iteration_count(value: int, name: str) -> int:
    try:
        count = operator.index(value)
    except TypeError as error:
        raise ValueError(f"{name} must be an integer from 1 to 30") from error
    if isinstance(value, bool) or not 1 <= count <= 30:
        raise ValueError(f"{name} must be an integer from 1 to 30")
    return count


def _schedule(values, *, level_count: int, defaults, name: str):
    selected = tuple(defaults[-level_count:] if values is None else values)
    if len(selected) != level_count:
        raise ValueError(f"{name} must contain one value per pyramid level")
    return selected


class ICGNWGPUFullPyramid:
    """Full GPU-resident image pyramid with a coarse-to-fine IC-GN solve.

    ``iterations_per_level`` and ``tolerance_per_level`` are ordered from the
    coarsest to the finest level.  Reference preparation runs once per level
    in :meth:`set_reference`; per target the reductions, prefilters, solves,
    seed transfers, UOD passes and the temporal history update run as one
    CUDA graph on the device.
    """

    def __init__(
        self,
        *,
        pyramid_levels: int = DEFAULT_FULL_PYRAMID_LEVELS,
        iterations_per_level: tuple[int, ...] | None = None,
        tolerance_per_level: tuple[float, ...] | None = None,
        power_preference: str = "high-performance",
        device_type: str = "auto",
        solver_workgroup_size: int = 16,
        interpolation: str = "bspline",
        motion_model: str = "affine",
        outlier_policy: str = "replace",
        median_filter_size: int = 3,
        median_filter_scope: str = "rejected",
        subset_size: int = DEFAULT_SUBSET_SIZE,
        subset_stride: int | None = None,
        spatial_weighting: str = "uniform",
        gaussian_sigma: float | None = None,
        initialization: str = "zero",
        matching_options: Mapping[str, Any] | None = None,
        temporal_max_age: int | None = None,
        temporal_fine_correction: bool = False,
        temporal_prediction: str = "none",
        divergence_patience: int | None = None,
        divergence_min_iterations: int = 4,
        pyramid_policy: str = "fixed",
        adaptive_acceptance: float = 0.95,
        device: int = 0,
        pipeline_slots: int = DEFAULT_IN_FLIGHT_FRAMES,
        persistent: bool = False,
        seed_search_radius: int | None = None,
        autotune: bool = False,
        solver_mode: str = "exact",
    ) -> None:
        self.solver_mode = normalize_solver_mode(solver_mode)
        self._autotune = bool(autotune)
        self.solver_tuning_ms: dict[str, float] = {}
        self.solver_validation: dict[str, dict] = {}
        if not isinstance(pyramid_policy, str) or pyramid_policy not in ("fixed", "adaptive"):
            raise ValueError("pyramid_policy must be 'fixed' or 'adaptive'")
        if pyramid_policy == "adaptive" and (initialization != "temporal" or pyramid_levels != 2):
            raise ValueError("adaptive pyramid requires temporal initialization and two levels")
        if (
            isinstance(adaptive_acceptance, bool)
            or not isinstance(adaptive_acceptance, (int, float))
            or not np.isfinite(adaptive_acceptance)
            or not 0 < adaptive_acceptance <= 1
        ):
            raise ValueError("adaptive_acceptance must be finite and in (0, 1]")
        self.divergence_patience = (
            None if divergence_patience is None else _iteration_count(divergence_patience, "divergence_patience")
        )
        self.divergence_min_iterations = _iteration_count(divergence_min_iterations, "divergence_min_iterations")
        if not isinstance(temporal_prediction, str) or temporal_prediction not in ("none", "velocity"):
            raise ValueError("temporal_prediction must be 'none' or 'velocity'")
        if temporal_prediction != "none" and initialization != "temporal":
            raise ValueError("temporal_prediction requires temporal initialization")
        if not isinstance(temporal_fine_correction, bool):
            raise ValueError("temporal_fine_correction must be a boolean")
        if temporal_fine_correction and (initialization != "temporal" or pyramid_levels != 2):
            raise ValueError("temporal_fine_correction requires temporal initialization and two levels")
        if not isinstance(initialization, str) or initialization not in _INITIALIZATIONS:
            raise ValueError("initialization must be 'zero', 'temporal', 'fourier', 'wgpu-matching' or 'zncc'")
        if seed_search_radius is not None:
            try:
                radius = operator.index(seed_search_radius)
            except TypeError as error:
                raise ValueError("seed_search_radius must be an integer from 1 to 64") from error
            if isinstance(seed_search_radius, bool) or not 1 <= radius <= 64:
                raise ValueError("seed_search_radius must be an integer from 1 to 64")
            if initialization not in ("zncc", "temporal", "fourier"):
                raise ValueError("seed_search_radius requires initialization='zncc', 'temporal' or 'fourier'")
            seed_search_radius = radius
        elif initialization == "zncc":
            seed_search_radius = 8
        self.seed_search_radius = seed_search_radius
        if matching_options is not None and initialization != "wgpu-matching":
            raise ValueError("matching_options requires initialization='wgpu-matching'")
        if temporal_max_age is not None:
            try:
                age = operator.index(temporal_max_age)
            except TypeError as error:
                raise ValueError("temporal_max_age must be a nonnegative integer or None") from error
            if isinstance(temporal_max_age, bool) or not 0 <= age <= 0xFFFFFFFE:
                raise ValueError("temporal_max_age must be between 0 and 4294967294 or None")
            temporal_max_age = age
        self.interpolation = normalize_interpolation(interpolation)
        self.motion_model = normalize_motion_model(motion_model)
        if initialization == "fourier" and self.motion_model == "quadratic":
            raise ValueError("Fourier initialization currently supports translation and affine models")
        self.outlier_policy = normalize_outlier_policy(outlier_policy)
        self.median_filter_size = normalize_median_filter_size(median_filter_size)
        self.median_filter_scope = normalize_median_filter_scope(median_filter_scope)
        if self.median_filter_scope == "all" and self.outlier_policy != "median":
            raise ValueError("median_filter_scope='all' requires outlier_policy='median'")
        if self.median_filter_size > 3 and self.outlier_policy != "median":
            raise ValueError("median_filter_size > 3 requires outlier_policy='median'")
        self.subset_size = normalize_subset_size(subset_size)
        self.subset_stride = normalize_subset_stride(subset_stride, subset_size=self.subset_size)
        self.spatial_weighting = normalize_spatial_weighting(spatial_weighting)
        self.gaussian_sigma = normalize_gaussian_sigma(gaussian_sigma, subset_size=self.subset_size)
        self.solver_workgroup_size = _normalize_solver_workgroup_size(solver_workgroup_size)
        self.device_type = _normalize_device_type(device_type)
        if power_preference not in ("high-performance", "low-power"):
            raise ValueError("power_preference must be 'high-performance' or 'low-power'")
        self.pyramid_levels = _level_count(pyramid_levels)
        if initialization == "wgpu-matching" and self.pyramid_levels < 2:
            raise ValueError("WGPU-Matching initialization requires at least two pyramid levels")
        iterations = _schedule(
            iterations_per_level,
            level_count=self.pyramid_levels,
            defaults=_DEFAULT_ITERATION_SCHEDULES[self.pyramid_levels],
            name="iterations_per_level",
        )
        tolerances = _schedule(
            tolerance_per_level,
            level_count=self.pyramid_levels,
            defaults=_FOUR_LEVEL_TOLERANCES if self.pyramid_levels == 4 else _DEFAULT_TOLERANCES,
            name="tolerance_per_level",
        )
        self.iterations_per_level = tuple(int(v) for v in iterations)
        self.tolerance_per_level = tuple(float(v) for v in tolerances)
        for it, tol in zip(self.iterations_per_level, self.tolerance_per_level, strict=True):
            _validated_config(it, tol, 0.8)
        try:
            slots = operator.index(pipeline_slots)
        except TypeError as error:
            raise ValueError("pipeline_depth must be a positive integer") from error
        if slots < 1:
            raise ValueError("pipeline_depth must be a positive integer")
        # Options that the GPU engine does not provide fail loudly after validation.
        if initialization == "wgpu-matching":
            raise ICGNError("initialization='wgpu-matching' is not available in this build")
        if self.device_type == "cpu":
            raise ICGNError("This engine executes on a CUDA GPU only; device_type='cpu' is not available.")
        self.initialization = initialization
        self.temporal_max_age = temporal_max_age
        self.temporal_fine_correction = temporal_fine_correction
        self.temporal_prediction = temporal_prediction
        self.pyramid_policy = pyramid_policy
        self.adaptive_acceptance = float(adaptive_acceptance)
        self._adaptive_next_levels = self.pyramid_levels
        self._adaptive_population = 0
        self.power_preference = power_preference
        self._pipeline_slots = slots
        self._persistent = bool(persistent)
        self._zncc_min = 0.8
        self._fourier: FourierInitializer | None = None
        self._lib = _native.load()
        self._registration_lock = threading.Lock()
        self._closed = False
        self._handle = self._create(device)
        self.device_index = int(device)
        self.device_name = f"CUDA device {self.device_index} (gbdic sm_103a)"
        self.solver = _tuning.variant_name(self.solver_workgroup_size, self._persistent, self.solver_mode)
        self.execution_device_type = "gpu"
        self._reference_ready = False
        self.roi = None
        self.reference_valid = None
        self.width = self.height = self.grid_width = self.grid_height = 0

    def _create(self, device: int) -> C.c_void_p:
        po = _native.PyramidOptions()
        po.base = native_options(
            device=int(device),
            motion_model=self.motion_model,
            interpolation=self.interpolation,
            subset_size=self.subset_size,
            subset_stride=self.subset_stride,
            spatial_weighting=self.spatial_weighting,
            gaussian_sigma=self.gaussian_sigma,
            outlier_policy=self.outlier_policy,
            median_filter_size=self.median_filter_size,
            median_filter_scope=self.median_filter_scope,
            lanes=self.solver_workgroup_size,
            pipeline_slots=self._pipeline_slots,
            persistent=self._persistent,
            divergence_patience=self.divergence_patience or 0,
            divergence_min_iterations=self.divergence_min_iterations,
            solver_mode=self.solver_mode,
        )
        po.levels = self.pyramid_levels
        for i in range(self.pyramid_levels):
            po.iterations[i] = self.iterations_per_level[i]
            po.tolerance[i] = self.tolerance_per_level[i]
        po.zncc_min = self._zncc_min
        po.initialization = {"zero": 0, "temporal": 1, "zncc": 2, "fourier": 3}[self.initialization]
        po.seed_search_radius = self.seed_search_radius or 0
        po.temporal_max_age = 0xFFFFFFFE if self.temporal_max_age is None else int(self.temporal_max_age)
        po.temporal_prediction = 1 if self.temporal_prediction == "velocity" else 0
        po.temporal_fine_correction = int(self.temporal_fine_correction)
        po.adaptive = int(self.pyramid_policy == "adaptive")
        handle = C.c_void_p()
        _native.check(self._lib.gbdic_pyramid_create(C.byref(po), C.byref(handle)), self._lib.gbdic_pyramid_last_error(None))
        return handle

    def _check(self, code: int) -> None:
        if code != _native.OK:
            _native.check(code, self._lib.gbdic_pyramid_last_error(self._handle))

    # ------------------------------------------------------------ reference
    def set_reference(
        self,
        image: ImageInput,
        *,
        iterations_per_level: tuple[int, ...] | None = None,
        tolerance_per_level: tuple[float, ...] | None = None,
        zncc_min: float = 0.8,
        roi_mask: np.ndarray | None = None,
        roi_policy: str = "full",
        roi_truncation: str = "none",
    ) -> ReferenceInfo:
        """Prepare every scale on the GPU (full_pyramid_backend.py:1135-1368)."""
        if self._closed:
            raise ICGNError("This engine is closed; create a new engine before set_reference().")
        started = time.perf_counter()
        iterations = self.iterations_per_level
        if iterations_per_level is not None:
            iterations = tuple(int(v) for v in _schedule(
                iterations_per_level, level_count=self.pyramid_levels,
                defaults=_DEFAULT_ITERATION_SCHEDULES[self.pyramid_levels], name="iterations_per_level"))
        tolerances = self.tolerance_per_level
        if tolerance_per_level is not None:
            tolerances = tuple(float(v) for v in _schedule(
                tolerance_per_level, level_count=self.pyramid_levels,
                defaults=_FOUR_LEVEL_TOLERANCES if self.pyramid_levels == 4 else _DEFAULT_TOLERANCES,
                name="tolerance_per_level"))
        new_zncc = float(zncc_min)
        for it, tol in zip(iterations, tolerances, strict=True):
            _validated_config(it, tol, new_zncc)
        reference = _as_uint8_gray(image)
        mask = validate_roi(roi_mask, roi_policy, reference.shape, self.motion_model, roi_truncation)
        height, width = reference.shape
        dims = []
        w, h = width, height
        for _ in range(self.pyramid_levels):
            gw, gh = subset_grid_shape(w, h, subset_size=self.subset_size, subset_stride=self.subset_stride)
            if gw < 1 or gh < 1:
                raise ValueError(f"Reference dimensions must each be at least {self.subset_size} pixels.")
            dims.append((w, h, gw, gh))
            w, h = w // 2, h // 2
        masks = [mask]
        for _ in range(1, self.pyramid_levels):
            masks.append(None if masks[-1] is None else reduce_mask(masks[-1]))
        plans = [prepare_roi(m, self.subset_size, self.subset_stride, policy=roi_policy, truncation=roi_truncation,
                             median_filter_size=self.median_filter_size) for m in masks]
        effective = plans[0] is not None and plans[0].effective
        keep: list[np.ndarray] = []
        rois = (_native.LevelRoi * self.pyramid_levels)()
        if effective:
            prefix = integral(mask)
            for level, plan in enumerate(plans):
                selected = np.ascontiguousarray(plan.selected, dtype=np.uint8).ravel()
                links = np.ascontiguousarray(plan.links_table(self.median_filter_size, self.outlier_policy))
                keep += [selected, links]
                rois[level].selected = selected.ctypes.data_as(C.POINTER(C.c_uint8))
                rois[level].links = links.ctypes.data_as(C.POINTER(C.c_float))
                if level < self.pyramid_levels - 1:
                    flags = np.ascontiguousarray(seed_permissions(
                        plans[level + 1], plan, source_scale=1 << (level + 1), destination_scale=1 << level,
                        size=self.subset_size, stride=self.subset_stride, reference_mask=mask, reference_prefix=prefix,
                    ), dtype=np.uint32).ravel()
                    keep.append(flags)
                    rois[level].seed_links = flags.ctypes.data_as(C.POINTER(C.c_uint32))
        temporal_links = None
        if effective and self.initialization == "temporal":
            temporal_links = np.ascontiguousarray(seed_permissions(
                plans[0], plans[-1], source_scale=1, destination_scale=1 << (self.pyramid_levels - 1),
                size=self.subset_size, stride=self.subset_stride, reference_mask=mask,
                reference_prefix=integral(mask),
            ), dtype=np.uint32).ravel()
        if (iterations, tolerances, new_zncc) != (self.iterations_per_level, self.tolerance_per_level, self._zncc_min):
            self.iterations_per_level, self.tolerance_per_level, self._zncc_min = iterations, tolerances, new_zncc
            old, self._handle = self._handle, self._create(self.device_index)
            self._lib.gbdic_pyramid_destroy(old)
        self._reference_ready = False
        info = _native.RefInfo()
        prep_start = time.perf_counter()
        self._check(self._lib.gbdic_pyramid_set_reference(
            self._handle, _native.ptr(reference), width, height, reference.strides[0],
            C.cast(rois, C.c_void_p) if effective else None, _native.ptr(temporal_links), C.byref(info)))
        prep_ms = (time.perf_counter() - prep_start) * 1e3
        self.width, self.height = width, height
        self.grid_width, self.grid_height = dims[0][2], dims[0][3]
        for level, plan in enumerate(plans):
            if plan is not None and plan.partial_indices is not None and plan.partial_indices.size:
                plans[level] = self._install_partial(level, plan, dims[level])
        self.roi = plans[0]
        admissible = np.empty(self.grid_width * self.grid_height, np.uint8)
        self._check(self._lib.gbdic_pyramid_export(self._handle, 0, _native.EXPORT_ADMISSIBLE,
                                                   _native.ptr(admissible), admissible.nbytes))
        self.reference_valid = immutable(admissible.reshape(self.grid_height, self.grid_width).astype(bool))
        self._adaptive_population = int(np.count_nonzero(self.reference_valid))
        self._adaptive_next_levels = self.pyramid_levels
        self._roi_level_counts = [
            int(p.selected.sum()) if p is not None else d[2] * d[3] for p, d in zip(plans, dims, strict=True)
        ]
        if self._fourier is not None:
            self._fourier.close()
        self._fourier = None
        if self.initialization == "fourier" and (mask is None or mask.any()):
            self._fourier = FourierInitializer(reference, mask, device=self.device_index)
        self._reference_ready = True
        usable = self.reference_valid if self.roi is None else self.reference_valid & self.roi.selected
        if self._autotune and usable.any():
            self._autotune_solver(reference)
        total = (time.perf_counter() - started) * 1e3
        return ReferenceInfo(
            preparation_wall_ms=total,
            runtime_build_wall_ms=total - info.device_ms,
            reference_build_wall_ms=info.device_ms,
            encoding_wall_ms=0.0,
            total_wall_ms=total,
            config=self._config_echo(),
            device=self.device_name,
            grid=(self.grid_width, self.grid_height),
            width=width,
            height=height,
            subset_size=self.subset_size,
            subset_stride=self.subset_stride,
            roi=self.roi,
            reference_valid=self.reference_valid,
        )

    def _install_partial(self, level: int, plan, dims) -> Any:
        """Partial-support windows of one level (the reference applies the
        policy at every scale, full_pyramid_backend.py:1222-1232)."""
        from .partial import install_partial_reference

        w, h = dims[0], dims[1]
        return install_partial_reference(
            plan, lambda what, dtype, shape: self.export_level(level, what, dtype, shape),
            lambda *args: self._check(self._lib.gbdic_pyramid_set_partial_support(self._handle, level, *args)),
            width=w, height=h, size=self.subset_size, stride=self.subset_stride, motion_model=self.motion_model,
            weighting=self.spatial_weighting, sigma=self.gaussian_sigma)

    def _config_echo(self) -> dict[str, Any]:
        echo: dict[str, Any] = {
            "iterations": self.iterations_per_level[-1],
            "tolerance": self.tolerance_per_level[-1],
            "znccMin": self._zncc_min,
            "pyramidLevels": self.pyramid_levels,
            "pyramidStrategy": "full",
            "iterationsPerLevel": list(self.iterations_per_level),
            "tolerancePerLevel": list(self.tolerance_per_level),
            "width": self.width,
            "height": self.height,
            "subsetSize": self.subset_size,
            "deviceType": self.device_type,
            "executionDeviceType": self.execution_device_type,
            "interpolation": self.interpolation,
            "motionModel": self.motion_model,
            "outlierPolicy": self.outlier_policy,
            "medianFilterSize": self.median_filter_size,
            "medianFilterScope": self.median_filter_scope,
            "subsetStride": self.subset_stride,
            "spatialWeighting": self.spatial_weighting,
            "solverWorkgroupSize": self.solver_workgroup_size,
            "solverMode": self.solver_mode,
            "gaussianSigma": self.gaussian_sigma,
        }
        if self.pyramid_policy == "adaptive":
            echo.update(pyramidPolicy="adaptive", adaptiveAcceptance=self.adaptive_acceptance,
                        adaptiveFeedback="ordered-single-slot")
        if self.divergence_patience is not None:
            echo.update(divergencePatience=self.divergence_patience,
                        divergenceMinIterations=self.divergence_min_iterations, divergenceLevels="finest")
        if self.initialization == "temporal":
            echo.update(
                initialization="temporal",
                temporalMaxAge=self.temporal_max_age,
                temporalSeedLevel="coarsest",
                temporalSeedState="filtered" if self.outlier_policy == "replace" and self.temporal_prediction == "none" else "raw",
            )
            if self.temporal_fine_correction:
                echo["temporalFineCorrection"] = True
            if self.temporal_prediction == "velocity":
                echo["temporalPrediction"] = "velocity"
        if self.initialization == "fourier":
            echo.update(initialization="fourier",
                        fourierWindow=None if self._fourier is None else self._fourier.window)
        if self.initialization == "zncc":
            echo["initialization"] = "zncc"
        if self.seed_search_radius:
            echo.update(seedSearch="zncc-integer", seedSearchRadius=self.seed_search_radius,
                        seedSearchLevel="coarsest")
        if self.roi is not None:
            echo["roi"] = {**self.roi.summary(), "selectedPerLevel": self._roi_level_counts}
        return echo

    def _prepare_target(self, target: ImageInput) -> np.ndarray:
        frame = _as_uint8_gray(target)
        if frame.shape != (self.height, self.width):
            raise ValueError(
                f"Target dimensions must be {self.width}x{self.height}; received {frame.shape[1]}x{frame.shape[0]}."
            )
        return frame

    def _begin_frame(self) -> int:
        """Levels the next frame runs (the adaptive policy's last decision)."""
        levels = self._adaptive_next_levels if self.pyramid_policy == "adaptive" else self.pyramid_levels
        if self.pyramid_policy == "adaptive":
            self._check(self._lib.gbdic_pyramid_set_active_levels(self._handle, levels))
        return levels

    def _adaptive_feedback(self, counters: np.ndarray) -> None:
        """full_pyramid_backend.py:1781-1790: the finest level alone while the
        accepted history covers `adaptive_acceptance` of the reference-valid
        windows and nothing expired; the whole pyramid otherwise."""
        accepted, expired = float(counters[1]), float(counters[3])
        self._adaptive_next_levels = (
            1 if self._adaptive_population > 0 and accepted / self._adaptive_population >= self.adaptive_acceptance
            and not expired else 2
        )

    def _result(self, packed: np.ndarray, counters: np.ndarray, timing: _native.Timing, accepted_at: float,
                prep_ms: float, levels_used: int | None = None) -> RegistrationResult:
        times = {
            "inputPreparationWallMs": prep_ms,
            "uploadWallMs": timing.upload_ms,
            "completionWaitWallMs": timing.execute_ms,
            "readbackCopyWallMs": timing.readback_ms,
            "executeReadbackWallMs": timing.execute_ms + timing.readback_ms,
            "deviceMs": timing.device_ms,
            "pyramidLevels": float(levels_used or self.pyramid_levels),
            "queueSubmissions": 1.0,
        }
        if self.initialization == "temporal":
            times["temporallySeededCoarseSubsets"] = float(counters[0])
            times["temporalAcceptedUpdates"] = float(counters[1])
            if self.temporal_prediction == "velocity":
                times["velocityPredictedSubsets"] = float(counters[2])
            if self.pyramid_policy == "adaptive":
                times["temporalExpiredSubsets"] = float(counters[3])
        build = time.perf_counter()
        result = result_from_packed(
            packed,
            motion_model=self.motion_model,
            timing=times,
            config=self._config_echo(),
            width=self.width,
            height=self.height,
            subset_size=self.subset_size,
            subset_stride=self.subset_stride,
            roi=self.roi,
            reference_valid=self.reference_valid,
        )
        if self.pyramid_policy == "adaptive":
            self._adaptive_feedback(counters)
            result.config["pyramidLevelsUsed"] = levels_used
        now = time.perf_counter()
        total = (now - accepted_at) * 1e3
        result.timing = {**result.timing, "resultBuildWallMs": (now - build) * 1e3, "pipelineLatencyWallMs": total,
                         "resultAgeWallMs": total, "totalWallMs": total}
        return result

    def _empty_result(self, started: float) -> RegistrationResult:
        packed = np.zeros((self.grid_height, self.grid_width, state_float_count(self.motion_model)), np.float32)
        packed[..., parameter_count(self.motion_model)] = -3.0
        elapsed = (time.perf_counter() - started) * 1e3
        return result_from_packed(
            packed, motion_model=self.motion_model,
            timing={"queueSubmissions": 0.0, "totalWallMs": elapsed, "resultAgeWallMs": elapsed},
            config=self._config_echo(), width=self.width, height=self.height, subset_size=self.subset_size,
            subset_stride=self.subset_stride, roi=self.roi, reference_valid=self.reference_valid,
        )

    # ------------------------------------------------------------ registration
    def _global_translation(self, slot: int, frame: np.ndarray | None = None, *, device_frame: int | None = None,
                            row_stride: int = 0) -> dict | None:
        """Fourier estimate of the target (full_pyramid_backend.py:1704-1714),
        set as the slot's coarsest seed; ambiguous targets raise ICGNError."""
        if self._fourier is None:
            return None
        try:
            if device_frame is not None:
                estimate = self._fourier.estimate_device(device_frame, row_stride)
            else:
                estimate = self._fourier.estimate(frame)
        except ValueError as error:
            raise ICGNError(str(error)) from error
        self._check(self._lib.gbdic_pyramid_set_translation(self._handle, slot, float(estimate["dx"]),
                                                            float(estimate["dy"])))
        return estimate

    @staticmethod
    def _attach_translation(result: RegistrationResult, estimate: dict | None) -> RegistrationResult:
        if estimate is not None:
            result.config["globalTranslation"] = estimate
            result.timing["fourierWallMs"] = estimate["wallMs"]
        return result

    def register(self, target: ImageInput) -> RegistrationResult:
        """One upload, one graph launch, one readback (1815-1832)."""
        if not self._reference_ready:
            raise ICGNError("Call set_reference() before register().")
        if not self._registration_lock.acquire(blocking=False):
            raise ICGNError("Another registration or registration stream is active.")
        try:
            accepted_at = time.perf_counter()
            frame = self._prepare_target(target)
            if self.roi is not None and self.roi.empty:
                return self._empty_result(accepted_at)
            estimate = self._global_translation(0, frame)
            prep_ms = (time.perf_counter() - accepted_at) * 1e3
            packed = np.empty((self.grid_height, self.grid_width, state_float_count(self.motion_model)), np.float32)
            counters = np.zeros(4, np.uint32)
            timing = _native.Timing()
            levels = self._begin_frame()
            self._check(self._lib.gbdic_pyramid_register(
                self._handle, _native.ptr(frame), frame.strides[0], _native.ptr(packed), _native.ptr(counters),
                C.byref(timing)))
            return self._attach_translation(self._result(packed, counters, timing, accepted_at, prep_ms, levels),
                                            estimate)
        finally:
            self._registration_lock.release()

    def register_stream(self, targets: Iterable[ImageInput], *, pipeline_depth: int = DEFAULT_IN_FLIGHT_FRAMES
                        ) -> Iterator[RegistrationResult]:
        """Ordered results with up to ``pipeline_depth`` targets in flight."""
        if not self._reference_ready:
            raise ICGNError("Call set_reference() before register_stream().")
        try:
            depth = operator.index(pipeline_depth)
        except TypeError as error:
            raise ValueError("pipeline_depth must be a positive integer") from error
        if isinstance(pipeline_depth, bool) or depth < 1:
            raise ValueError("pipeline_depth must be a positive integer")
        if self.pyramid_policy == "adaptive":
            # The level decision needs the preceding frame's result (1857-1860).
            depth = 1
        if depth > self._pipeline_slots:
            raise ValueError(f"pipeline_depth must be at most {self._pipeline_slots} for this engine")
        return self._stream(targets, depth)

    def _stream(self, targets: Iterable[ImageInput], depth: int) -> Iterator[RegistrationResult]:
        if not self._registration_lock.acquire(blocking=False):
            raise ICGNError("Another registration or registration stream is active.")
        available = deque(range(depth))
        pending: deque[tuple[int, float, float, dict | None, int]] = deque()
        try:
            if self.roi is not None and self.roi.empty:
                for target in targets:
                    started = time.perf_counter()
                    self._prepare_target(target)
                    yield self._empty_result(started)
                return

            def retire() -> RegistrationResult:
                slot, accepted_at, prep_ms, estimate, levels = pending.popleft()
                packed = np.empty((self.grid_height, self.grid_width, state_float_count(self.motion_model)), np.float32)
                counters = np.zeros(4, np.uint32)
                timing = _native.Timing()
                self._check(self._lib.gbdic_pyramid_retire(self._handle, slot, _native.ptr(packed),
                                                           _native.ptr(counters), C.byref(timing)))
                available.append(slot)
                return self._attach_translation(
                    self._result(packed, counters, timing, accepted_at, prep_ms, levels), estimate)

            for target in targets:
                if not available:
                    yield retire()
                slot = available.popleft()
                accepted_at = time.perf_counter()
                frame = self._prepare_target(target)
                try:
                    estimate = self._global_translation(slot, frame)
                except ICGNError:
                    available.appendleft(slot)
                    raise
                prep_ms = (time.perf_counter() - accepted_at) * 1e3
                levels = self._begin_frame()
                self._check(self._lib.gbdic_pyramid_submit(self._handle, slot, _native.ptr(frame), frame.strides[0]))
                pending.append((slot, accepted_at, prep_ms, estimate, levels))
            while pending:
                yield retire()
        finally:
            while pending:
                slot = pending.popleft()[0]
                self._lib.gbdic_pyramid_retire(self._handle, slot, None, None, None)
            self._registration_lock.release()

    def register_device(self, device_frame: int, device_state: int, *, stream: int | None = None,
                        translation: tuple[float, float] | None = None) -> None:
        """Resident registration of a device frame into a device state buffer.
        With Fourier initialization, `translation` (dx, dy) replaces the
        initializer's own estimate as the global seed (e.g. one computed on
        the device from another window)."""
        if not self._reference_ready:
            raise ICGNError("Call set_reference() before register().")
        if translation is not None:
            if self.initialization != "fourier":
                raise ValueError("translation requires initialization='fourier'")
            self._check(self._lib.gbdic_pyramid_set_translation(self._handle, 0, float(translation[0]),
                                                                float(translation[1])))
        else:
            self._global_translation(0, device_frame=device_frame, row_stride=self.width)
        self._begin_frame()
        self._check(self._lib.gbdic_pyramid_register_device(
            self._handle, C.c_void_p(device_frame), C.c_void_p(device_state), C.c_void_p(stream or 0)))

    def set_solver_variant(self, lanes: int, persistent: bool = False, mode: str | None = None) -> None:
        """Select the solver variant of every level (lanes per subset, grid or
        persistent queue, and optionally the pixel loop)."""
        self._check(self._lib.gbdic_pyramid_set_solver_variant(
            self._handle, _normalize_solver_workgroup_size(lanes), int(bool(persistent))))
        self.solver_workgroup_size = int(lanes)
        self._persistent = bool(persistent)
        if mode is not None:
            self.set_solver_mode(mode)
        self.solver = _tuning.variant_name(int(lanes), bool(persistent), self.solver_mode)

    def set_solver_mode(self, mode: str) -> None:
        """Select the pixel loop ('exact' or 'fast') of every level."""
        mode = normalize_solver_mode(mode)
        self._check(self._lib.gbdic_pyramid_set_solver_mode(self._handle, _native.SOLVER_MODES[mode]))
        self.solver_mode = mode
        self.solver = _tuning.variant_name(self.solver_workgroup_size, self._persistent, mode)

    def _autotune_solver(self, reference: np.ndarray) -> None:
        """Fastest validated variant on the reference shifted by (-1, +2) px;
        the temporal history is reset afterwards."""
        target = np.ascontiguousarray(np.roll(reference, shift=(-1, 2), axis=(0, 1)))

        def run():
            self.reset_temporal_state()
            r = self.register(target)
            packed = np.concatenate([r.parameters, r.status[..., None], r.iterations[..., None]], -1)
            return packed, float(r.timing["deviceMs"])

        best, self.solver_tuning_ms, self.solver_validation = _tuning.autotune(self.set_solver_variant, run)
        self.set_solver_variant(*best)
        self.reset_temporal_state()

    def set_profiling(self, enable: bool) -> None:
        """Time every solver launch of the resident path with CUDA events and
        count executed Gauss-Newton iterations (resets the counters)."""
        self._check(self._lib.gbdic_pyramid_profile(self._handle, int(bool(enable))))

    def read_profile(self) -> dict[str, float]:
        ms, launches, timed, iters = C.c_double(), C.c_int64(), C.c_int64(), C.c_uint64()
        self._check(self._lib.gbdic_pyramid_profile_read(
            self._handle, C.byref(ms), C.byref(launches), C.byref(timed), C.byref(iters)))
        return {"solver_ms": ms.value, "launches": launches.value, "timed_launches": timed.value,
                "iterations": iters.value}

    def reset_temporal_state(self) -> None:
        """Forget the temporal history (676-694); no-op before set_reference.
        The adaptive policy starts again from the whole pyramid."""
        self._adaptive_next_levels = self.pyramid_levels
        if self._handle is not None:
            self._check(self._lib.gbdic_pyramid_reset_temporal(self._handle))

    def export_level(self, level: int, what: int, dtype, shape) -> np.ndarray:
        out = np.empty(shape, dtype=dtype)
        self._check(self._lib.gbdic_pyramid_export(self._handle, level, what, _native.ptr(out), out.nbytes))
        return out

    def level_grid(self, level: int) -> tuple[int, int]:
        gw, gh = C.c_int32(), C.c_int32()
        self._check(self._lib.gbdic_pyramid_level_grid(self._handle, level, C.byref(gw), C.byref(gh)))
        return gw.value, gh.value

    def close(self) -> None:
        if self._closed:
            return
        self._reference_ready = False
        self._closed = True
        if self._fourier is not None:
            self._fourier.close()
            self._fourier = None
        handle, self._handle = self._handle, None
        if handle:
            self._lib.gbdic_pyramid_destroy(handle)

    def __enter__(self) -> ICGNWGPUFullPyramid:
        return self

    def __exit__(self, *_: object) -> None:
        self.close()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass
