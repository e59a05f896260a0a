"""Single-scale IC-GN engine on the GB300 (drop-in for ICGNWGPU).

Mirrors live_dic/wgpu_backend.py:ICGNWGPU (856-3099): same constructor
arguments and validation messages, same methods and result types.  The GPU
work (reference preparation, FIR prefilter, IC-GN, UOD, final ZNCC) runs in
libgbdic.so through its C ABI; this module only validates, plans the static
ROI geometry and packs results.
"""

from __future__ import annotations

import ctypes as C
import operator
import threading
import time
from collections import deque
from collections.abc import Iterable, Iterator
from functools import wraps
from typing import Any

import numpy as np

from . import _native
from . import autotune as _tuning
from .engine import ICGNError, ImageInput, ReferenceInfo, RegistrationResult, _as_uint8_gray, result_from_packed
from .interpolation import INTERPOLATION_CODES, normalize_interpolation
from .motion import MOTION_MODEL_CODES, normalize_motion_model, parameter_count, state_float_count
from .outlier import (
    MEDIAN_FILTER_SCOPE_CODES,
    OUTLIER_POLICY_CODES,
    normalize_median_filter_scope,
    normalize_median_filter_size,
    normalize_outlier_policy,
)
from .pyramid_recovery import pyramid_dependency_mask, reduce_half, transfer_pyramid_seed
from .roi import RoiPlan, immutable, integral, prepare_roi, reduce_mask, seed_permissions, validate_roi
from .subset import DEFAULT_SUBSET_SIZE, normalize_subset_size, normalize_subset_stride, subset_grid_shape
from .weighting import SPATIAL_WEIGHTING_CODES, normalize_gaussian_sigma, normalize_spatial_weighting

MAX_ITERATIONS = 30
DEFAULT_IN_FLIGHT_FRAMES = 2
DEFAULT_PYRAMID_LEVELS = 1


def _validated_config(iterations: int, tolerance: float, zncc_min: float) -> dict[str, float | int]:
    """Solver controls (reference: wgpu_backend.py:504-524)."""
    count, tol, zmin = int(iterations), float(tolerance), float(zncc_min)
    if not 1 <= count <= MAX_ITERATIONS:
        raise ValueError(f"iterations must be between 1 and {MAX_ITERATIONS}")
    if not np.isfinite(tol) or tol <= 0.0:
        raise ValueError("tolerance must be a finite positive number")
    if not np.isfinite(zmin) or not 0.0 <= zmin <= 1.0:
        raise ValueError("zncc_min must be between 0 and 1")
    return {"iterations": count, "tolerance": tol, "znccMin": zmin}


def _normalize_device_type(value: str) -> str:
    if not isinstance(value, str) or value.strip().lower() not in ("auto", "gpu", "cpu"):
        raise ValueError("device_type must be 'auto', 'gpu', or 'cpu'")
    return value.strip().lower()


def _normalize_solver_workgroup_size(value: int) -> int:
    """Lanes per subset: the reference's 16, 32 or 128, plus 64 on this GPU."""
    try:
        size = operator.index(value)
    except TypeError as error:
        raise ValueError("solver_workgroup_size must be 16, 32, 64, or 128") from error
    if isinstance(value, bool) or size not in (16, 32, 64, 128):
        raise ValueError("solver_workgroup_size must be 16, 32, 64, or 128")
    return size


def normalize_solver_mode(value: str) -> str:
    """Pixel loop of the IC-GN solver (no reference counterpart): 'exact'
    keeps the reference's pixel-to-lane order and summation, 'fast' runs the
    sliding-window loop for B-spline translation / affine windows, 'staged'
    and 'staged-wide' run the exact loop on taps staged by TMA in a per-warp
    shared-memory tile (56 x 44 or 72 x 56 floats; bit-identical to 'exact').
    Configurations a mode does not cover keep the exact loop."""
    if not isinstance(value, str) or value not in _native.SOLVER_MODES:
        raise ValueError("solver_mode must be 'exact', 'fast', 'staged' or 'staged-wide'")
    return value


def _exclusive_call(method):
    """One registration at a time per engine (wgpu_backend.py:826-838)."""

    @wraps(method)
    def guarded(self, *args, **kwargs):
        if not self._registration_lock.acquire(blocking=False):
            raise ICGNError("Another registration or registration stream is active.")
        try:
            return method(self, *args, **kwargs)
        finally:
            self._registration_lock.release()

    return guarded


def _exclusive_stream(method):
    """Hold the lock until the generator is exhausted or closed (841-853)."""

    @wraps(method)
    def guarded(self, *args, **kwargs):
        if not self._registration_lock.acquire(blocking=False):
            raise ICGNError("Another registration or registration stream is active.")
        try:
            yield from method(self, *args, **kwargs)
        finally:
            self._registration_lock.release()

    return guarded


def native_options(
    *,
    device: int,
    motion_model: str,
    interpolation: str,
    subset_size: int,
    subset_stride: int,
    spatial_weighting: str,
    gaussian_sigma: float,
    outlier_policy: str,
    median_filter_size: int,
    median_filter_scope: str,
    lanes: int,
    pipeline_slots: int,
    persistent: bool,
    divergence_patience: int = 0,
    divergence_min_iterations: int = 4,
    solver_mode: str = "exact",
) -> _native.Options:
    o = _native.Options()
    o.device = device
    o.motion_model = MOTION_MODEL_CODES[motion_model]
    o.interpolation = INTERPOLATION_CODES[interpolation]
    o.subset_size = subset_size
    o.subset_stride = subset_stride
    o.spatial_weighting = SPATIAL_WEIGHTING_CODES[spatial_weighting]
    o.gaussian_sigma = gaussian_sigma
    o.outlier_policy = OUTLIER_POLICY_CODES[outlier_policy]
    o.median_filter_size = median_filter_size
    o.median_filter_scope = MEDIAN_FILTER_SCOPE_CODES[median_filter_scope]
    o.threads_per_subset = lanes
    o.divergence_patience = divergence_patience
    o.divergence_min_iterations = divergence_min_iterations
    o.pipeline_slots = pipeline_slots
    o.persistent = int(persistent)
    o.solver_mode = _native.SOLVER_MODES[solver_mode]
    return o


class ICGNWGPU:
    """Persistent single-scale IC-GN engine on one CUDA device.

    Construction validates every argument before any device work.  The
    reference is prepared on the GPU by :meth:`set_reference` and stays
    resident in HBM; each :meth:`register` uploads one 8-bit target, runs the
    FIR prefilter, the IC-GN solve and the UOD pass, and returns the packed
    field as zero-copy NumPy views.  ``solver_workgroup_size`` is the number
    of CUDA lanes that share one subset (16, 32, 64 or 128); results at
    different widths differ only by float reduction order.  ``solver_mode``
    (an extension) selects the pixel loop: 'exact' (the reference's order)
    or 'fast' (sliding-window B-spline sampling, within the parity
    tolerances of the exact loop); the autotuner considers both.
    ``device_type='cpu'`` is rejected: there is no CPU execution path.
    """

    roi: RoiPlan | None = None
    reference_valid: np.ndarray | None = None

    def __init__(
        self,
        *,
        power_preference: str = "high-performance",
        device_type: str = "auto",
        prefer_subgroups: bool | None = None,
        solver_workgroup_size: int = 16,
        pyramid_levels: int = DEFAULT_PYRAMID_LEVELS,
        interpolation: str = "bspline",
        motion_model: str = "affine",
        outlier_policy: str = "replace",
        median_filter_size: int = 3,
        median_filter_scope: str = "rejected",
        subset_size: int = DEFAULT_SUBSET_SIZE,
        subset_stride: int | None = None,
        spatial_weighting: str = "uniform",
        gaussian_sigma: float | None = None,
        device: int = 0,
        pipeline_slots: int = DEFAULT_IN_FLIGHT_FRAMES,
        persistent: bool = False,
        autotune: bool = False,
        solver_mode: str = "exact",
    ) -> None:
        self.device_type = _normalize_device_type(device_type)
        self.solver_mode = normalize_solver_mode(solver_mode)
        if power_preference not in ("high-performance", "low-power"):
            raise ValueError("power_preference must be 'high-performance' or 'low-power'")
        self.interpolation = normalize_interpolation(interpolation)
        self.motion_model = normalize_motion_model(motion_model)
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
        if prefer_subgroups is True and (
            self.subset_size != DEFAULT_SUBSET_SIZE or self.subset_stride != DEFAULT_SUBSET_SIZE
        ):
            raise ValueError("prefer_subgroups=True requires subset_size=16 and subset_stride=16")
        if prefer_subgroups is True and (
            self.interpolation != "bspline" or self.motion_model != "affine" or self.spatial_weighting != "uniform"
        ):
            raise ValueError(
                "prefer_subgroups=True requires interpolation='bspline', "
                "motion_model='affine', and spatial_weighting='uniform'"
            )
        try:
            levels = operator.index(pyramid_levels)
        except TypeError as error:
            raise ValueError("pyramid_levels must be an integer from 1 to 3") from error
        if isinstance(pyramid_levels, bool) or not 1 <= levels <= 3:
            raise ValueError("pyramid_levels must be an integer from 1 to 3")
        try:
            slots = operator.index(pipeline_slots)
        except TypeError as error:
            raise ValueError("pipeline_depth must be a positive integer") from error
        if slots < 1:
            raise ValueError("pipeline_depth must be a positive integer")
        if self.device_type == "cpu":
            raise ICGNError("This engine executes on a CUDA GPU only; device_type='cpu' is not available.")
        self.pyramid_levels = levels
        self._pipeline_slots = slots
        self._persistent = bool(persistent)
        self._autotune = bool(autotune)
        self.solver_tuning_ms: dict[str, float] = {}
        self.solver_validation: dict[str, dict] = {}
        self._lib = _native.load()
        self._registration_lock = threading.Lock()
        self._closed = False
        handle = C.c_void_p()
        options = native_options(
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
            pipeline_slots=slots,
            persistent=self._persistent,
            solver_mode=self.solver_mode,
        )
        code = self._lib.gbdic_create(C.byref(options), C.byref(handle))
        _native.check(code, self._lib.gbdic_last_error(None))
        self._handle = handle
        self.device_index = int(device)
        self.device_name = f"CUDA device {self.device_index} (gbdic sm_103a)"
        self.solver = _tuning.variant_name(self.solver_workgroup_size, self._persistent, self.solver_mode)
        self.execution_device_type = "gpu"
        self.width = self.height = self.grid_width = self.grid_height = 0
        self._reference_ready = False
        # incremented by every reference preparation (device-side users key
        # captured work on it)
        self.reference_generation = 0
        self._target_ready = False
        self._config: dict[str, float | int] = {"iterations": 30, "tolerance": 1e-3, "znccMin": 0.8}
        self.roi = None
        self.reference_valid = None
        self._pyramid_engines: list[ICGNWGPU] = []
        self._roi_seed_permissions: np.ndarray | None = None

    # ------------------------------------------------------------ helpers
    def _check(self, code: int) -> None:
        if code != _native.OK:
            _native.check(code, self._lib.gbdic_last_error(self._handle))

    def set_solver_variant(self, lanes: int, persistent: bool = False, mode: str | None = None) -> None:
        """Select the solver variant: lanes per subset, grid or persistent
        queue, and (optionally) the pixel loop."""
        self._check(self._lib.gbdic_set_solver_variant(self._handle, _normalize_solver_workgroup_size(lanes),
                                                       int(bool(persistent))))
        self.solver_workgroup_size = int(lanes)
        self._persistent = bool(persistent)
        if mode is not None:
            self.set_solver_mode(mode)
        self.solver = _tuning.variant_name(int(lanes), bool(persistent), self.solver_mode)

    def set_solver_mode(self, mode: str) -> None:
        """Select the pixel loop ('exact' or 'fast') without re-preparing the reference."""
        mode = normalize_solver_mode(mode)
        self._check(self._lib.gbdic_set_solver_mode(self._handle, _native.SOLVER_MODES[mode]))
        self.solver_mode = mode
        self.solver = _tuning.variant_name(self.solver_workgroup_size, self._persistent, mode)

    def _autotune_solver(self, reference: np.ndarray) -> None:
        """Choose the fastest validated variant on the reference shifted by
        (-1, +2) pixels (wgpu_backend.py:2213-2296)."""
        target = np.ascontiguousarray(np.roll(reference, shift=(-1, 2), axis=(0, 1)))

        def run():
            r = self.register(target)
            packed = np.concatenate([r.parameters, r.status[..., None], r.iterations[..., None]], -1)
            return packed, float(r.timing["deviceMs"])

        best, self.solver_tuning_ms, self.solver_validation = _tuning.autotune(self.set_solver_variant, run)
        self.set_solver_variant(*best)

    def _cfg(self, config: dict[str, float | int]) -> _native.SolverCfg:
        return _native.SolverCfg(int(config["iterations"]), float(config["tolerance"]), float(config["znccMin"]))

    def _resolve_config(self, iterations, tolerance, zncc_min) -> dict[str, float | int]:
        return _validated_config(
            int(self._config["iterations"]) if iterations is None else iterations,
            float(self._config["tolerance"]) if tolerance is None else tolerance,
            float(self._config["znccMin"]) if zncc_min is None else zncc_min,
        )

    def _prepare_target(self, target: ImageInput) -> np.ndarray:
        frame = _as_uint8_gray(target)
        if frame.shape != (self.height, self.width):
            raise ValueError(
                f"Target dimensions must be {self.width}x{self.height}; received {frame.shape[1]}x{frame.shape[0]}."
            )
        return frame

    def _config_echo(self, config: dict[str, float | int]) -> dict[str, Any]:
        echo: dict[str, Any] = {
            **config,
            "pyramidLevels": self.pyramid_levels,
            "pyramidStrategy": "selective" if self.pyramid_levels > 1 else "single",
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
        if self.roi is not None:
            echo["roi"] = self.roi.summary()
        return echo

    def _new_packed(self) -> np.ndarray:
        return np.empty((self.grid_height, self.grid_width, state_float_count(self.motion_model)), dtype=np.float32)

    def _result(self, packed: np.ndarray, timing: dict[str, float], config) -> RegistrationResult:
        return result_from_packed(
            packed,
            motion_model=self.motion_model,
            timing=timing,
            config=self._config_echo(config),
            width=self.width,
            height=self.height,
            subset_size=self.subset_size,
            subset_stride=self.subset_stride,
            roi=self.roi,
            reference_valid=self.reference_valid,
        )

    @staticmethod
    def _timing(t: _native.Timing) -> dict[str, float]:
        return {
            "uploadWallMs": t.upload_ms,
            "executeReadbackWallMs": t.execute_ms + t.readback_ms,
            "readbackCopyWallMs": t.readback_ms,
            "deviceMs": t.device_ms,
            "totalWallMs": t.total_ms,
        }

    # ------------------------------------------------------------ reference
    def set_reference(
        self,
        image: ImageInput,
        *,
        iterations: int = 30,
        tolerance: float = 1e-3,
        zncc_min: float = 0.8,
        roi_mask: np.ndarray | None = None,
        roi_policy: str = "full",
        roi_truncation: str = "none",
    ) -> ReferenceInfo:
        if self._closed:
            raise ICGNError("This engine is closed; create a new engine before set_reference().")
        started = time.perf_counter()
        frame = _as_uint8_gray(image)
        height, width = frame.shape
        gw, gh = subset_grid_shape(width, height, subset_size=self.subset_size, subset_stride=self.subset_stride)
        if gw < 1 or gh < 1:
            raise ValueError(f"Reference dimensions must each be at least {self.subset_size} pixels.")
        config = _validated_config(iterations, tolerance, zncc_min)
        mask = validate_roi(roi_mask, roi_policy, frame.shape, self.motion_model, roi_truncation)
        roi = prepare_roi(mask, self.subset_size, self.subset_stride, policy=roi_policy, truncation=roi_truncation,
                          median_filter_size=self.median_filter_size)
        selected = links = None
        if roi is not None and roi.effective:
            selected = np.ascontiguousarray(roi.selected, dtype=np.uint8).ravel()
            links = np.ascontiguousarray(roi.links_table(self.median_filter_size, self.outlier_policy))
        self._reference_ready = False
        self._target_ready = False
        self._close_pyramid_engines()
        info = _native.RefInfo()
        prep_start = time.perf_counter()
        self._check(
            self._lib.gbdic_set_reference(
                self._handle, _native.ptr(frame), width, height, frame.strides[0],
                _native.ptr(selected), _native.ptr(links), C.byref(info),
            )
        )
        prep_ms = (time.perf_counter() - prep_start) * 1e3
        self.width, self.height, self.grid_width, self.grid_height = width, height, gw, gh
        self._config = config
        if roi is not None and roi.partial_indices is not None and roi.partial_indices.size:
            roi = self._prepare_partial(roi)
        self.roi = roi
        admissible = self._export(_native.EXPORT_ADMISSIBLE, np.uint8, (gh, gw))
        self.reference_valid = immutable(admissible.astype(bool))
        self._reference_ready = True
        self.reference_generation += 1
        if self.pyramid_levels > 1:
            self._prepare_pyramid(frame, zncc_min=config["znccMin"])
        usable = self.reference_valid if roi is None else self.reference_valid & roi.selected
        if self._autotune and usable.any():
            self._autotune_solver(frame)
        total_ms = (time.perf_counter() - started) * 1e3
        return ReferenceInfo(
            preparation_wall_ms=prep_ms,
            runtime_build_wall_ms=prep_ms - info.device_ms,
            reference_build_wall_ms=info.device_ms,
            encoding_wall_ms=0.0,
            total_wall_ms=total_ms,
            config={k: v for k, v in self._config_echo(config).items() if k not in ("width", "height")},
            device=self.device_name,
            grid=(gw, gh),
            width=width,
            height=height,
            subset_size=self.subset_size,
            subset_stride=self.subset_stride,
            roi=roi,
            reference_valid=self.reference_valid,
        )

    def set_profiling(self, enable: bool) -> None:
        """Time every solver launch of the resident path with CUDA events and
        count executed Gauss-Newton iterations (resets the counters)."""
        self._check(self._lib.gbdic_profile(self._handle, int(bool(enable))))

    def read_profile(self) -> dict[str, float]:
        ms, launches, timed, iters = C.c_double(), C.c_int64(), C.c_int64(), C.c_uint64()
        self._check(self._lib.gbdic_profile_read(
            self._handle, C.byref(ms), C.byref(launches), C.byref(timed), C.byref(iters)))
        return {"solver_ms": ms.value, "launches": launches.value, "timed_launches": timed.value,
                "iterations": iters.value}

    def set_reference_device(self, device_image: int, width: int, height: int, *, row_stride: int | None = None,
                             iterations: int = 30, tolerance: float = 1e-3, zncc_min: float = 0.8) -> float:
        """GPU reference preparation of a device-resident 8-bit image (dense
        rows `row_stride` bytes apart), without ROI; returns the device
        preparation time in ms.  For pipelines that rebuild the reference for
        every pair on the GPU."""
        if self._closed:
            raise ICGNError("This engine is closed; create a new engine before set_reference().")
        if self.pyramid_levels > 1:
            raise ICGNError("set_reference_device() supports pyramid_levels=1; use set_reference().")
        gw, gh = subset_grid_shape(width, height, subset_size=self.subset_size, subset_stride=self.subset_stride)
        if gw < 1 or gh < 1:
            raise ValueError(f"Reference dimensions must each be at least {self.subset_size} pixels.")
        config = _validated_config(iterations, tolerance, zncc_min)
        self._reference_ready = False
        self._target_ready = False
        info = _native.RefInfo()
        self._check(self._lib.gbdic_set_reference_device(
            self._handle, C.c_void_p(device_image), int(width), int(height), int(row_stride or width), None, None,
            C.byref(info)))
        self.width, self.height, self.grid_width, self.grid_height = int(width), int(height), gw, gh
        self._config = config
        self.roi = None
        admissible = self._export(_native.EXPORT_ADMISSIBLE, np.uint8, (gh, gw))
        self.reference_valid = immutable(admissible.astype(bool))
        self._reference_ready = True
        self.reference_generation += 1
        return float(info.device_ms)

    def _prepare_partial(self, roi: RoiPlan) -> RoiPlan:
        """Partial-window metadata from the GPU-prepared plane (float64 host
        preparation, partial.py:26-121), uploaded with the support tables."""
        from .partial import install_partial_reference

        return install_partial_reference(
            roi, self._export,
            lambda *args: self._check(self._lib.gbdic_set_partial_support(self._handle, *args)),
            width=self.width, height=self.height, size=self.subset_size, stride=self.subset_stride,
            motion_model=self.motion_model, weighting=self.spatial_weighting, sigma=self.gaussian_sigma)

    def set_reference_arrays(
        self,
        width: int,
        height: int,
        plane: np.ndarray,
        metadata: np.ndarray,
        inverse: np.ndarray,
        *,
        iterations: int = 30,
        tolerance: float = 1e-3,
        zncc_min: float = 0.8,
    ) -> None:
        """Upload reference arrays prepared elsewhere, in the reference's own
        layout (plane H*W*4, metadata grid*16|28, inverse grid*n*n)."""
        gw, gh = subset_grid_shape(width, height, subset_size=self.subset_size, subset_stride=self.subset_stride)
        n = parameter_count(self.motion_model)
        stride = 28 if self.motion_model == "quadratic" else 16
        plane = np.ascontiguousarray(plane, dtype=np.float32).ravel()
        metadata = np.ascontiguousarray(metadata, dtype=np.float32).ravel()
        inverse = np.ascontiguousarray(inverse, dtype=np.float32).ravel()
        if plane.size != width * height * 4 or metadata.size != gw * gh * stride or inverse.size != gw * gh * n * n:
            raise ValueError("reference arrays do not match the image and grid dimensions")
        config = _validated_config(iterations, tolerance, zncc_min)
        info = _native.RefInfo()
        self._check(
            self._lib.gbdic_set_reference_arrays(
                self._handle, width, height, _native.ptr(plane), _native.ptr(metadata), _native.ptr(inverse),
                None, C.byref(info),
            )
        )
        self.width, self.height, self.grid_width, self.grid_height = width, height, gw, gh
        self._config = config
        self.roi = None
        flags = metadata.reshape(-1, stride)[:, 1]
        self.reference_valid = immutable(((flags > 0.5) | (flags == -4)).reshape(gh, gw))
        self._reference_ready = True
        self.reference_generation += 1

    # ------------------------------------------------------------ exports
    def _export(self, what: int, dtype, shape) -> np.ndarray:
        out = np.empty(shape, dtype=dtype)
        self._check(self._lib.gbdic_export(self._handle, what, _native.ptr(out), out.nbytes))
        return out

    def export_metadata(self) -> np.ndarray:
        stride = 28 if self.motion_model == "quadratic" else 16
        return self._export(_native.EXPORT_METADATA, np.float32, (self.grid_width * self.grid_height, stride))

    def export_reference(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(plane H*W*4, inverse grid*n*n, metadata grid*16|28) as prepared on the GPU."""
        n = parameter_count(self.motion_model)
        count = self.grid_width * self.grid_height
        plane = self._export(_native.EXPORT_PLANE, np.float32, (self.height * self.width * 4,))
        inverse = self._export(_native.EXPORT_INVERSE, np.float32, (count * n * n,))
        metadata = self.export_metadata().ravel()
        return plane, inverse, metadata

    def export_coefficients(self) -> np.ndarray:
        """B-spline coefficient plane of the last target (bspline mode)."""
        return self._export(_native.EXPORT_COEFFICIENTS, np.float32, (self.height, self.width))

    def export_weights(self) -> np.ndarray:
        return self._export(_native.EXPORT_WEIGHTS, np.float32, (self.subset_size * self.subset_size,))

    def export_raw_state(self) -> np.ndarray:
        return self._export(_native.EXPORT_RAW_STATE, np.float32, (self.grid_height, self.grid_width, state_float_count(self.motion_model)))

    def apply_outlier_filter(self, state: np.ndarray, *, seed_mode: bool = False) -> np.ndarray:
        """Run this engine's outlier policy on a packed state field
        (grid_height, grid_width, 8|16) on the GPU and return the result."""
        stride = state_float_count(self.motion_model)
        src = np.ascontiguousarray(state, dtype=np.float32)
        if src.shape != (self.grid_height, self.grid_width, stride):
            raise ValueError(f"state must have shape {(self.grid_height, self.grid_width, stride)}")
        out = np.empty_like(src)
        self._check(self._lib.gbdic_apply_uod(self._handle, _native.ptr(src), int(seed_mode), _native.ptr(out)))
        return out

    # ------------------------------------------------------------ solves
    def _empty_roi_result(self, started: float, config) -> RegistrationResult:
        packed = np.zeros((self.grid_height, self.grid_width, state_float_count(self.motion_model)), np.float32)
        packed[..., parameter_count(self.motion_model)] = -3.0
        elapsed = (time.perf_counter() - started) * 1e3
        return self._result(packed, {"queueSubmissions": 0.0, "totalWallMs": elapsed, "resultAgeWallMs": elapsed}, config)

    def _check_final_zncc(self) -> None:
        if self.motion_model != "affine" or self.spatial_weighting != "uniform":
            raise ValueError("include_zncc requires affine motion and uniform full windows")

    def _attach_final_zncc(self, result: RegistrationResult) -> None:
        start = time.perf_counter()
        zncc = np.empty(self.grid_width * self.grid_height, np.float32)
        self._check(self._lib.gbdic_final_zncc(self._handle, _native.ptr(zncc)))
        zncc[zncc < -1.0] = np.nan
        result._zncc = immutable(zncc.reshape(self.grid_height, self.grid_width))
        elapsed = (time.perf_counter() - start) * 1e3
        result.timing = {**result.timing, "finalZnccWallMs": elapsed, "totalWallMs": result.timing["totalWallMs"] + elapsed}

    @_exclusive_call
    def register(
        self,
        target: ImageInput,
        *,
        iterations: int | None = None,
        tolerance: float | None = None,
        zncc_min: float | None = None,
        include_zncc: bool = False,
    ) -> RegistrationResult:
        if not self._reference_ready:
            raise ICGNError("Call set_reference() before register().")
        if include_zncc:
            self._check_final_zncc()
            if self.pyramid_levels != 1:
                raise ValueError("include_zncc requires a single pyramid level")
        started = time.perf_counter()
        frame = self._prepare_target(target)
        self._config = self._resolve_config(iterations, tolerance, zncc_min)
        if self.roi is not None and self.roi.empty:
            result = self._empty_roi_result(started, self._config)
            if include_zncc:
                result._zncc = immutable(np.full((self.grid_height, self.grid_width), np.nan, np.float32))
            return result
        packed = self._new_packed()
        timing = _native.Timing()
        self._check(
            self._lib.gbdic_register(
                self._handle, _native.ptr(frame), frame.strides[0], C.byref(self._cfg(self._config)),
                _native.ptr(packed), C.byref(timing),
            )
        )
        self._target_ready = True
        times = self._timing(timing)
        times["totalWallMs"] = (time.perf_counter() - started) * 1e3
        result = self._result(packed, times, self._config)
        if self._pyramid_engines:
            result = self._recover_pyramid(0, frame, packed, result)
        if include_zncc:
            self._attach_final_zncc(result)
        return result

    # ------------------------------------------------------------ selective pyramid recovery
    def _close_pyramid_engines(self) -> None:
        engines = getattr(self, "_pyramid_engines", [])
        for engine in engines:
            engine.close()
        engines.clear()
        self._roi_seed_permissions = None

    def _prepare_pyramid(self, reference: np.ndarray, *, zncc_min: float) -> None:
        """Coarse references of the selective recovery (wgpu_backend.py:2303-2362):
        one single-scale engine per coarser level on the reduced reference
        (12 iterations, tolerance 1e-2), reduced ROI masks and coarse-to-fine
        seed permissions."""
        self._close_pyramid_engines()
        reduced = reference
        mask = None if self.roi is None else self.roi.mask
        for _ in range(1, self.pyramid_levels):
            reduced = reduce_half(reduced)
            mask = None if mask is None else reduce_mask(mask)
            engine = ICGNWGPU(
                solver_workgroup_size=self.solver_workgroup_size, pyramid_levels=1,
                interpolation=self.interpolation, motion_model=self.motion_model,
                outlier_policy=self.outlier_policy, median_filter_size=self.median_filter_size,
                subset_size=self.subset_size, subset_stride=self.subset_stride,
                spatial_weighting=self.spatial_weighting, gaussian_sigma=self.gaussian_sigma,
                device=self.device_index, pipeline_slots=1,
            )
            try:
                engine.set_reference(reduced, iterations=12, tolerance=1e-2, zncc_min=zncc_min, roi_mask=mask,
                                     roi_policy="full" if self.roi is None else self.roi.policy,
                                     roi_truncation="none" if self.roi is None else self.roi.truncation)
            except Exception:
                engine.close()
                self._close_pyramid_engines()
                raise
            self._pyramid_engines.append(engine)
        levels = [self, *self._pyramid_engines]
        for level in levels:
            level._roi_seed_permissions = None
        if self.roi is not None and self.roi.effective:
            prefix = integral(self.roi.mask)
            for index, (destination, source) in enumerate(zip(levels[:-1], levels[1:], strict=True)):
                destination._roi_seed_permissions = seed_permissions(
                    source.roi, destination.roi, source_scale=1 << (index + 1), destination_scale=1 << index,
                    size=self.subset_size, stride=self.subset_stride, reference_mask=self.roi.mask,
                    reference_prefix=prefix)

    def _register_seeded_states(self, frame: np.ndarray, seeds: np.ndarray, active: np.ndarray) -> np.ndarray:
        """Seeded solve from full seed states (the reference's
        _register_seeded_frame, wgpu_backend.py:1951-2036); returns the packed field."""
        packed = self._new_packed()
        timing = _native.Timing()
        act = np.ascontiguousarray(active, dtype=np.uint32)
        if self.roi is not None:
            act = act * self.roi.selected.astype(np.uint32)
        self._check(self._lib.gbdic_register_seeded(
            self._handle, _native.ptr(frame), frame.strides[0], _native.ptr(np.ascontiguousarray(seeds)),
            _native.ptr(np.ascontiguousarray(act)), C.byref(self._cfg(self._config)), _native.ptr(packed),
            C.byref(timing)))
        self._target_ready = True
        return packed

    def _register_seeded_resident(self, seeds: np.ndarray, active: np.ndarray) -> np.ndarray:
        """_register_seeded_states on the target already resident in slot 0
        (put there by gbdic_reduce_frame)."""
        packed = self._new_packed()
        timing = _native.Timing()
        act = np.ascontiguousarray(active, dtype=np.uint32)
        if self.roi is not None:
            act = act * self.roi.selected.astype(np.uint32)
        self._check(self._lib.gbdic_register_seeded_resident(
            self._handle, _native.ptr(np.ascontiguousarray(seeds)), _native.ptr(np.ascontiguousarray(act)),
            C.byref(self._cfg(self._config)), _native.ptr(packed), C.byref(timing)))
        self._target_ready = True
        return packed

    def _recover_pyramid(self, slot: int, frame: np.ndarray, fine_packed: np.ndarray,
                         fine_result: RegistrationResult) -> RegistrationResult:
        """Re-solve failed fine subsets from coarse-to-fine seeds
        (wgpu_backend.py:2038-2197)."""
        recoverable = np.zeros(fine_result.status.shape, dtype=np.bool_)
        if self.grid_width > 2 and self.grid_height > 2:
            recoverable[1:-1, 1:-1] = True
        failed = (np.asarray(fine_result.status) < 0.5) & recoverable
        if self.roi is not None:
            failed &= self.roi.selected
        failed_count = int(np.count_nonzero(failed))
        if failed_count == 0:
            return fine_result
        started = time.perf_counter()
        # The coarser targets are reduced on the device from the frame this
        # engine holds in `slot`, level by level (bit-identical to
        # _reduce_half, wgpu_backend.py:318-334).
        finer, finer_slot = self, int(slot)
        for engine in self._pyramid_engines:
            engine._check(engine._lib.gbdic_reduce_frame(engine._handle, finer._handle, finer_slot))
            finer, finer_slot = engine, 0
        requested_by_level = []
        requested = failed
        destination_scale = 1
        for level_index, engine in enumerate(self._pyramid_engines):
            level_scale = 1 << (level_index + 1)
            requested = pyramid_dependency_mask(
                source_grid=(engine.grid_width, engine.grid_height), source_scale=level_scale,
                destination_scale=destination_scale, requested=requested, subset_size=self.subset_size,
                subset_stride=self.subset_stride)
            requested_by_level.append(requested)
            if engine.roi is not None:
                requested &= engine.roi.selected
            destination_scale = level_scale
        n = parameter_count(self.motion_model)
        source = None  # (parameters, status, available, scale)
        for level_index in range(len(self._pyramid_engines) - 1, -1, -1):
            engine = self._pyramid_engines[level_index]
            level_scale = 1 << (level_index + 1)
            level_requested = requested_by_level[level_index]
            if source is None:
                seeds = np.zeros((engine.grid_height, engine.grid_width, state_float_count(self.motion_model)),
                                 np.float32)
                active = level_requested.astype(np.uint32)
            else:
                seeds, active = transfer_pyramid_seed(
                    source[0], source[1], motion_model=self.motion_model, source_available=source[2],
                    source_scale=source[3], destination_scale=level_scale,
                    destination_grid=(engine.grid_width, engine.grid_height), requested=level_requested,
                    subset_size=self.subset_size, subset_stride=self.subset_stride,
                    permissions=engine._roi_seed_permissions)
            level_packed = engine._register_seeded_resident(seeds, active)
            source = (level_packed[..., :n], level_packed[..., n], level_requested, level_scale)
        seeds, active = transfer_pyramid_seed(
            source[0], source[1], motion_model=self.motion_model, source_available=source[2],
            source_scale=source[3], destination_scale=1, destination_grid=(self.grid_width, self.grid_height),
            requested=failed, subset_size=self.subset_size, subset_stride=self.subset_stride,
            permissions=self._roi_seed_permissions)
        recovered = self._new_packed()
        timing = _native.Timing()
        self._check(self._lib.gbdic_retry_seeded(
            self._handle, int(slot), _native.ptr(np.ascontiguousarray(seeds)), _native.ptr(np.ascontiguousarray(active)),
            C.byref(self._cfg(self._config)), _native.ptr(recovered), C.byref(timing)))
        recovered_count = int(np.count_nonzero(failed & (recovered[..., n] >= 0.5)))
        preserved = np.asarray(fine_result.status) >= 0.5
        recovered[preserved] = fine_packed[preserved]
        times = dict(fine_result.timing)
        times.update(self._timing(timing))
        pyramid_ms = (time.perf_counter() - started) * 1e3
        times.update({"pyramidFailedBefore": float(failed_count), "pyramidRecovered": float(recovered_count),
                      "pyramidLevels": float(self.pyramid_levels), "pyramidWallMs": pyramid_ms,
                      "totalWallMs": fine_result.timing["totalWallMs"] + pyramid_ms})
        return self._result(recovered, times, self._config)

    # ------------------------------------------------------------ spatial seeds
    def _spatial_permissions(self) -> tuple[np.ndarray, np.ndarray]:
        """(usable windows, 3x3 permission words) as the reference builds them
        for its spatial-seed passes (wgpu_backend.py:2696-2711)."""
        shape = (self.grid_height, self.grid_width)
        valid = np.asarray(self.reference_valid, dtype=bool).copy()
        if self.roi is not None:
            valid &= self.roi.selected
        permissions = np.zeros(shape, dtype=np.uint32)
        padded = np.pad(valid, 1)
        for dy in range(-1, 2):
            for dx in range(-1, 2):
                neighbour = padded[1 + dy: 1 + dy + shape[0], 1 + dx: 1 + dx + shape[1]]
                permissions |= (valid & neighbour).astype(np.uint32) << ((dy + 1) * 3 + dx + 1)
        if self.roi is not None:
            permissions &= np.asarray(self.roi.neighbour_bits, dtype=np.uint32)
        return valid, permissions

    def _spatial_inputs(self, parameters: Any, accepted: Any, what: str) -> tuple[np.ndarray, np.ndarray]:
        if not self._reference_ready:
            raise ICGNError(f"Call set_reference() before {what}().")
        shape = (self.grid_height, self.grid_width)
        values = np.asarray(parameters, dtype=np.float32)
        mask = np.asarray(accepted)
        if values.shape != (*shape, 6):
            raise ValueError(f"parameters must have shape {(*shape, 6)}")
        if mask.shape != shape or mask.dtype != np.bool_:
            raise ValueError(f"accepted must be a Boolean array with shape {shape}")
        if not np.isfinite(values[mask]).all():
            raise ValueError("accepted parameters must be finite")
        return values, mask

    def affine_frontier_seeds(self, parameters: Any, accepted: Any) -> tuple[np.ndarray, np.ndarray]:
        """Median first-order transports of accepted affine neighbours onto
        the next frontier (wgpu_backend.py:2671-2771).  Returns seeds
        (grid_h, grid_w, 6) and the Boolean frontier; these are guesses for
        register_seeded, not accepted results."""
        values, mask = self._spatial_inputs(parameters, accepted, "affine_frontier_seeds")
        if self.motion_model != "affine":
            raise ValueError("affine_frontier_seeds requires motion_model='affine'")
        shape = (self.grid_height, self.grid_width)
        valid, permissions = self._spatial_permissions()
        accepted_valid = mask & valid
        packed = np.zeros((*shape, 8), dtype=np.float32)
        packed[..., :6] = np.where(accepted_valid[..., None], values, 0)
        packed[..., 6] = accepted_valid
        seeds = np.zeros((*shape, 8), dtype=np.float32)
        active = np.zeros(shape, dtype=np.uint8)
        permissions = np.ascontiguousarray(permissions)
        self._check(self._lib.gbdic_affine_frontier(self._handle, _native.ptr(packed), _native.ptr(permissions),
                                                    _native.ptr(seeds), _native.ptr(active)))
        return seeds[..., :6].copy(), active.astype(bool)

    _CANDIDATE_MODES = {"neighbours": 0, "median": 1, "neighbours+median": 2}

    def spatial_seed_candidates(
        self,
        parameters: Any,
        accepted: Any,
        *,
        prior: Any = None,
        sample_step: int = 1,
        min_gain: float = 0.0,
        min_displacement: float = 0.0,
        failed_only: bool = False,
        candidate_mode: str = "neighbours",
    ) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Translation seed selection on the target of the last register()
        (spatial_seed.wgsl:65-190, `choose`): ZNCC of the own translation, the
        prior's, the 3x3 neighbours' and/or their median, every
        `sample_step`-th pixel, bilinear target.  Returns (seeds (gh, gw, 6)
        for improved subsets, the Boolean improved mask, scores (gh, gw, 2):
        own and best ZNCC, 0 where not scored)."""
        values, mask = self._spatial_inputs(parameters, accepted, "spatial_seed_candidates")
        if not self._target_ready:
            raise ICGNError("Call register() before spatial_seed_candidates().")
        if candidate_mode not in self._CANDIDATE_MODES:
            raise ValueError(f"candidate_mode must be one of {tuple(self._CANDIDATE_MODES)}")
        if isinstance(sample_step, bool) or not 1 <= int(sample_step) <= self.subset_size:
            raise ValueError("sample_step must be an integer in [1, subset_size]")
        if not (float(min_gain) >= 0.0 and float(min_displacement) >= 0.0):
            raise ValueError("min_gain and min_displacement must be non-negative")
        shape = (self.grid_height, self.grid_width)
        _, permissions = self._spatial_permissions()
        packed = np.zeros((*shape, 8), dtype=np.float32)
        packed[..., :6] = np.nan_to_num(values, nan=0.0, posinf=0.0, neginf=0.0)
        packed[..., 6] = mask
        prior_packed = None
        if prior is not None:
            pv = np.asarray(prior, dtype=np.float32)
            if pv.shape != (*shape, 6):
                raise ValueError(f"prior must have shape {(*shape, 6)}")
            prior_packed = np.zeros((*shape, 8), dtype=np.float32)
            prior_packed[..., :6] = pv
        cfg = _native.ChooseCfg(int(sample_step), float(min_gain), float(min_displacement), int(bool(failed_only)),
                                self._CANDIDATE_MODES[candidate_mode])
        seeds = np.zeros((*shape, 8), dtype=np.float32)
        scores = np.zeros((*shape, 4), dtype=np.float32)
        active = np.zeros(shape, dtype=np.uint8)
        permissions = np.ascontiguousarray(permissions)
        self._check(self._lib.gbdic_spatial_choose(self._handle, _native.ptr(packed), _native.ptr(prior_packed),
                                                   _native.ptr(permissions), C.byref(cfg), _native.ptr(seeds),
                                                   _native.ptr(scores), _native.ptr(active)))
        return seeds[..., :6].copy(), active.astype(bool), scores[..., :2].copy()

    @_exclusive_call
    def register_seeded(
        self,
        target: ImageInput,
        parameters: Any,
        active: Any,
        *,
        iterations: int | None = None,
        tolerance: float | None = None,
        zncc_min: float | None = None,
        include_zncc: bool = False,
    ) -> RegistrationResult:
        """Solve the active subsets from supplied initial warps
        (reference: wgpu_backend.py:2774-2819).  ``parameters`` has shape
        (grid_height, grid_width, 6) in result order; ``active`` is a Boolean
        grid.  Inactive or ROI-excluded windows are not solved."""
        if not self._reference_ready:
            raise ICGNError("Call set_reference() before register_seeded().")
        if self.motion_model != "affine":
            raise ValueError("register_seeded currently requires motion_model='affine'")
        if include_zncc:
            self._check_final_zncc()
        shape = (self.grid_height, self.grid_width)
        values = np.asarray(parameters, dtype=np.float32)
        mask = np.asarray(active)
        if values.shape != (*shape, 6):
            raise ValueError(f"parameters must have shape {(*shape, 6)}")
        if mask.shape != shape or mask.dtype != np.bool_:
            raise ValueError(f"active must be a Boolean array with shape {shape}")
        if not np.isfinite(values[mask]).all():
            raise ValueError("active parameters must be finite")
        started = time.perf_counter()
        frame = self._prepare_target(target)
        self._config = self._resolve_config(iterations, tolerance, zncc_min)
        seeds = np.zeros((*shape, 8), dtype=np.float32)
        seeds[..., :6] = np.where(mask[..., None], values, 0)
        act = mask.astype(np.uint32)
        if self.roi is not None:
            act = act * self.roi.selected.astype(np.uint32)
        packed = self._new_packed()
        timing = _native.Timing()
        self._check(
            self._lib.gbdic_register_seeded(
                self._handle, _native.ptr(frame), frame.strides[0], _native.ptr(seeds), _native.ptr(np.ascontiguousarray(act)),
                C.byref(self._cfg(self._config)), _native.ptr(packed), C.byref(timing),
            )
        )
        self._target_ready = True
        times = self._timing(timing)
        times["totalWallMs"] = (time.perf_counter() - started) * 1e3
        result = self._result(packed, times, self._config)
        if include_zncc:
            self._attach_final_zncc(result)
        return result

    @_exclusive_stream
    def register_stream(
        self,
        targets: Iterable[ImageInput],
        *,
        pipeline_depth: int = DEFAULT_IN_FLIGHT_FRAMES,
        iterations: int | None = None,
        tolerance: float | None = None,
        zncc_min: float | None = None,
    ) -> Iterator[RegistrationResult]:
        """Register a sequence with up to ``pipeline_depth`` frames in flight;
        results come back in input order (wgpu_backend.py:2997-3051)."""
        if not self._reference_ready:
            raise ICGNError("Call set_reference() before register_stream().")
        try:
            depth = operator.index(pipeline_depth)
        except TypeError as error:
            raise ValueError("pipeline_depth must be a positive integer") from error
        if isinstance(pipeline_depth, bool) or depth < 1:
            raise ValueError("pipeline_depth must be a positive integer")
        if depth > self._pipeline_slots:
            raise ValueError(f"pipeline_depth must be at most {self._pipeline_slots} for this engine")
        self._config = self._resolve_config(iterations, tolerance, zncc_min)
        if self.roi is not None and self.roi.empty:
            for target in targets:
                started = time.perf_counter()
                self._prepare_target(target)
                yield self._empty_roi_result(started, self._config)
            return
        cfg = self._cfg(self._config)
        available = deque(range(depth))
        pending: deque[tuple[int, float]] = deque()

        def retire() -> RegistrationResult:
            slot, started, frame = pending.popleft()
            packed = self._new_packed()
            timing = _native.Timing()
            self._check(self._lib.gbdic_retire(self._handle, slot, _native.ptr(packed), C.byref(timing)))
            times = self._timing(timing)
            times["pipelineLatencyWallMs"] = (time.perf_counter() - started) * 1e3
            times["totalWallMs"] = times["pipelineLatencyWallMs"]
            result = self._result(packed, times, self._config)
            if self._pyramid_engines:
                result = self._recover_pyramid(slot, frame, packed, result)
            available.append(slot)
            return result

        try:
            for target in targets:
                if not available:
                    yield retire()
                slot = available.popleft()
                started = time.perf_counter()
                frame = self._prepare_target(target)
                self._check(self._lib.gbdic_submit(self._handle, slot, _native.ptr(frame), frame.strides[0], C.byref(cfg)))
                pending.append((slot, started, frame))
            while pending:
                yield retire()
        finally:
            while pending:
                slot, _, _ = pending.popleft()
                self._lib.gbdic_retire(self._handle, slot, None, None)

    def register_many(self, targets: Iterable[ImageInput], *, pipeline_depth: int = DEFAULT_IN_FLIGHT_FRAMES,
                      iterations: int | None = None, tolerance: float | None = None,
                      zncc_min: float | None = None) -> list[RegistrationResult]:
        return list(
            self.register_stream(targets, pipeline_depth=pipeline_depth, iterations=iterations,
                                 tolerance=tolerance, zncc_min=zncc_min)
        )

    def register_device(self, device_frame: int, device_state: int, *, stream: int | None = None) -> None:
        """Resident registration: ``device_frame`` (dense 8-bit rows) and
        ``device_state`` are CUDA device addresses; no host synchronisation."""
        if not self._reference_ready:
            raise ICGNError("Call set_reference() before register().")
        self._check(
            self._lib.gbdic_register_device(
                self._handle, C.c_void_p(device_frame), C.byref(self._cfg(self._config)),
                C.c_void_p(device_state), C.c_void_p(stream or 0),
            )
        )

    # ------------------------------------------------------------ lifetime
    def close(self) -> None:
        """Release GPU resources; repeated calls are harmless."""
        if self._closed:
            return
        self._reference_ready = False
        self._closed = True
        self._close_pyramid_engines()
        handle, self._handle = self._handle, None
        if handle:
            self._lib.gbdic_destroy(handle)

    def __enter__(self) -> ICGNWGPU:
        return self

    def __exit__(self, *_: object) -> None:
        self.close()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass
