"""Batched registration of many fixed-reference jobs in one step.

No reference counterpart: the reference creates one ICGNWGPU engine per
image size and registers pairs one call at a time (wgpu_backend.py:2893-2944),
so its analogue of a batch is a loop of per-pair calls.  Here every job keeps
the arithmetic of ICGNWGPU.register (B-spline interpolation, uniform
weighting, zero seed, the job's outlier pass) and a step runs all jobs as one
CUDA graph: every target's prefilter, one persistent IC-GN launch per
shape-function class over a device work queue ("persistent"), or one
persistent launch over every job with the shape function dispatched per job
("single"), then the outlier passes.
A job's result is bit-identical to ICGNWGPU.register with the same lanes per
subset.

    with ICGNBatch() as batch:
        batch.add(reference_a, subset_size=21, subset_stride=7)
        batch.add(reference_b, motion_model="quadratic", subset_size=41, subset_stride=13)
        results = batch.register([target_a, target_b])
"""

from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass
from statistics import median

import numpy as np

from . import _native
from .autotune import compare_solver_outputs
from .engine import ICGNError, RegistrationResult, _as_uint8_gray, result_from_packed
from .motion import MOTION_MODEL_CODES, normalize_motion_model, parameter_count, state_float_count
from .outlier import normalize_outlier_policy
from .roi import prepare_roi, validate_roi
from .subset import normalize_subset_size, normalize_subset_stride, subset_grid_shape

_POLICY = {"disabled": 0, "replace": 1, "flag": 2}
_MODES = {"persistent": _native.BATCH_PERSISTENT, "per-job": _native.BATCH_PER_JOB, "single": _native.BATCH_SINGLE}
LANE_CHOICES = (16, 32, 64, 128)


@dataclass(frozen=True)
class BatchJobInfo:
    width: int
    height: int
    grid_width: int
    grid_height: int
    motion_model: str
    subset_size: int
    subset_stride: int
    outlier_policy: str
    valid_count: int
    preparation_device_ms: float
    roi: object = None

    @property
    def subsets(self) -> int:
        return self.grid_width * self.grid_height


class ICGNBatch:
    """Many registration jobs of uneven image size, subset size and shape
    function, registered together."""

    def __init__(self, *, device: int = 0, solver_workgroup_size: int = 16, mode: str = "single",
                 ctas_per_sm: int = 0) -> None:
        self._check_variant(solver_workgroup_size, mode, ctas_per_sm)
        self._lib = _native.load()
        handle = C.c_void_p()
        code = self._lib.gbdic_batch_create(int(device), C.byref(handle))
        _native.check(code, self._lib.gbdic_batch_last_error(None))
        self._handle = handle
        self.jobs: list[BatchJobInfo] = []
        self._configs: list[dict] = []
        self.set_variant(solver_workgroup_size, mode, ctas_per_sm)
        self.tuning_ms: dict[str, float] = {}
        self.validation: dict[str, dict] = {}

    # ------------------------------------------------------------ plumbing
    @staticmethod
    def _check_variant(lanes: int, mode: str, ctas_per_sm: int) -> None:
        if isinstance(lanes, bool) or lanes not in LANE_CHOICES:
            raise ValueError(f"solver_workgroup_size must be one of {LANE_CHOICES}")
        if mode not in _MODES:
            raise ValueError(f"mode must be one of {tuple(_MODES)}")
        if isinstance(ctas_per_sm, bool) or not 0 <= int(ctas_per_sm) <= 32:
            raise ValueError("ctas_per_sm must be in [0, 32]")

    def _check(self, code: int) -> None:
        _native.check(code, self._lib.gbdic_batch_last_error(self._handle))

    def _require_open(self) -> None:
        if self._handle is None:
            raise ICGNError("This batch is closed.")

    # ------------------------------------------------------------ jobs
    def add(
        self,
        reference,
        *,
        motion_model: str = "affine",
        subset_size: int = 21,
        subset_stride: int | None = None,
        outlier_policy: str = "replace",
        roi_mask: np.ndarray | None = None,
        iterations: int = 30,
        tolerance: float = 1e-3,
        zncc_min: float = 0.8,
    ) -> int:
        """Add a job with its reference image; returns the job index."""
        self._require_open()
        model = normalize_motion_model(motion_model)
        size = normalize_subset_size(subset_size)
        stride = normalize_subset_stride(subset_stride, subset_size=size)
        policy = normalize_outlier_policy(outlier_policy)
        if policy not in _POLICY:
            raise ValueError("batch jobs support outlier_policy 'disabled', 'replace' or 'flag'")
        if isinstance(iterations, bool) or not 1 <= int(iterations) <= 30:
            raise ValueError("iterations must be in [1, 30]")
        if not float(tolerance) > 0.0:
            raise ValueError("tolerance must be positive")
        frame = _as_uint8_gray(reference)
        height, width = frame.shape
        gw, gh = subset_grid_shape(width, height, subset_size=size, subset_stride=stride)
        if gw < 1 or gh < 1:
            raise ValueError(f"Reference dimensions must each be at least {size} pixels.")
        mask = validate_roi(roi_mask, "full", frame.shape, model, "none")
        roi = prepare_roi(mask, size, stride)
        selected = links = None
        if roi is not None and roi.effective:
            selected = np.ascontiguousarray(roi.selected, dtype=np.uint8).ravel()
            links = np.ascontiguousarray(roi.links_table(3, policy))
        job = _native.BatchJob(MOTION_MODEL_CODES[model], size, stride, _POLICY[policy],
                               _native.SolverCfg(int(iterations), float(tolerance), float(zncc_min)))
        info = _native.RefInfo()
        index = C.c_int32()
        self._check(self._lib.gbdic_batch_add(self._handle, C.byref(job), _native.ptr(frame), width, height,
                                              frame.strides[0], _native.ptr(selected), _native.ptr(links),
                                              C.byref(info), C.byref(index)))
        self.jobs.append(BatchJobInfo(width, height, gw, gh, model, size, stride, policy, info.valid_count,
                                      info.device_ms, roi))
        self._configs.append({"motionModel": model, "subsetSize": size, "subsetStride": stride,
                              "outlierPolicy": policy, "iterations": int(iterations),
                              "tolerance": float(tolerance), "znccMin": float(zncc_min)})
        return int(index.value)

    def set_variant(self, lanes: int, mode: str = "single", ctas_per_sm: int = 0) -> None:
        """Lanes per subset, step mode ('persistent': a persistent queue per
        shape-function class, 'single': one persistent queue over every job,
        'per-job': one launch per job) and persistent CTAs per SM (0: all
        resident)."""
        self._require_open()
        self._check_variant(lanes, mode, ctas_per_sm)
        self._check(self._lib.gbdic_batch_set_variant(self._handle, int(lanes), _MODES[mode], int(ctas_per_sm)))
        self.variant = (int(lanes), mode, int(ctas_per_sm))

    @property
    def variant_name(self) -> str:
        lanes, mode, ctas = self.variant
        return f"{lanes}-lane {mode}" + (f" {ctas}/SM" if ctas and mode != "per-job" else "")

    # ------------------------------------------------------------ steps
    def _register_packed(self, targets) -> tuple[list[np.ndarray], dict[str, float]]:
        self._require_open()
        if not self.jobs:
            raise ICGNError("Add at least one job before register().")
        if len(targets) != len(self.jobs):
            raise ValueError(f"expected {len(self.jobs)} targets, got {len(targets)}")
        frames, outs = [], []
        for job, target in zip(self.jobs, targets, strict=True):
            frame = _as_uint8_gray(target)
            if frame.shape != (job.height, job.width):
                raise ValueError(f"target shape {frame.shape} does not match the job's reference "
                                 f"{(job.height, job.width)}")
            frames.append(frame)
            outs.append(np.empty((job.grid_height, job.grid_width, state_float_count(job.motion_model)),
                                 np.float32))
        frame_ptrs = (C.c_void_p * len(frames))(*[f.ctypes.data for f in frames])
        strides = (C.c_int64 * len(frames))(*[f.strides[0] for f in frames])
        out_ptrs = (C.c_void_p * len(outs))(*[o.ctypes.data for o in outs])
        timing = _native.Timing()
        started = time.perf_counter()
        self._check(self._lib.gbdic_batch_register(self._handle, frame_ptrs, strides, out_ptrs, C.byref(timing)))
        wall = (time.perf_counter() - started) * 1e3
        return outs, {"uploadWallMs": timing.upload_ms, "executeReadbackWallMs": timing.execute_ms,
                      "readbackCopyWallMs": timing.readback_ms, "deviceMs": timing.device_ms,
                      "totalWallMs": wall, "batchJobs": float(len(self.jobs))}

    def register(self, targets) -> list[RegistrationResult]:
        """Register one target per job (host arrays in, host results out)."""
        outs, shared = self._register_packed(targets)
        return [
            result_from_packed(out, motion_model=job.motion_model, timing=dict(shared), config=dict(cfg),
                               width=job.width, height=job.height, subset_size=job.subset_size,
                               subset_stride=job.subset_stride, roi=job.roi)
            for job, cfg, out in zip(self.jobs, self._configs, outs, strict=True)
        ]

    def load_device(self, job: int, device_pointer: int, row_stride: int, stream: int | None = None) -> None:
        """Copy a device-resident target (raw CUDA pointer) into job `job`."""
        self._require_open()
        self._check(self._lib.gbdic_batch_load_device(self._handle, int(job), C.c_void_p(int(device_pointer)),
                                                      int(row_stride), None if stream is None else C.c_void_p(stream)))

    def run_device(self, stream: int | None = None, *, profile: bool = False, timed: bool = False) -> float | None:
        """One step from the loaded targets on `stream`.  Returns the device
        milliseconds when `timed` (the solver launches alone when `profile`)."""
        self._require_open()
        timing = _native.Timing() if (timed or profile) else None
        self._check(self._lib.gbdic_batch_run_device(self._handle, None if stream is None else C.c_void_p(stream),
                                                     int(bool(profile)),
                                                     C.byref(timing) if timing is not None else None))
        return None if timing is None else timing.device_ms

    def export_state(self, job: int, *, raw: bool = False) -> np.ndarray:
        self._require_open()
        info = self.jobs[job]
        out = np.empty((info.grid_height, info.grid_width, state_float_count(info.motion_model)), np.float32)
        what = _native.EXPORT_RAW_STATE if raw else _native.EXPORT_OUTPUT_STATE
        self._check(self._lib.gbdic_batch_export(self._handle, int(job), what, _native.ptr(out), out.nbytes))
        return out

    # ------------------------------------------------------------ tuning
    def autotune(self, targets, *, candidates=None, repeats: int = 3) -> tuple[int, str, int]:
        """Time every variant on `targets` (one per job), keep the fastest
        whose fields pass the reference's solver acceptance rule
        (wgpu_backend.py:222-299) against the per-job 32-lane baseline."""
        if candidates is None:
            candidates = [(lanes, mode, ctas) for mode in ("persistent", "single") for lanes in LANE_CHOICES
                          for ctas in (0, 2)]
            candidates += [(lanes, "per-job", 0) for lanes in LANE_CHOICES]
        self.set_variant(32, "per-job", 0)
        baseline, _ = self._register_packed(targets)
        timings, validation = {}, {}
        best, best_ms = (32, "per-job", 0), float("inf")
        for lanes, mode, ctas in candidates:
            self.set_variant(lanes, mode, ctas)
            name = self.variant_name
            fields, _ = self._register_packed(targets)
            checks = [compare_solver_outputs(b, f) for b, f in zip(baseline, fields, strict=True)]
            ok = all(c["valid"] for c in checks)
            validation[name] = {"valid": ok, "jobs": checks}
            samples = [self._register_packed(targets)[1]["deviceMs"] for _ in range(repeats)]
            timings[name] = float(median(samples))
            if ok and timings[name] < best_ms:
                best, best_ms = (lanes, mode, ctas), timings[name]
        self.tuning_ms, self.validation = timings, validation
        self.set_variant(*best)
        return best

    # ------------------------------------------------------------ lifetime
    def close(self) -> None:
        handle, self._handle = self._handle, None
        if handle:
            self._lib.gbdic_batch_destroy(handle)

    def __enter__(self) -> ICGNBatch:
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


__all__ = ["BatchJobInfo", "ICGNBatch", "parameter_count"]
