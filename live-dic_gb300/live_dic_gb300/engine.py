"""Public result and error types, and input normalisation.

Mirrors the reference's live_dic/engine.py: ICGNError (56), ReferenceInfo
(81-103), RegistrationResult (105-327) and _as_uint8_gray (778-828).
"""

from __future__ import annotations

import io
import json
import os
from collections.abc import Mapping, Sequence
from dataclasses import dataclass
from typing import Any

import numpy as np

from .motion import AFFINE_PARAMETER_ORDER, parameter_order

PARAMETER_ORDER = AFFINE_PARAMETER_ORDER
MIN_FRAME_DIMENSION = 16
ImageInput = Any


class ICGNError(RuntimeError):
    """Raised when the GPU runtime or the IC-GN computation fails."""


@dataclass(frozen=True, slots=True)
class ReferenceInfo:
    """Dimensions and timings of one reference preparation."""

    preparation_wall_ms: float
    runtime_build_wall_ms: float
    reference_build_wall_ms: float
    encoding_wall_ms: float
    total_wall_ms: float
    config: Mapping[str, Any]
    device: str
    grid: tuple[int, int]
    width: int
    height: int
    subset_size: int
    subset_stride: int
    roi: Any = None
    reference_valid: np.ndarray | None = None

    @property
    def roi_selected(self) -> np.ndarray | None:
        return None if self.roi is None else self.roi.selected


@dataclass(slots=True)
class RegistrationResult:
    """Dense registration result over the subset grid.

    ``parameters[..., :]`` is ``[tx, du/dx, du/dy, ty, dv/dx, dv/dy]``, with
    the six second derivatives appended for the quadratic model.  Status: 1
    accepted, 2 displacement outlier, 0 not converged, negative rejected
    (-1 support/singular, -2 low correlation, -3 outside the ROI)."""

    parameters: np.ndarray
    status: np.ndarray
    iterations: np.ndarray
    accepted: int
    replaced: int
    mean_translation: tuple[float, float] | None
    mean_iterations: float | None
    timing: Mapping[str, float]
    config: Mapping[str, Any]
    width: int = 512
    height: int = 512
    subset_size: int = 16
    subset_stride: int = 16
    roi: Any = None
    reference_valid: np.ndarray | None = None
    _zncc: np.ndarray | None = None

    @property
    def zncc(self) -> np.ndarray | None:
        """Optional read-only final normalised correlation; NaN = unavailable."""
        return self._zncc

    @property
    def roi_selected(self) -> np.ndarray | None:
        return None if self.roi is None else self.roi.selected

    @property
    def populations(self) -> dict[str, int | float | None]:
        selected = self.status.size if self.roi is None else self.roi.selected_count
        admissible = None
        if self.reference_valid is not None:
            valid = self.reference_valid
            if self.roi is not None:
                valid = valid & self.roi.selected
            admissible = int(np.count_nonzero(valid))
        partial = 0
        if self.roi is not None and getattr(self.roi, "partial_indices", None) is not None:
            partial = int(self.roi.partial_indices.size)
        return {
            "gridTotal": self.status.size,
            "roiSelected": selected,
            "roiExcluded": self.status.size - selected,
            "roiPartial": partial,
            "referenceAdmissible": admissible,
            "accepted": self.accepted,
            "rejectedSelected": selected - self.accepted,
            "acceptedFractionSelected": self.accepted / selected if selected else None,
        }

    @property
    def displacement(self) -> np.ndarray:
        """(tx, ty) field as a zero-copy view of the parameters."""
        return self.parameters[..., 0:4:3]

    @property
    def accepted_mask(self) -> np.ndarray:
        mask = self.status > 0.5
        return mask if self.roi is None else mask & self.roi.selected

    @property
    def flagged(self) -> int:
        return self.replaced

    @property
    def outlier_mask(self) -> np.ndarray:
        return self.status > 1.5

    @property
    def replaced_mask(self) -> np.ndarray:
        return self.outlier_mask

    @property
    def parameter_order(self) -> tuple[str, ...]:
        return parameter_order(str(self.config.get("motionModel", "affine")))

    def rmse(self, truth: Sequence[float]) -> float | None:
        """Vector RMSE of the accepted displacements against a constant (dx, dy)."""
        expected = np.asarray(truth, dtype=np.float64)
        if expected.shape != (2,):
            raise ValueError("truth must contain exactly two values: (dx, dy)")
        mask = self.accepted_mask
        if not np.any(mask):
            return None
        error = self.displacement[mask].astype(np.float64) - expected
        return float(np.sqrt(np.mean(np.sum(error * error, axis=1))))

    def save_npz(self, path: str | os.PathLike[str]) -> None:
        """Write one self-contained field (and its static ROI) to an .npz file."""
        extra: dict[str, np.ndarray] = {}
        if self.roi is not None:
            extra.update(self.roi.archive_fields())
        if self.reference_valid is not None:
            extra["reference_valid"] = self.reference_valid
        np.savez_compressed(
            path,
            parameters=self.parameters,
            displacement=self.displacement,
            status=self.status,
            iterations=self.iterations,
            parameter_order=np.asarray(self.parameter_order),
            config_json=np.asarray(json.dumps(dict(self.config), sort_keys=True, allow_nan=False)),
            populations_json=np.asarray(json.dumps(self.populations, allow_nan=False)),
            **extra,
        )


def result_from_packed(
    packed: np.ndarray,
    *,
    motion_model: str,
    timing: Mapping[str, float],
    config: Mapping[str, Any],
    width: int,
    height: int,
    subset_size: int,
    subset_stride: int,
    roi: Any = None,
    reference_valid: np.ndarray | None = None,
) -> RegistrationResult:
    """Zero-copy views of one packed (grid_h, grid_w, stride) float32 field
    (reference: wgpu_backend.py:_result_from_raw, 2595-2668)."""
    from . import _native

    n = len(parameter_order(motion_model))
    parameters = packed[..., :n]
    status = packed[..., n]
    iterations = packed[..., n + 1]
    # One pass in the library gathers the accepted subsets' translations and
    # iteration counts in grid order (the values and order of the boolean
    # selections parameters[..., 0][status > 0.5] etc.); the FP64 means are
    # then NumPy's over those contiguous arrays.
    flat = np.ascontiguousarray(packed, dtype=np.float32)
    count = flat.size // flat.shape[-1]
    picked = np.empty((3, count), np.float32)
    accepted_c, replaced_c = _native.C.c_int64(), _native.C.c_int64()
    lib = _native.load()
    _native.check(lib.gbdic_field_summary(
        _native.ptr(flat), count, flat.shape[-1], n, _native.ptr(picked[0]), _native.ptr(picked[1]),
        _native.ptr(picked[2]), _native.C.byref(accepted_c), _native.C.byref(replaced_c)),
        lib.gbdic_last_error(None))
    accepted = int(accepted_c.value)
    mean_translation = None
    mean_iterations = None
    if accepted:
        mean_translation = (
            float(np.mean(picked[0, :accepted], dtype=np.float64)),
            float(np.mean(picked[1, :accepted], dtype=np.float64)),
        )
        mean_iterations = float(np.mean(picked[2, :accepted], dtype=np.float64))
    return RegistrationResult(
        parameters=parameters,
        status=status,
        iterations=iterations,
        accepted=accepted,
        replaced=int(replaced_c.value),
        mean_translation=mean_translation,
        mean_iterations=mean_iterations,
        timing=dict(timing),
        config=dict(config),
        width=width,
        height=height,
        subset_size=subset_size,
        subset_stride=subset_stride,
        roi=roi,
        reference_valid=reference_valid,
    )


def _rgb_to_luma(source: np.ndarray) -> np.ndarray:
    """ITU-R 601-2 luma in the fixed-point form Pillow uses for mode "L":
    (19595 R + 38470 G + 7471 B + 2^15) >> 16."""
    rgb = source[..., :3].astype(np.uint32)
    luma = (rgb[..., 0] * 19595 + rgb[..., 1] * 38470 + rgb[..., 2] * 7471 + 0x8000) >> 16
    return luma.astype(np.uint8)


def _decode_file(data: Any) -> np.ndarray:
    try:
        from PIL import Image  # optional dependency
    except ImportError as error:  # pragma: no cover - depends on the environment
        raise ValueError("Reading image files requires Pillow; pass a NumPy array instead.") from error
    opened = Image.open(io.BytesIO(data) if isinstance(data, bytes) else data)
    with opened:
        if opened.mode == "F" or opened.mode.startswith("I"):
            return _as_uint8_gray(np.asarray(opened))
        return np.asarray(opened.convert("L"), dtype=np.uint8)


def _as_uint8_gray(image: ImageInput) -> np.ndarray:
    """Contiguous 8-bit grayscale frame: floats are scaled by 255 when their
    maximum is <= 1, clipped and truncated; integers must lie in [0, 255];
    RGB(A) is converted to luma; both dimensions must be >= 16."""
    if isinstance(image, (str, os.PathLike, bytes)):
        array = _decode_file(image)
    else:
        source = np.asarray(image)
        if source.ndim not in (2, 3):
            raise ValueError("Expected a 2D, RGB, or RGBA image.")
        if source.ndim == 3 and source.shape[2] not in (3, 4):
            raise ValueError("Expected an RGB or RGBA image with 3 or 4 channels.")
        if np.issubdtype(source.dtype, np.floating):
            source = np.nan_to_num(source, nan=0.0, posinf=255.0, neginf=0.0)
            scale = 255.0 if source.size and float(np.max(source)) <= 1.0 else 1.0
            source = np.clip(source * scale, 0, 255).astype(np.uint8)
        elif source.dtype != np.uint8:
            if not np.issubdtype(source.dtype, np.integer):
                raise ValueError(f"Unsupported image dtype {source.dtype}.")
            if source.size and (int(np.min(source)) < 0 or int(np.max(source)) > 255):
                raise ValueError(
                    "Integer image values must be in [0, 255]. Convert higher-bit-depth "
                    "images explicitly to uint8 with the same calibrated intensity range "
                    "for the reference and every target."
                )
            source = source.astype(np.uint8)
        array = source if source.ndim == 2 else _rgb_to_luma(source)
    height, width = array.shape
    if height < MIN_FRAME_DIMENSION or width < MIN_FRAME_DIMENSION:
        raise ValueError(
            f"Image dimensions must each be at least {MIN_FRAME_DIMENSION} pixels; received {array.shape}."
        )
    return np.ascontiguousarray(array)
