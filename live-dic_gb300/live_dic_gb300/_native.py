"""ctypes binding of libgbdic.so (include/gbdic.h).

The library is built in-tree by live-dic_gb300/build.py.  Loading fails
loudly with ICGNError when it is missing: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

from .engine import ICGNError

LIBRARY_PATH = Path(__file__).resolve().parent / "libgbdic.so"

OK, EINVAL, ESTATE, ECUDA, ETIMEOUT = 0, -1, -2, -3, -4
EXPORT_COEFFICIENTS, EXPORT_PLANE, EXPORT_METADATA, EXPORT_INVERSE = 0, 1, 2, 3
EXPORT_RAW_STATE, EXPORT_OUTPUT_STATE, EXPORT_WEIGHTS, EXPORT_FRAME = 4, 5, 6, 7
EXPORT_ADMISSIBLE, EXPORT_SEED, EXPORT_ACTIVE = 8, 9, 10


class Options(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("motion_model", C.c_int32),
        ("interpolation", C.c_int32),
        ("subset_size", C.c_int32),
        ("subset_stride", C.c_int32),
        ("spatial_weighting", C.c_int32),
        ("gaussian_sigma", C.c_float),
        ("outlier_policy", C.c_int32),
        ("median_filter_size", C.c_int32),
        ("median_filter_scope", C.c_int32),
        ("threads_per_subset", C.c_int32),
        ("divergence_patience", C.c_int32),
        ("divergence_min_iterations", C.c_int32),
        ("pipeline_slots", C.c_int32),
        ("persistent", C.c_int32),
        ("solver_mode", C.c_int32),
    ]


SOLVER_MODES = {"exact": 0, "fast": 1, "staged": 2, "staged-wide": 3}


class SolverCfg(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("tolerance", C.c_float), ("zncc_min", C.c_float)]


class RefInfo(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("grid_width", C.c_int32),
        ("grid_height", C.c_int32),
        ("valid_count", C.c_int32),
        ("device_ms", C.c_double),
    ]


class Timing(C.Structure):
    _fields_ = [
        ("upload_ms", C.c_double),
        ("execute_ms", C.c_double),
        ("readback_ms", C.c_double),
        ("total_ms", C.c_double),
        ("device_ms", C.c_double),
    ]


class NoAllocFrame(C.Structure):
    """Arguments of gbdic_register_noalloc (all pointers are device pointers)."""

    _fields_ = [
        ("frame", C.c_void_p),
        ("plane", C.c_void_p),
        ("metadata", C.c_void_p),
        ("inverse", C.c_void_p),
        ("weights", C.c_void_p),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("motion_model", C.c_int32),
        ("interpolation", C.c_int32),
        ("subset_size", C.c_int32),
        ("subset_stride", C.c_int32),
        ("threads_per_subset", C.c_int32),
        ("roi_enabled", C.c_int32),
        ("cfg", SolverCfg),
    ]


class PyramidOptions(C.Structure):
    _fields_ = [
        ("base", Options),
        ("levels", C.c_int32),
        ("iterations", C.c_int32 * 4),
        ("tolerance", C.c_float * 4),
        ("zncc_min", C.c_float),
        ("initialization", C.c_int32),
        ("temporal_max_age", C.c_uint32),
        ("temporal_prediction", C.c_int32),
        ("seed_search_radius", C.c_int32),
        ("temporal_fine_correction", C.c_int32),
        ("adaptive", C.c_int32),
    ]


class LevelRoi(C.Structure):
    _fields_ = [
        ("selected", C.POINTER(C.c_uint8)),
        ("links", C.POINTER(C.c_float)),
        ("seed_links", C.POINTER(C.c_uint32)),
    ]


class BatchJob(C.Structure):
    _fields_ = [
        ("motion_model", C.c_int32),
        ("subset_size", C.c_int32),
        ("subset_stride", C.c_int32),
        ("outlier_policy", C.c_int32),
        ("cfg", SolverCfg),
    ]


BATCH_PERSISTENT, BATCH_PER_JOB, BATCH_SINGLE = 0, 1, 2


class ChooseCfg(C.Structure):
    _fields_ = [
        ("sample_step", C.c_int32),
        ("min_gain", C.c_float),
        ("min_displacement", C.c_float),
        ("failed_only", C.c_int32),
        ("candidate_mode", C.c_int32),
    ]

class NnGemmDesc(C.Structure):
    _fields_ = [
        ("a", C.c_void_p), ("b", C.c_void_p),
        ("M", C.c_int32), ("N", C.c_int32), ("K", C.c_int32), ("k_split", C.c_int32),
        ("d_f32", C.c_void_p), ("d_bf16", C.c_void_p),
        ("ldd", C.c_int32), ("split_stride", C.c_int64),
        ("bias", C.c_void_p), ("relu", C.c_int32), ("accumulate", C.c_int32),
    ]


class NnConvShape(C.Structure):
    _fields_ = [(name, C.c_int32) for name in ("B", "H", "W", "C", "OH", "OW", "Cout", "Kp")]


P = C.c_void_p
I32, I64 = C.c_int32, C.c_int64
_SIGNATURES = {
    "gbdic_abi_version": (C.c_int, []),
    "gbdic_create": (C.c_int, [C.POINTER(Options), C.POINTER(P)]),
    "gbdic_destroy": (None, [P]),
    "gbdic_last_error": (C.c_char_p, [P]),
    "gbdic_set_reference": (C.c_int, [P, P, I32, I32, I64, P, P, C.POINTER(RefInfo)]),
    "gbdic_set_reference_arrays": (C.c_int, [P, I32, I32, P, P, P, P, C.POINTER(RefInfo)]),
    "gbdic_set_reference_device": (C.c_int, [P, P, I32, I32, I64, P, P, C.POINTER(RefInfo)]),
    "gbdic_register": (C.c_int, [P, P, I64, C.POINTER(SolverCfg), P, C.POINTER(Timing)]),
    "gbdic_register_seeded": (C.c_int, [P, P, I64, P, P, C.POINTER(SolverCfg), P, C.POINTER(Timing)]),
    "gbdic_retry_seeded": (C.c_int, [P, I32, P, P, C.POINTER(SolverCfg), P, C.POINTER(Timing)]),
    "gbdic_final_zncc": (C.c_int, [P, P]),
    "gbdic_submit": (C.c_int, [P, I32, P, I64, C.POINTER(SolverCfg)]),
    "gbdic_retire": (C.c_int, [P, I32, P, C.POINTER(Timing)]),
    "gbdic_register_device": (C.c_int, [P, P, C.POINTER(SolverCfg), P, P]),
    "gbdic_export": (C.c_int, [P, I32, P, I64]),
    "gbdic_apply_uod": (C.c_int, [P, P, I32, P]),
    "gbdic_pyramid_create": (C.c_int, [C.POINTER(PyramidOptions), C.POINTER(P)]),
    "gbdic_pyramid_destroy": (None, [P]),
    "gbdic_pyramid_last_error": (C.c_char_p, [P]),
    "gbdic_pyramid_set_reference": (C.c_int, [P, P, I32, I32, I64, P, P, C.POINTER(RefInfo)]),
    "gbdic_pyramid_level_grid": (C.c_int, [P, I32, C.POINTER(I32), C.POINTER(I32)]),
    "gbdic_pyramid_submit": (C.c_int, [P, I32, P, I64]),
    "gbdic_pyramid_retire": (C.c_int, [P, I32, P, P, C.POINTER(Timing)]),
    "gbdic_pyramid_register": (C.c_int, [P, P, I64, P, P, C.POINTER(Timing)]),
    "gbdic_pyramid_register_device": (C.c_int, [P, P, P, P]),
    "gbdic_pyramid_reset_temporal": (C.c_int, [P]),
    "gbdic_pyramid_export": (C.c_int, [P, I32, I32, P, I64]),
    "gbdic_profile": (C.c_int, [P, I32]),
    "gbdic_profile_read": (C.c_int, [P, P, P, P, P]),
    "gbdic_pyramid_profile": (C.c_int, [P, I32]),
    "gbdic_pyramid_profile_read": (C.c_int, [P, P, P, P, P]),
    "gbdic_fp32_peak_probe": (C.c_int, [I32, P]),
    "gbdic_register_noalloc": (C.c_int, [C.POINTER(NoAllocFrame), P, P]),
    "gbdic_set_solver_variant": (C.c_int, [P, I32, I32]),
    "gbdic_pyramid_set_solver_variant": (C.c_int, [P, I32, I32]),
    "gbdic_set_solver_mode": (C.c_int, [P, I32]),
    "gbdic_reduce_frame": (C.c_int, [P, P, I32]),
    "gbdic_register_seeded_resident": (C.c_int, [P, P, P, C.POINTER(SolverCfg), P, C.POINTER(Timing)]),
    "gbdic_pyramid_set_solver_mode": (C.c_int, [P, I32]),
    "gbdic_batch_create": (C.c_int, [I32, C.POINTER(P)]),
    "gbdic_batch_destroy": (C.c_int, [P]),
    "gbdic_batch_last_error": (C.c_char_p, [P]),
    "gbdic_batch_add": (C.c_int, [P, C.POINTER(BatchJob), P, I32, I32, I64, P, P, C.POINTER(RefInfo), C.POINTER(I32)]),
    "gbdic_batch_set_variant": (C.c_int, [P, I32, I32, I32]),
    "gbdic_batch_register": (C.c_int, [P, P, P, P, C.POINTER(Timing)]),
    "gbdic_batch_load_device": (C.c_int, [P, I32, P, I64, P]),
    "gbdic_batch_run_device": (C.c_int, [P, P, I32, C.POINTER(Timing)]),
    "gbdic_batch_export": (C.c_int, [P, I32, I32, P, I64]),
    "gbdic_affine_frontier": (C.c_int, [P, P, P, P, P]),
    "gbdic_spatial_choose": (C.c_int, [P, P, P, P, C.POINTER(ChooseCfg), P, P, P]),
    "gbdic_nn_gemm": (C.c_int, [C.POINTER(NnGemmDesc), P, P]),
    "gbdic_nn_conv_gemm": (C.c_int, [C.POINTER(NnGemmDesc), I32, C.POINTER(NnConvShape), P, P]),
    "gbdic_nn_relu_bias_backward": (C.c_int, [P, I32, P, I64, I32, P, P, P, P, P]),
    "gbdic_nn_splitk_bias_relu": (C.c_int, [P, I32, I64, I32, I64, P, I32, P, P]),
    "gbdic_nn_im2col_t": (C.c_int, [C.POINTER(NnConvShape), P, P, I32, P]),
    "gbdic_nn_patches": (C.c_int, [P, P, P, P, I32, I32, I32, P, P, I32, C.c_float, P]),
    "gbdic_nn_im2col": (C.c_int, [C.POINTER(NnConvShape), P, P, P]),
    "gbdic_nn_dgrad_gather": (C.c_int, [C.POINTER(NnConvShape), P, P, P]),
    "gbdic_nn_transpose": (C.c_int, [P, I32, I32, I32, P, I32, I32, P]),
    "gbdic_nn_relu_backward": (C.c_int, [P, I32, P, P, I64, I32, P]),
    "gbdic_nn_bias_grad": (C.c_int, [P, I32, P, I64, I32, P, P]),
    "gbdic_nn_splitk_reduce": (C.c_int, [P, I32, I32, I32, I32, P, P]),
    "gbdic_nn_adam": (C.c_int, [P, P, P, P, I64, P, P]),
    "gbdic_nn_adam_many": (C.c_int, [P, P, P, P, P, I32, P, P]),
    "gbdic_nn_pack_weights": (C.c_int, [P, I32, I32, I32, P, P, I32, P]),
    "gbdic_nn_regression_loss": (C.c_int, [P, I32, P, I32, I32, P, P, I32, P, P]),
    "gbdic_reduce_half": (C.c_int, [P, I32, I32, P, P]),
    "gbdic_nn_lattice_seeds": (C.c_int, [P, P, I32, I32, I32, I32, I32, I32, I32, C.c_float, C.c_float, P, P, P]),
    "gbdic_nn_conv_c2_direct": (C.c_int, [C.POINTER(NnConvShape), P, P, P, P, P]),
    "gbdic_nn_consensus": (C.c_int, [P, P, I32, I32, P, P, I32, P, I32, P, I32, P, I32, C.c_float, P]),
    "gbdic_nn_reseed_select": (C.c_int, [P, I32, P, I32, P, P, P, P]),
    "gbdic_nn_reseed_select_list": (C.c_int, [P, I32, P, I32, P, P, P, P, P]),
    "gbdic_nn_merge_rows": (C.c_int, [P, P, I32, I32, P, P]),
    "gbdic_nn_node_rows": (C.c_int, [P, I32, I32, I32, I32, I32, P, P, I32, C.c_float, C.c_float, P]),
    "gbdic_register_seeded_device": (C.c_int, [P, P, P, P, C.POINTER(SolverCfg), P, P]),
    "gbdic_resolve_seeded_device": (C.c_int, [P, P, P, P, C.POINTER(SolverCfg), P, P]),
    "gbdic_search_seeds_device": (C.c_int, [P, P, P, P, P, I32, I32, P]),
    "gbdic_search_seeds_listed_device": (C.c_int, [P, P, P, P, P, P, I32, I32, P]),
    "gbdic_solve_listed_device": (C.c_int, [P, P, P, P, P, I32, P, I32, I32, C.POINTER(SolverCfg), P, P]),
    "gbdic_pyramid_set_translation": (C.c_int, [P, I32, C.c_float, C.c_float]),
    "gbdic_set_partial_support": (C.c_int, [P, I32, P, P, I32, P, P, P]),
    "gbdic_field_summary": (C.c_int, [P, I64, I32, I32, P, P, P, C.POINTER(I64), C.POINTER(I64)]),
    "gbdic_pyramid_set_partial_support": (C.c_int, [P, I32, I32, P, P, I32, P, P, P]),
    "gbdic_pyramid_set_active_levels": (C.c_int, [P, I32]),
    "gbdic_fourier_create": (C.c_int, [I32, P, P, I32, C.POINTER(P)]),
    "gbdic_fourier_destroy": (C.c_int, [P]),
    "gbdic_fourier_last_error": (C.c_char_p, [P]),
    "gbdic_fourier_estimate": (C.c_int, [P, P, I64, I32, I32, I32, I32, P]),
    "gbdic_fourier_shift_device": (C.c_int, [P, P, I64, I32, I32, I32, C.c_float, P, I32, I32, P]),
}
EXPORTED_SYMBOLS = tuple(_SIGNATURES)

_lib = None
_lock = threading.Lock()


def load() -> C.CDLL:
    """Load libgbdic.so (once).  Raises ICGNError when it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIBRARY_PATH.exists():
                raise ICGNError(
                    f"The CUDA library {LIBRARY_PATH} is missing; build it with "
                    "`python live-dic_gb300/build.py` (nvcc for sm_103a is required)."
                )
            lib = C.CDLL(str(LIBRARY_PATH))
            for name, (restype, argtypes) in _SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = restype
                fn.argtypes = argtypes
            _lib = lib
    return _lib


def ptr(array: np.ndarray | None) -> int | None:
    return None if array is None else array.ctypes.data


def check(code: int, message: bytes | None) -> None:
    """Map a gbdic return code to the reference's exception types."""
    if code == OK:
        return
    text = (message or b"").decode("utf-8", "replace") or f"gbdic error {code}"
    if code == EINVAL:
        raise ValueError(text)
    raise ICGNError(text)


def cuda_device_count() -> int:
    """Number of visible CUDA devices (0 without a driver)."""
    try:
        rt = C.CDLL("libcudart.so")
    except OSError:
        try:
            import torch  # PyTorch is only used to locate the runtime here

            return int(torch.cuda.device_count())
        except Exception:
            return 0
    count = C.c_int(0)
    if rt.cudaGetDeviceCount(C.byref(count)) != 0:
        return 0
    return int(count.value)
