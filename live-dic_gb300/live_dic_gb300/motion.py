"""Motion models, parameter order and state layout
(reference: live_dic/motion.py:7-56)."""

from __future__ import annotations

MOTION_MODELS = ("affine", "translation", "quadratic")
MOTION_MODEL_CODES = {"affine": 0, "translation": 1, "quadratic": 2}
AFFINE_PARAMETER_ORDER = ("tx", "du_dx", "du_dy", "ty", "dv_dx", "dv_dy")
QUADRATIC_PARAMETER_ORDER = AFFINE_PARAMETER_ORDER + (
    "d2u_dx2",
    "d2u_dxdy",
    "d2u_dy2",
    "d2v_dx2",
    "d2v_dxdy",
    "d2v_dy2",
)
_ERROR = "motion_model must be 'affine', 'translation', or 'quadratic'"


def normalize_motion_model(value: str) -> str:
    if not isinstance(value, str) or value.strip().lower() not in MOTION_MODELS:
        raise ValueError(_ERROR)
    return value.strip().lower()


def parameter_order(motion_model: str) -> tuple[str, ...]:
    model = normalize_motion_model(motion_model)
    return QUADRATIC_PARAMETER_ORDER if model == "quadratic" else AFFINE_PARAMETER_ORDER


def parameter_count(motion_model: str) -> int:
    return len(parameter_order(motion_model))


def state_float_count(motion_model: str) -> int:
    """Floats per subset in the packed state: 8, or 16 for the quadratic model."""
    return 16 if normalize_motion_model(motion_model) == "quadratic" else 8
