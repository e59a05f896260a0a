"""Target reconstruction modes (reference: live_dic/interpolation.py:5-27).

``bspline`` samples Gaussian-smoothed cubic B-spline coefficients; ``linear``
(bilinear) and ``cubic`` (Keys, a = -0.5) interpolate the raw bytes."""

from __future__ import annotations

INTERPOLATION_MODES = ("bspline", "linear", "cubic")
INTERPOLATION_CODES = {"bspline": 0, "linear": 1, "cubic": 2}


def normalize_interpolation(value: str) -> str:
    if not isinstance(value, str) or value.strip().lower() not in INTERPOLATION_MODES:
        raise ValueError("interpolation must be 'bspline', 'linear', or 'cubic'")
    return value.strip().lower()
