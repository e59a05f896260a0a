"""Spatial integration weights (reference: live_dic/weighting.py:7-32)."""

from __future__ import annotations

import math

SPATIAL_WEIGHTING_CODES = {"uniform": 0, "gaussian": 1}


def normalize_spatial_weighting(value: str) -> str:
    weighting = str(value).strip().lower()
    if weighting not in SPATIAL_WEIGHTING_CODES:
        raise ValueError("spatial_weighting must be 'uniform' or 'gaussian'")
    return weighting


def normalize_gaussian_sigma(value: float | None, *, subset_size: int) -> float:
    """Sigma in pixels; defaults to a quarter of the subset width."""
    sigma = 0.25 * subset_size if value is None else float(value)
    if not math.isfinite(sigma) or sigma <= 0.0:
        raise ValueError("gaussian_sigma must be finite and greater than zero")
    return sigma
