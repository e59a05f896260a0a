"""Displacement outlier policy (reference: live_dic/outlier.py:8-55)."""

from __future__ import annotations

import operator

OUTLIER_POLICIES = ("replace", "flag", "disabled", "median")
OUTLIER_POLICY_CODES = {"flag": 0, "replace": 1, "disabled": 2, "median": 3}
MEDIAN_FILTER_SIZES = (3, 5, 7, 9)
MEDIAN_FILTER_SCOPES = ("rejected", "all")
MEDIAN_FILTER_SCOPE_CODES = {"rejected": 0, "all": 1}


def normalize_outlier_policy(value: str) -> str:
    if not isinstance(value, str) or value.strip().lower() not in OUTLIER_POLICIES:
        raise ValueError("outlier_policy must be 'replace', 'flag', 'disabled', or 'median'")
    return value.strip().lower()


def normalize_median_filter_size(value: int) -> int:
    message = "median_filter_size must be one of 3, 5, 7, or 9 subsets"
    try:
        size = operator.index(value)
    except TypeError as error:
        raise ValueError(message) from error
    if isinstance(value, bool) or size not in MEDIAN_FILTER_SIZES:
        raise ValueError(message)
    return size


def normalize_median_filter_scope(value: str) -> str:
    if not isinstance(value, str) or value.strip().lower() not in MEDIAN_FILTER_SCOPES:
        raise ValueError("median_filter_scope must be 'rejected' or 'all'")
    return value.strip().lower()
