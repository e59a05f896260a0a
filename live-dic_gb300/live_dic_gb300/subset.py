"""Square subset grid validation (reference: live_dic/subset.py:7-65)."""

from __future__ import annotations

import operator

DEFAULT_SUBSET_SIZE = 16
MIN_SUBSET_SIZE = 4
MAX_SUBSET_SIZE = 46_340


def normalize_subset_size(value: int) -> int:
    message = f"subset_size must be an integer from {MIN_SUBSET_SIZE} to {MAX_SUBSET_SIZE}"
    try:
        size = operator.index(value)
    except TypeError as error:
        raise ValueError(message) from error
    if isinstance(value, bool) or not MIN_SUBSET_SIZE <= size <= MAX_SUBSET_SIZE:
        raise ValueError(message)
    return size


def normalize_subset_stride(value: int | None, *, subset_size: int) -> int:
    if value is None:
        return subset_size
    try:
        stride = operator.index(value)
    except TypeError as error:
        raise ValueError("subset_stride must be a positive integer") from error
    if isinstance(value, bool) or not 1 <= stride <= subset_size:
        raise ValueError("subset_stride must be between 1 and subset_size")
    return stride


def subset_grid_shape(width: int, height: int, *, subset_size: int, subset_stride: int) -> tuple[int, int]:
    """(grid_width, grid_height) of fully contained windows."""
    if width < subset_size or height < subset_size:
        return (0, 0)
    return (1 + (width - subset_size) // subset_stride, 1 + (height - subset_size) // subset_stride)
