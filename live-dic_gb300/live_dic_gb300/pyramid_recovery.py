"""Host logic of the single-scale engine's selective pyramid recovery.

Restates the reference's host-side helpers (wgpu_backend.py):

* ``reduce_half`` (318-334): five-tap [1 4 6 4 1]/16 reduction along x then
  y with reflect padding, every second sample, truncation to uint8.  The
  reference evaluates it in float32; every partial sum there is a multiple of
  1/256 below 256 and therefore exact, so the integer form below (sum of the
  5x5 integer weights, floor division by 256) gives identical bytes.
* ``transfer_pyramid_seed`` (337-454): bilinear blend of the four coarse
  warps around each requested finer subset centre, Taylor-recentred, with
  translation x (source/destination scale) and curvature x the inverse, in
  float64; the ROI fallback neighbour (permissions >> 5).
* ``pyramid_dependency_mask`` (456-503): the four-source closure of the
  requested subsets on the next coarser grid.

Only failed fine subsets go through the coarse levels, so these run on the
host as in the reference; the solves themselves are the GPU engines'.
"""

from __future__ import annotations

import numpy as np

from .motion import parameter_count, state_float_count

_TAPS = np.array((1, 4, 6, 4, 1), dtype=np.int64)


def reduce_half(image: np.ndarray) -> np.ndarray:
    """Half-resolution level of a uint8 image (floor of each dimension)."""
    source = np.asarray(image, dtype=np.int64)
    height, width = source.shape
    rh, rw = height // 2, width // 2
    padded_x = np.pad(source, ((0, 0), (2, 2)), mode="reflect")
    horizontal = sum(_TAPS[i] * padded_x[:, i: i + 2 * rw: 2] for i in range(5))
    padded_y = np.pad(horizontal, ((2, 2), (0, 0)), mode="reflect")
    total = sum(_TAPS[i] * padded_y[i: i + 2 * rh: 2] for i in range(5))
    return np.ascontiguousarray(np.clip(total // 256, 0, 255).astype(np.uint8))


def _fine_to_coarse(index, *, source_scale, destination_scale, subset_size, subset_stride):
    centre = 0.5 * subset_size
    offset = (1.0 - destination_scale) * 0.5 - (1.0 - source_scale) * 0.5
    return (destination_scale * (centre + subset_stride * index) + offset) / source_scale


def pyramid_dependency_mask(*, source_grid, source_scale, destination_scale, requested, subset_size,
                            subset_stride) -> np.ndarray:
    source_width, source_height = source_grid
    mask = np.zeros((source_height, source_width), dtype=np.bool_)
    destinations = np.argwhere(requested)
    if destinations.size == 0 or source_width < 2 or source_height < 2:
        return mask
    kw = dict(source_scale=source_scale, destination_scale=destination_scale, subset_size=subset_size,
              subset_stride=subset_stride)
    x = _fine_to_coarse(destinations[:, 1], **kw)
    y = _fine_to_coarse(destinations[:, 0], **kw)
    centre = 0.5 * subset_size
    lower_x = np.clip(np.floor((x - centre) / subset_stride), 0, source_width - 2).astype(np.intp)
    lower_y = np.clip(np.floor((y - centre) / subset_stride), 0, source_height - 2).astype(np.intp)
    for corner in range(4):
        mask[lower_y + (corner >> 1), lower_x + (corner & 1)] = True
    return mask


def transfer_pyramid_seed(parameters: np.ndarray, status: np.ndarray, *, motion_model: str,
                          source_available: np.ndarray, source_scale: int, destination_scale: int,
                          destination_grid, requested: np.ndarray, subset_size: int, subset_stride: int,
                          permissions: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    """(seed states (gh, gw, 8|16) float32, activity uint32) for `requested`."""
    destination_width, destination_height = destination_grid
    n = parameter_count(motion_model)
    seeds = np.zeros((destination_height, destination_width, state_float_count(motion_model)), np.float32)
    active = requested.astype(np.uint32, copy=True)
    source_height, source_width = status.shape
    if source_width < 2 or source_height < 2:
        return seeds, active
    destinations = np.argwhere(requested)
    if destinations.size == 0:
        return seeds, active
    dy_idx, dx_idx = destinations[:, 0], destinations[:, 1]
    kw = dict(source_scale=source_scale, destination_scale=destination_scale, subset_size=subset_size,
              subset_stride=subset_stride)
    x = _fine_to_coarse(dx_idx, **kw)
    y = _fine_to_coarse(dy_idx, **kw)
    centre = 0.5 * subset_size
    grid_x, grid_y = (x - centre) / subset_stride, (y - centre) / subset_stride
    lower_x = np.clip(np.floor(grid_x), 0, source_width - 2).astype(np.intp)
    lower_y = np.clip(np.floor(grid_y), 0, source_height - 2).astype(np.intp)
    frac_x = np.clip(grid_x - lower_x, 0.0, 1.0)
    frac_y = np.clip(grid_y - lower_y, 0.0, 1.0)
    translation_scale = source_scale / destination_scale
    curvature_scale = destination_scale / source_scale
    accumulated = np.zeros((destinations.shape[0], n), np.float64)
    weight_sum = np.zeros(destinations.shape[0], np.float64)
    for corner in range(5):
        if corner == 4:
            if permissions is None:
                break
            fallback = permissions[dy_idx, dx_idx] >> np.uint32(5)
            index = np.maximum(fallback.astype(np.int64) - 1, 0)
            sx, sy = index % source_width, index // source_width
            valid = (fallback != 0) & (weight_sum == 0) & source_available[sy, sx] & (status[sy, sx] >= 0.5)
            weight = valid.astype(np.float64)
        else:
            sx, sy = lower_x + (corner & 1), lower_y + (corner >> 1)
            valid = (status[sy, sx] >= -0.5) & source_available[sy, sx]
            if permissions is not None:
                valid &= (permissions[dy_idx, dx_idx] & (1 << corner)) != 0
            wx = frac_x if corner & 1 else 1.0 - frac_x
            wy = frac_y if corner & 2 else 1.0 - frac_y
            weight = wx * wy * valid
        p = parameters[sy, sx]
        ddx = x - (centre + subset_stride * sx)
        ddy = y - (centre + subset_stride * sy)
        t = np.array(p, dtype=np.float64, copy=True)
        if motion_model == "quadratic":
            dx2, dxy, dy2 = ddx * ddx, ddx * ddy, ddy * ddy
            t[:, 0] += p[:, 1] * ddx + p[:, 2] * ddy + 0.5 * p[:, 6] * dx2 + p[:, 7] * dxy + 0.5 * p[:, 8] * dy2
            t[:, 3] += p[:, 4] * ddx + p[:, 5] * ddy + 0.5 * p[:, 9] * dx2 + p[:, 10] * dxy + 0.5 * p[:, 11] * dy2
            t[:, 1] += p[:, 6] * ddx + p[:, 7] * ddy
            t[:, 2] += p[:, 7] * ddx + p[:, 8] * ddy
            t[:, 4] += p[:, 9] * ddx + p[:, 10] * ddy
            t[:, 5] += p[:, 10] * ddx + p[:, 11] * ddy
            t[:, 6:12] *= curvature_scale
        else:
            t[:, 0] += p[:, 1] * ddx + p[:, 2] * ddy
            t[:, 3] += p[:, 4] * ddx + p[:, 5] * ddy
        t[:, (0, 3)] *= translation_scale
        accumulated += weight[:, None] * t
        weight_sum += weight
    ok = weight_sum > 0.0
    seeds[dy_idx[ok], dx_idx[ok], :n] = accumulated[ok] / weight_sum[ok, None]
    return seeds, active
