"""Static ROI geometry, computed once per reference on the host.

Restates the reference's live_dic/roi.py (validate_roi 29-60, integral 63,
select_windows 74-86, reduce_mask 89-97, _links_clear 100-107, RoiPlan
110-170, prepare_roi 178-263, seed_permissions 358-437): full-window
selection through a summed-area table of forbidden pixels, 3x3 (or 9x9)
neighbour-permission bits for UOD, and coarse-to-fine seed permissions.
The mask layout, bit layouts and hash format are the reference's, so plans
and archives are interchangeable.
"""

from __future__ import annotations

import hashlib
import struct
from dataclasses import dataclass

import numpy as np

from .outlier import normalize_median_filter_size
from .subset import subset_grid_shape

# Admission limits of partial-support windows (roi.py:20-21 of the reference):
# Hessian condition on coordinates normalised by the subset size, and the
# weighted RMS contrast in grey levels.
PARTIAL_MAX_NORMALIZED_CONDITION = 1e8
PARTIAL_MIN_WEIGHTED_CONTRAST = 1.0


def immutable(array: np.ndarray) -> np.ndarray:
    """Read-only copy that owns its bytes."""
    return np.frombuffer(array.tobytes(order="C"), dtype=array.dtype).reshape(array.shape)


def validate_roi(
    mask: np.ndarray | None,
    policy: str,
    shape: tuple[int, int],
    motion_model: str,
    truncation: str = "none",
) -> np.ndarray | None:
    if not isinstance(policy, str) or policy not in ("full", "partial"):
        raise ValueError("roi_policy must be 'full' or 'partial'")
    if not isinstance(truncation, str) or truncation not in ("none", "visibility"):
        raise ValueError("roi_truncation must be 'none' or 'visibility'")
    if truncation != "none" and (policy != "partial" or mask is None):
        raise ValueError("roi_truncation requires roi_policy='partial' and a mask")
    if mask is None:
        return None
    if motion_model not in ("translation", "affine"):
        raise ValueError("ROI supports only translation and affine motion models")
    if not isinstance(mask, np.ndarray) or mask.dtype != np.bool_:
        raise TypeError("roi_mask must be a two-dimensional boolean NumPy array")
    if mask.ndim != 2 or mask.shape != shape:
        raise ValueError(f"roi_mask must have reference shape {shape}")
    return immutable(np.logical_and(mask, True))


def integral(mask: np.ndarray) -> np.ndarray:
    """Exclusive 2-D prefix sum of forbidden pixels (int64), padded by one."""
    forbidden = (~mask).astype(np.int64)
    out = np.zeros((mask.shape[0] + 1, mask.shape[1] + 1), dtype=np.int64)
    out[1:, 1:] = forbidden.cumsum(axis=0).cumsum(axis=1)
    return out


def boxes_clear(prefix: np.ndarray, x0, y0, x1, y1) -> np.ndarray:
    """True where the half-open pixel box [x0, x1) x [y0, y1) holds no forbidden pixel."""
    return prefix[y1, x1] - prefix[y0, x1] - prefix[y1, x0] + prefix[y0, x0] == 0


def select_windows(mask: np.ndarray, size: int, stride: int, *, summed_area: np.ndarray | None = None) -> np.ndarray:
    height, width = mask.shape
    gw, gh = subset_grid_shape(width, height, subset_size=size, subset_stride=stride)
    ys, xs = np.meshgrid(np.arange(gh) * stride, np.arange(gw) * stride, indexing="ij")
    prefix = integral(mask) if summed_area is None else summed_area
    return boxes_clear(prefix, xs, ys, xs + size, ys + size)


def _reflect(n: int, pad: int) -> np.ndarray:
    idx = np.arange(-pad, n + pad)
    idx = np.where(idx < 0, -idx, idx)
    return np.where(idx >= n, 2 * n - 2 - idx, idx)


def reduce_mask(mask: np.ndarray) -> np.ndarray:
    """A coarse pixel is allowed only if all 25 reflected source pixels of the
    5x5 reduction footprint centred on (2x, 2y) are allowed."""
    h, w = mask.shape
    h2, w2 = h // 2, w // 2
    padded = mask[_reflect(h, 2)][:, _reflect(w, 2)]
    out = np.ones((h2, w2), dtype=bool)
    for dy in range(5):
        for dx in range(5):
            out &= padded[dy : dy + 2 * h2 : 2, dx : dx + 2 * w2 : 2]
    return immutable(out)


def _links_clear(prefix: np.ndarray, ax, ay, bx, by) -> np.ndarray:
    """Closed pixel box around the segment a-b is free of forbidden pixels."""
    h, w = np.array(prefix.shape) - 1
    x0 = np.maximum(0, np.ceil(np.minimum(ax, bx) - 0.5).astype(int))
    y0 = np.maximum(0, np.ceil(np.minimum(ay, by) - 0.5).astype(int))
    x1 = np.minimum(w, np.floor(np.maximum(ax, bx) + 0.5).astype(int) + 1)
    y1 = np.minimum(h, np.floor(np.maximum(ay, by) + 0.5).astype(int) + 1)
    return boxes_clear(prefix, x0, y0, x1, y1)


@dataclass(frozen=True, slots=True)
class RoiPlan:
    """Immutable ROI arrays shared by a reference and all its results."""

    mask: np.ndarray
    selected: np.ndarray
    neighbour_bits: np.ndarray
    mask_hash: str
    effective: bool
    selected_count: int
    policy: str = "full"
    truncation: str = "none"
    partial_indices: np.ndarray | None = None
    support_words: np.ndarray | None = None
    support_boxes: np.ndarray | None = None
    coverage: np.ndarray | None = None
    support_condition: np.ndarray | None = None
    support_rank: np.ndarray | None = None
    support_contrast: np.ndarray | None = None
    median_neighbour_words: np.ndarray | None = None

    @property
    def empty(self) -> bool:
        return self.selected_count == 0

    def summary(self) -> dict:
        return {
            "policy": self.policy,
            "truncation": self.truncation,
            "partial": 0 if self.partial_indices is None else int(self.partial_indices.size),
            "maskShape": list(self.mask.shape),
            "maskSha256": self.mask_hash,
            "gridTotal": self.selected.size,
            "selected": self.selected_count,
            "excluded": self.selected.size - self.selected_count,
            "hashFormat": "live-dic-roi-v1\\0 + uint64le(height,width) + C-order uint8 bool",
        }

    def archive_fields(self) -> dict[str, np.ndarray]:
        fields = {"roi_mask": self.mask, "roi_selected": self.selected}
        if self.partial_indices is not None:
            fields.update(
                roi_partial_indices=self.partial_indices,
                roi_support_words=self.support_words,
                roi_support_boxes=self.support_boxes,
                roi_coverage=self.coverage,
            )
        return fields

    def links_table(self, median_filter_size: int, outlier_policy: str) -> np.ndarray:
        """Per-subset float4 UOD permission words (3x3 bits in word 0, or the
        9x9 lattice in four 24-bit words for a wider median)."""
        links = np.zeros((self.selected.size, 4), dtype=np.float32)
        if outlier_policy == "median" and median_filter_size > 3 and self.median_neighbour_words is not None:
            links[:] = self.median_neighbour_words
        else:
            links[:, 0] = self.neighbour_bits.ravel()
        return links


def prepare_roi(
    mask: np.ndarray | None,
    size: int,
    stride: int,
    *,
    policy: str = "full",
    truncation: str = "none",
    median_filter_size: int = 3,
) -> RoiPlan | None:
    median_filter_size = normalize_median_filter_size(median_filter_size)
    if mask is None:
        return None
    height, width = mask.shape
    all_allowed = bool(mask.all())
    prefix = None if all_allowed else integral(mask)
    gw, gh = subset_grid_shape(width, height, subset_size=size, subset_stride=stride)
    selected = np.ones((gh, gw), dtype=bool) if all_allowed else select_windows(mask, size, stride, summed_area=prefix)
    partial_indices = support_words = support_boxes = coverage = None
    if policy == "partial":
        selected, partial_indices, support_words, support_boxes, coverage = _partial_windows(
            mask, selected, size, stride, truncation=truncation)
    elif policy != "full" or truncation != "none":
        raise ValueError("Unknown ROI policy/truncation")
    y, x = np.indices(selected.shape)
    ax = x * stride + (size - 1) / 2
    ay = y * stride + (size - 1) / 2

    def allowed_offset(dx: int, dy: int) -> np.ndarray:
        nx, ny = x + dx, y + dy
        inside = (nx >= 0) & (ny >= 0) & (nx < selected.shape[1]) & (ny < selected.shape[0])
        ok = inside & selected & selected[ny.clip(0, selected.shape[0] - 1), nx.clip(0, selected.shape[1] - 1)]
        if prefix is not None:
            ok &= _links_clear(prefix, ax, ay, ax + dx * stride, ay + dy * stride)
        return ok

    bits = np.zeros(selected.shape, dtype=np.uint32)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            bits |= allowed_offset(dx, dy).astype(np.uint32) << np.uint32((dy + 1) * 3 + dx + 1)
    median_words = None
    if median_filter_size > 3:
        radius = median_filter_size // 2
        words = np.zeros((*selected.shape, 4), dtype=np.float32)
        for dy in range(-radius, radius + 1):
            for dx in range(-radius, radius + 1):
                bit = (dy + 4) * 9 + dx + 4
                words[..., bit // 24] += allowed_offset(dx, dy).astype(np.float32) * float(1 << (bit % 24))
        median_words = immutable(words.reshape(-1, 4))
    digest = hashlib.sha256(b"live-dic-roi-v1\0" + struct.pack("<QQ", *mask.shape) + mask.tobytes(order="C")).hexdigest()
    return RoiPlan(
        mask,
        immutable(selected),
        immutable(bits),
        digest,
        not all_allowed,
        int(selected.sum()),
        policy,
        truncation,
        partial_indices,
        support_words,
        support_boxes,
        coverage,
        median_neighbour_words=median_words,
    )


# ---------------------------------------------------------------- partial support
def pack_support(support: np.ndarray) -> np.ndarray:
    """Row-major pixel bits, bit 0 of little-endian uint32 words first
    (roi.py:266-270)."""
    bits = np.packbits(np.asarray(support, bool).ravel(), bitorder="little")
    bits = np.pad(bits, (0, (-bits.size) % 4))
    return bits.view("<u4").astype(np.uint32, copy=False)


def unpack_support(words: np.ndarray, size: int) -> np.ndarray:
    raw = np.asarray(words, dtype="<u4").view(np.uint8)
    return np.unpackbits(raw, bitorder="little")[: size * size].reshape(size, size).astype(bool)


def _central_component(support: np.ndarray) -> np.ndarray:
    """Pixels 4-connected to the window centre (roi.py:279-300); an even
    window needs all four central pixels allowed."""
    size = support.shape[0]
    lo, hi = (size - 1) // 2, size // 2
    out = np.zeros_like(support, dtype=bool)
    if not support[lo: hi + 1, lo: hi + 1].all():
        return out
    stack = [(lo, lo)]
    out[lo, lo] = True
    while stack:
        y, x = stack.pop()
        for ny, nx in ((y - 1, x), (y + 1, x), (y, x - 1), (y, x + 1)):
            if 0 <= ny < size and 0 <= nx < size and support[ny, nx] and not out[ny, nx]:
                out[ny, nx] = True
                stack.append((ny, nx))
    return out


_VISIBILITY: dict[int, np.ndarray] = {}


def _visibility_paths(size: int) -> np.ndarray:
    """For every pixel, the packed set of pixel cells touched by the segment
    from the window centre to it (roi.py:303-327): slab intersection of the
    segment with each closed unit cell, boundary touches included."""
    if size in _VISIBILITY:
        return _VISIBILITY[size]
    y, x = np.indices((size, size)).reshape(2, -1).astype(np.float64)
    centre = (size - 1) / 2
    lower = np.zeros((size * size, size * size))
    upper = np.ones_like(lower)
    for coord in (x, y):
        delta = coord - centre
        moving = delta != 0
        a = np.full_like(lower, -np.inf)
        b = np.full_like(upper, np.inf)
        a[moving] = (coord[None, :] - 0.5 - centre) / delta[moving, None]
        b[moving] = (coord[None, :] + 0.5 - centre) / delta[moving, None]
        lower = np.maximum(lower, np.minimum(a, b))
        upper = np.minimum(upper, np.maximum(a, b))
        upper[np.ix_(~moving, np.abs(coord - centre) > 0.5)] = -1
    paths = immutable(np.stack([pack_support(row) for row in lower <= upper]))
    _VISIBILITY[size] = paths
    return paths


def _partial_windows(mask: np.ndarray, complete: np.ndarray, size: int, stride: int, *, truncation: str):
    """Windows cut by the ROI whose central component survives
    (roi.py:330-366): (selected, indices, support words, boxes, coverage)."""
    if truncation not in ("none", "visibility"):
        raise ValueError("roi_truncation must be 'none' or 'visibility'")
    selected = complete.copy()
    indices, words, boxes = [], [], []
    coverage = complete.astype(np.float32)
    for gy, gx in np.argwhere(~complete):
        local = mask[gy * stride: gy * stride + size, gx * stride: gx * stride + size]
        support = _central_component(local)
        if not support.any():
            continue
        if truncation == "visibility":
            visible = ~np.any(_visibility_paths(size) & ~pack_support(support), axis=1)
            support = _central_component(support & visible.reshape(size, size))
            if not support.any():
                continue
        selected[gy, gx] = True
        indices.append(gy * complete.shape[1] + gx)
        words.append(pack_support(support))
        sy, sx = np.nonzero(support)
        boxes.append((sx.min(), sy.min(), sx.max(), sy.max()))
        coverage[gy, gx] = support.sum() / (size * size)
    count = (size * size + 31) // 32
    return (selected, immutable(np.asarray(indices, np.uint32)),
            immutable(np.asarray(words, np.uint32).reshape(-1, count)),
            immutable(np.asarray(boxes, np.float32).reshape(-1, 4)), immutable(coverage))


def seed_permissions(
    source: RoiPlan,
    destination: RoiPlan,
    *,
    source_scale: int,
    destination_scale: int,
    size: int,
    stride: int,
    reference_mask: np.ndarray,
    reference_prefix: np.ndarray | None = None,
) -> np.ndarray:
    """Per destination subset: bits 0-3 allow the four bilinear source corners,
    bit 4 marks a selected destination, bits 5-31 hold 1 + the linear index of
    a fallback source subset (0 = none) used when no corner is admissible."""
    y, x = np.indices(destination.selected.shape)
    centre = size / 2
    sh, sw = source.selected.shape
    sx = (destination_scale * (centre + x * stride) + (source_scale - destination_scale) / 2) / source_scale
    sy = (destination_scale * (centre + y * stride) + (source_scale - destination_scale) / 2) / source_scale
    lower_x = np.clip(np.floor((sx - centre) / stride), 0, max(0, sw - 2)).astype(int)
    lower_y = np.clip(np.floor((sy - centre) / stride), 0, max(0, sh - 2)).astype(int)
    bits = destination.selected.astype(np.uint32) << np.uint32(4)
    prefix = reference_prefix if reference_prefix is not None else integral(reference_mask)
    half = (size - 1) / 2
    for corner in range(4):
        nx = lower_x + (corner & 1)
        ny = lower_y + (corner >> 1)
        inside = (nx < sw) & (ny < sh)
        nx = nx.clip(0, sw - 1)
        ny = ny.clip(0, sh - 1)
        ok = inside & source.selected[ny, nx] & destination.selected
        ok &= _links_clear(
            prefix,
            destination_scale * (half + x * stride),
            destination_scale * (half + y * stride),
            source_scale * (half + nx * stride),
            source_scale * (half + ny * stride),
        )
        bits |= ok.astype(np.uint32) << np.uint32(corner)
    if source_scale > destination_scale and source.selected.size < (1 << 27) - 1:
        my, mx = np.nonzero(destination.selected & ((bits & 15) == 0))
        best = np.full(mx.shape, np.inf)
        chosen = np.zeros(mx.shape, dtype=np.uint32)
        for dy in range(-2, 4):
            for dx in range(-2, 4):
                nx = lower_x[my, mx] + dx
                ny = lower_y[my, mx] + dy
                inside = (nx >= 0) & (ny >= 0) & (nx < sw) & (ny < sh)
                cx = nx.clip(0, sw - 1)
                cy = ny.clip(0, sh - 1)
                distance = (sx[my, mx] - (centre + cx * stride)) ** 2 + (sy[my, mx] - (centre + cy * stride)) ** 2
                ok = inside & source.selected[cy, cx] & (distance < best)
                ok &= _links_clear(
                    prefix,
                    destination_scale * (half + mx * stride),
                    destination_scale * (half + my * stride),
                    source_scale * (half + cx * stride),
                    source_scale * (half + cy * stride),
                )
                best[ok] = distance[ok]
                chosen[ok] = (cy[ok] * sw + cx[ok] + 1).astype(np.uint32)
        bits[my, mx] |= chosen << np.uint32(5)
    return immutable(bits)
