"""Static ROI geometry, computed once per reference on the host.

What it computes is the reference's live_dic/roi.py: window selection
(validate_roi 29-60, integral 63-65, select_windows 74-86), the coarse
pyramid mask (reduce_mask 89-97), the segment-box link test (100-107), the
plan record (RoiPlan 110-170), UOD neighbour permissions and the 9x9 median
lattice (prepare_roi 178-263), partial-support windows (266-366) and
coarse-to-fine seed permissions (369-437).  The formats are interface and
stay the reference's: the 3x3 bit order (dy+1)*3 + dx+1, the 9x9 lattice in
four 24-bit float words, support words (row-major pixels, bit 0 of
little-endian uint32 words first), seed words (bits 0-3 corners, bit 4
selected, bits 5-31 fallback index + 1) and the mask hash
("live-dic-roi-v1\\0" + uint64le(height, width) + the mask's 0/1 bytes).

The computation is organised differently: every neighbour link of a plan is
evaluated once for all offsets of the widest stencil in use (shared by the
3x3 bits and the median lattice), through a zero-padded selection grid; the
mask reduction is a separable AND; support words are built by integer
shifts; the central component is a connected-component labelling; the
visibility sets are computed cell by cell for all end points at once; and
seed permissions are evaluated for the four corners and the 36 fallback
candidates as stacked arrays.
"""

from __future__ import annotations

import hashlib
from dataclasses import dataclass

import numpy as np

from .outlier import normalize_median_filter_size
from .subset import subset_grid_shape

# Admission limits of partial-support windows (roi.py:20-21 of the reference):
# Hessian condition on coordinates normalised by the subset size, and the
# weighted RMS contrast in grey levels.
PARTIAL_MAX_NORMALIZED_CONDITION = 1e8
PARTIAL_MIN_WEIGHTED_CONTRAST = 1.0

_HASH_PREFIX = b"live-dic-roi-v1\0"
_LATTICE = 9          # side of the median neighbour lattice
_WORD_BITS = 24       # exact integers per float32 word


def immutable(array: np.ndarray) -> np.ndarray:
    """Read-only array backed by its own bytes (no alias of the caller's)."""
    data = np.ascontiguousarray(array)
    return np.frombuffer(data.tobytes(), dtype=data.dtype).reshape(data.shape)


def validate_roi(
    mask: np.ndarray | None,
    policy: str,
    shape: tuple[int, int],
    motion_model: str,
    truncation: str = "none",
) -> np.ndarray | None:
    """Argument checks with the reference's messages; returns an owned,
    canonical (0/1 bytes) copy of the mask."""
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
    return immutable(mask.astype(np.bool_, copy=True))


def mask_digest(mask: np.ndarray) -> str:
    """SHA-256 of the hash prefix, the shape as two little-endian uint64 and
    the mask's bytes in C order (one 0/1 byte per pixel)."""
    h = hashlib.sha256(_HASH_PREFIX)
    h.update(np.asarray(mask.shape, dtype="<u8").tobytes())
    h.update(np.ascontiguousarray(mask, dtype=np.bool_).view(np.uint8).tobytes())
    return h.hexdigest()


# ---------------------------------------------------------------- counting forbidden pixels
def integral(mask: np.ndarray) -> np.ndarray:
    """Summed-area table of forbidden pixels, int64, with a zero first row
    and column: entry [y, x] counts the forbidden pixels of [0, x) x [0, y)."""
    h, w = mask.shape
    table = np.zeros((h + 1, w + 1), dtype=np.int64)
    np.cumsum(np.logical_not(mask), axis=0, dtype=np.int64, out=table[1:, 1:])
    np.cumsum(table[1:, 1:], axis=1, out=table[1:, 1:])
    return table


def boxes_clear(prefix: np.ndarray, x0, y0, x1, y1) -> np.ndarray:
    """True where the half-open box [x0, x1) x [y0, y1) has no forbidden pixel."""
    forbidden = (prefix[y1, x1] + prefix[y0, x0]) - (prefix[y0, x1] + prefix[y1, x0])
    return forbidden == 0


def select_windows(mask: np.ndarray, size: int, stride: int, *, summed_area: np.ndarray | None = None) -> np.ndarray:
    """Windows whose whole S x S footprint is allowed."""
    height, width = mask.shape
    gw, gh = subset_grid_shape(width, height, subset_size=size, subset_stride=stride)
    table = integral(mask) if summed_area is None else summed_area
    x0 = (np.arange(gw) * stride)[None, :]
    y0 = (np.arange(gh) * stride)[:, None]
    return boxes_clear(table, x0, y0, x0 + size, y0 + size)


def _segment_clear(prefix: np.ndarray, ax, ay, bx, by) -> np.ndarray:
    """The closed pixel box spanned by the segment between two pixel-centre
    points (every pixel the segment touches, corners included) holds no
    forbidden pixel.  A pixel k covers [k - 0.5, k + 0.5]."""
    h, w = prefix.shape[0] - 1, prefix.shape[1] - 1
    first_x = np.ceil(np.minimum(ax, bx) - 0.5).astype(np.int64)
    first_y = np.ceil(np.minimum(ay, by) - 0.5).astype(np.int64)
    last_x = np.floor(np.maximum(ax, bx) + 0.5).astype(np.int64)
    last_y = np.floor(np.maximum(ay, by) + 0.5).astype(np.int64)
    return boxes_clear(prefix, np.maximum(first_x, 0), np.maximum(first_y, 0),
                       np.minimum(last_x + 1, w), np.minimum(last_y + 1, h))


def reduce_mask(mask: np.ndarray) -> np.ndarray:
    """Mask of the next pyramid level: coarse pixel (x, y) is allowed when
    the 5 x 5 reduction footprint centred on (2x, 2y), reflected at the
    borders without repeating the edge, is allowed.  Evaluated as an AND
    along x, then along y."""
    h, w = mask.shape
    h2, w2 = h // 2, w // 2
    padded = np.pad(np.asarray(mask, bool), 2, mode="reflect")
    across = np.logical_and.reduce([padded[:, k: k + 2 * w2: 2] for k in range(5)])
    down = np.logical_and.reduce([across[k: k + 2 * h2: 2, :] for k in range(5)])
    return immutable(down)


# ---------------------------------------------------------------- the plan
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
        out = {
            "policy": self.policy,
            "truncation": self.truncation,
            "partial": 0 if self.partial_indices is None else int(self.partial_indices.size),
        }
        if self.policy == "partial":
            out.update(supportConditionLimit=PARTIAL_MAX_NORMALIZED_CONDITION,
                       supportContrastRmsMinimum=PARTIAL_MIN_WEIGHTED_CONTRAST, supportConnectivity=4,
                       evenCenter="all four central pixels required")
        out.update(
            maskShape=list(self.mask.shape),
            maskSha256=self.mask_hash,
            gridTotal=self.selected.size,
            selected=self.selected_count,
            excluded=self.selected.size - self.selected_count,
            hashFormat="live-dic-roi-v1\\0 + uint64le(height,width) + C-order uint8 bool",
        )
        return out

    def archive_fields(self) -> dict[str, np.ndarray]:
        fields = {"roi_mask": self.mask, "roi_selected": self.selected}
        if self.partial_indices is not None:
            fields.update(roi_partial_indices=self.partial_indices, roi_support_words=self.support_words,
                          roi_support_boxes=self.support_boxes, roi_coverage=self.coverage)
            if self.support_condition is not None:
                fields.update(roi_support_condition=self.support_condition, roi_support_rank=self.support_rank,
                              roi_support_contrast=self.support_contrast)
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


def _neighbour_links(selected: np.ndarray, prefix: np.ndarray | None, size: int, stride: int,
                     radius: int) -> dict[tuple[int, int], np.ndarray]:
    """For every offset (dx, dy) with |dx|, |dy| <= radius: both windows
    selected and, with a mask, the box around the two window centres clear."""
    gh, gw = selected.shape
    grid = np.zeros((gh + 2 * radius, gw + 2 * radius), dtype=bool)
    grid[radius: radius + gh, radius: radius + gw] = selected
    half = 0.5 * (size - 1)
    cx = (np.arange(gw) * stride + half)[None, :]
    cy = (np.arange(gh) * stride + half)[:, None]
    links = {}
    for dy in range(-radius, radius + 1):
        for dx in range(-radius, radius + 1):
            other = grid[radius + dy: radius + dy + gh, radius + dx: radius + dx + gw]
            ok = selected & other
            if prefix is not None:
                ok = ok & _segment_clear(prefix, cx, cy, cx + dx * stride, cy + dy * stride)
            links[dx, dy] = ok
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
    if policy not in ("full", "partial") or (policy == "full" and truncation != "none"):
        raise ValueError("Unknown ROI policy/truncation")
    height, width = mask.shape
    everywhere = bool(mask.all())
    prefix = None if everywhere else integral(mask)
    gw, gh = subset_grid_shape(width, height, subset_size=size, subset_stride=stride)
    if everywhere:
        selected = np.ones((gh, gw), dtype=bool)
    else:
        selected = select_windows(mask, size, stride, summed_area=prefix)
    partial = (None,) * 4
    if policy == "partial":
        selected, *partial = _partial_windows(mask, selected, size, stride, truncation=truncation)
    radius = max(1, median_filter_size // 2)
    links = _neighbour_links(selected, prefix, size, stride, radius)
    bits = np.zeros(selected.shape, dtype=np.uint32)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            bits |= links[dx, dy].astype(np.uint32) << np.uint32(3 * (dy + 1) + dx + 1)
    median_words = None
    if median_filter_size > 3:
        # the fixed 9x9 lattice (bit (dy + 4) * 9 + dx + 4), 24 bits per word,
        # whatever the median's own size
        words = np.zeros((*selected.shape, 4), dtype=np.float64)
        centre = _LATTICE // 2
        for (dx, dy), ok in links.items():
            word, bit = divmod((dy + centre) * _LATTICE + dx + centre, _WORD_BITS)
            words[..., word] += ok * float(2 ** bit)
        median_words = immutable(words.astype(np.float32).reshape(-1, 4))
    return RoiPlan(
        mask, immutable(selected), immutable(bits), mask_digest(mask), not everywhere, int(selected.sum()), policy,
        truncation, *partial, median_neighbour_words=median_words,
    )


# ---------------------------------------------------------------- partial support
def pack_support(support: np.ndarray) -> np.ndarray:
    """Pixels in row-major order; pixel i is bit i % 32 of word i // 32."""
    flat = np.asarray(support, bool).ravel()
    count = (flat.size + 31) // 32
    bits = np.zeros(count * 32, dtype=np.uint64)
    bits[: flat.size] = flat
    return (bits.reshape(count, 32) << np.arange(32, dtype=np.uint64)).sum(axis=1).astype(np.uint32)


def unpack_support(words: np.ndarray, size: int) -> np.ndarray:
    w = np.asarray(words, dtype=np.uint32).ravel()
    bits = (w[:, None] >> np.arange(32, dtype=np.uint32)) & np.uint32(1)
    return bits.ravel()[: size * size].reshape(size, size).astype(bool)


_FOUR_NEIGHBOURS = np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], dtype=bool)


def _central_component(support: np.ndarray) -> np.ndarray:
    """The 4-connected component of `support` that holds the window centre:
    the centre pixel of an odd window, or all four central pixels of an
    even one (otherwise the component is empty)."""
    from scipy import ndimage

    size = support.shape[0]
    a, b = (size - 1) // 2, size // 2
    if not support[a: b + 1, a: b + 1].all():
        return np.zeros(support.shape, dtype=bool)
    labels, _ = ndimage.label(support, structure=_FOUR_NEIGHBOURS)
    return labels == labels[a, a]


_VISIBILITY: dict[int, np.ndarray] = {}


def _visibility_paths(size: int) -> np.ndarray:
    """Boolean (pixels x cells) table: cell c lies on the closed segment from
    the window centre to the centre of pixel p, touches of a cell's edge or
    corner included.  Each cell [c - 0.5, c + 0.5]^2 is clipped against all
    segments at once (slab method: the segment's parameter interval inside
    the cell along x and along y must overlap within [0, 1])."""
    if size in _VISIBILITY:
        return _VISIBILITY[size]
    centre = 0.5 * (size - 1)
    py, px = np.indices((size, size)).reshape(2, -1).astype(np.float64)
    steps = (px - centre, py - centre)
    table = np.zeros((size * size, size * size), dtype=bool)
    for cell in range(size * size):
        cy, cx = divmod(cell, size)
        enter = np.zeros(size * size)
        leave = np.ones(size * size)
        for step, c in zip(steps, (cx, cy), strict=True):
            lo_edge, hi_edge = c - 0.5 - centre, c + 0.5 - centre
            fixed = step == 0.0
            with np.errstate(divide="ignore", invalid="ignore"):
                t0 = np.where(fixed, -np.inf, lo_edge / step)
                t1 = np.where(fixed, np.inf, hi_edge / step)
            enter = np.maximum(enter, np.minimum(t0, t1))
            leave = np.minimum(leave, np.maximum(t0, t1))
            if abs(c - centre) > 0.5:
                # a segment that does not move along this axis stays on the centre line
                leave = np.where(fixed, -1.0, leave)
        table[:, cell] = enter <= leave
    _VISIBILITY[size] = table
    return table


def _partial_windows(mask: np.ndarray, complete: np.ndarray, size: int, stride: int, *, truncation: str):
    """Windows cut by the mask whose central component survives.  Returns
    (selected, window indices, support words, support boxes (x0, y0, x1, y1),
    coverage)."""
    if truncation not in ("none", "visibility"):
        raise ValueError("roi_truncation must be 'none' or 'visibility'")
    gh, gw = complete.shape
    selected = complete.copy()
    coverage = complete.astype(np.float32)
    kept: list[tuple[int, np.ndarray]] = []
    paths = _visibility_paths(size) if truncation == "visibility" else None
    for index in np.flatnonzero(~complete):
        gy, gx = divmod(int(index), gw)
        window = mask[gy * stride: gy * stride + size, gx * stride: gx * stride + size]
        support = _central_component(window)
        if support.any() and paths is not None:
            blocked = ~support.ravel()
            visible = ~(paths & blocked[None, :]).any(axis=1)
            support = _central_component(support & visible.reshape(size, size))
        if not support.any():
            continue
        selected[gy, gx] = True
        coverage[gy, gx] = np.count_nonzero(support) / float(size * size)
        kept.append((int(index), support))
    words = (size * size + 31) // 32
    indices = np.array([i for i, _ in kept], dtype=np.uint32)
    packed = np.array([pack_support(s) for _, s in kept], dtype=np.uint32).reshape(-1, words)
    boxes = np.zeros((len(kept), 4), dtype=np.float32)
    for row, (_, s) in enumerate(kept):
        cols, rows = np.flatnonzero(s.any(axis=0)), np.flatnonzero(s.any(axis=1))
        boxes[row] = (cols[0], rows[0], cols[-1], rows[-1])
    return selected, immutable(indices), immutable(packed), immutable(boxes), immutable(coverage)


# ---------------------------------------------------------------- seed permissions
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
    a fallback source subset (0 = none) used when no corner is admissible.

    Source corners follow the seed transfer's edge-anchored layout (window
    centre at S/2 + k*step, half a coarse pixel of phase between the scales).
    A corner, or a fallback candidate, is admissible when it is selected and
    the reference-resolution box around the segment between the two window
    centres ((S - 1)/2 + k*step, times each scale) is clear.  The fallback
    (coarse-to-fine transfers only) is the nearest admissible source among
    the 6 x 6 subsets around the lower corner; equal distances keep the
    first in row-major (dy, dx) order."""
    dsel = np.asarray(destination.selected, bool)
    ssel = np.asarray(source.selected, bool)
    sh, sw = ssel.shape
    gy, gx = np.indices(dsel.shape)
    edge = 0.5 * size
    mid = 0.5 * (size - 1)
    phase = 0.5 * (source_scale - destination_scale)
    # destination window centre in source-level edge coordinates
    sx = (destination_scale * (edge + gx * stride) + phase) / source_scale
    sy = (destination_scale * (edge + gy * stride) + phase) / source_scale
    low_x = np.clip(np.floor((sx - edge) / stride), 0, max(0, sw - 2)).astype(np.int64)
    low_y = np.clip(np.floor((sy - edge) / stride), 0, max(0, sh - 2)).astype(np.int64)
    prefix = integral(reference_mask) if reference_prefix is None else reference_prefix
    ax, ay = destination_scale * (mid + gx * stride), destination_scale * (mid + gy * stride)

    def admissible(nx, ny, ax, ay):
        inside = (nx >= 0) & (ny >= 0) & (nx < sw) & (ny < sh)
        cx, cy = np.clip(nx, 0, sw - 1), np.clip(ny, 0, sh - 1)
        ok = inside & ssel[cy, cx]
        ok &= _segment_clear(prefix, ax, ay, source_scale * (mid + cx * stride), source_scale * (mid + cy * stride))
        return ok, cx, cy

    corner_x = low_x[None] + np.array([0, 1, 0, 1])[:, None, None]
    corner_y = low_y[None] + np.array([0, 0, 1, 1])[:, None, None]
    corners, _, _ = admissible(corner_x, corner_y, ax[None], ay[None])
    corners &= dsel[None]
    words = dsel.astype(np.uint32) << np.uint32(4)
    for k in range(4):
        words |= corners[k].astype(np.uint32) << np.uint32(k)
    if source_scale > destination_scale and ssel.size < (1 << 27) - 1:
        my, mx = np.nonzero(dsel & ((words & 15) == 0))
        if my.size:
            off_y, off_x = np.divmod(np.arange(36), 6)
            nx = low_x[my, mx][None, :] + (off_x - 2)[:, None]
            ny = low_y[my, mx][None, :] + (off_y - 2)[:, None]
            ok, cx, cy = admissible(nx, ny, ax[my, mx][None, :], ay[my, mx][None, :])
            dist = (sx[my, mx][None, :] - (edge + cx * stride)) ** 2 + (sy[my, mx][None, :] - (edge + cy * stride)) ** 2
            dist = np.where(ok, dist, np.inf)
            best = np.argmin(dist, axis=0)
            pick = np.arange(my.size)
            found = np.isfinite(dist[best, pick])
            fallback = np.where(found, cy[best, pick] * sw + cx[best, pick] + 1, 0).astype(np.uint32)
            words[my, mx] |= fallback << np.uint32(5)
    return immutable(words)
