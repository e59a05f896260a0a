"""CPU oracle of one full-pyramid frame (TEST INFRASTRUCTURE ONLY).

Composes the C oracle's restatements in the order of the reference's
ICGNWGPUFullPyramid._encode_slot (full_pyramid_backend.py:1436-1569):
integer reductions, temporal velocity prediction and projection onto the
coarsest active grid (full_pyramid.wgsl:83-122,437-450), the coarsest seeded
solve and UOD, coarse-to-fine transfer (251-435) with the temporal fine
correction on the finest grid (452-506), finer solves and UOD, then the
history updates (126-148, 508-554) including the coarse history of the fine
correction.  The per-level reference arrays are taken as given (the GPU
engine's exported plane / metadata / inverse), so a comparison covers the
per-frame path bit for bit.  Counters: [projected, accepted updates,
velocity-predicted, expired (adaptive policy only)].

ROI (`rois`, one LevelRoi per level, plus `temporal_links`): the solver's
status -3 propagation, the UOD neighbour permissions, the coarse-to-fine and
temporal seed permissions (bits 0-3 corners, bit 4 selected, bits 5-31 the
fallback source; full_pyramid.wgsl:397-450).  `search_radius` > 0: the
integer ZNCC search at the coarsest level (every subset, or with temporal
seeding only those the projection left without a seed, whose status the
projection marks -1), on `reference_levels[-1]`.  `global_shift`: the
Fourier initialization, whose uniform coarsest seed (dx, dy) / 2^(levels-1)
for every selected subset (full_pyramid_backend.py:1704-1714) takes the
frame's estimate `register(frame, shift=(dx, dy))`, followed with a search
radius by the search centred on it.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import oracle as oc
from . import reference_prep as rp


@dataclass
class LevelRoi:
    selected: np.ndarray            # uint8 per subset
    links: np.ndarray               # float32 (count, 4): UOD neighbour permissions
    seed_links: np.ndarray | None   # uint32 per subset: transfer from the next coarser level


@dataclass
class LevelArrays:
    width: int
    height: int
    grid_w: int
    grid_h: int
    plane: np.ndarray
    metadata: np.ndarray
    inverse: np.ndarray


class PyramidOracle:
    def __init__(self, levels: list[LevelArrays], *, subset_size: int, subset_stride: int,
                 iterations: tuple[int, ...], tolerances: tuple[float, ...], zncc_min: float = 0.8,
                 model: str = "affine", interpolation: str = "bspline", lanes: int = 32,
                 outlier_policy: str = "replace", median_size: int = 3, temporal: bool = False,
                 velocity: bool = False, fine_correction: bool = False, adaptive: bool = False,
                 max_age: int = 0xFFFFFFFE, divergence_patience: int = 0, divergence_min_iterations: int = 4,
                 rois: list[LevelRoi] | None = None, temporal_links: np.ndarray | None = None,
                 search_radius: int = 0, reference_levels: list[np.ndarray] | None = None,
                 global_shift: bool = False):
        self.levels = levels
        self.rois, self.temporal_links = rois, temporal_links
        self.search_radius, self.reference_levels = search_radius, reference_levels
        self.global_shift = global_shift
        if search_radius and reference_levels is None:
            raise ValueError("the seed search needs the reference image of every level")
        self.L = len(levels)
        self.S, self.s = subset_size, subset_stride
        self.iterations, self.tolerances, self.zncc_min = iterations, tolerances, zncc_min
        self.model, self.interp, self.lanes = model, interpolation, lanes
        self.policy, self.median_size = outlier_policy, median_size
        self.temporal, self.velocity = temporal, velocity
        self.fine_correction, self.adaptive = fine_correction, adaptive
        self.max_age = max_age
        self.patience, self.min_iterations = divergence_patience, divergence_min_iterations
        self.ss = 16 if model == "quadratic" else 8
        self.status_at = 12 if model == "quadratic" else 6
        self.taps = rp.runtime_fir_taps()
        self.reset()

    def _empty_history(self, count: int) -> tuple[np.ndarray, np.ndarray]:
        state = np.zeros((count, self.ss), np.float32)
        state[:, self.status_at] = -1.0
        return state, np.full(count, 0xFFFFFFFF, np.uint32)

    def reset(self) -> None:
        fine = self.levels[0].grid_w * self.levels[0].grid_h
        self.history, self.ages = self._empty_history(fine)
        self.prev_history, self.prev_ages = self._empty_history(fine)
        top = self.levels[-1]
        self.coarse_history, self.coarse_ages = self._empty_history(top.grid_w * top.grid_h)

    def _grid(self, level: int) -> tuple[int, int]:
        return self.levels[level].grid_w, self.levels[level].grid_h

    def _solve_level(self, level: int, frame: np.ndarray, seed, active) -> tuple[np.ndarray, np.ndarray]:
        lv = self.levels[level]
        coef = oc.prefilter(frame, self.taps) if self.interp == "bspline" else None
        schedule = self.L - 1 - level
        raw = oc.solve(frame, coef, lv.plane, lv.metadata, lv.inverse, subset_size=self.S, subset_stride=self.s,
                       model=self.model, interpolation=self.interp, lanes=self.lanes,
                       iterations=self.iterations[schedule], tolerance=self.tolerances[schedule],
                       zncc_min=self.zncc_min, seed_state=seed, active=active,
                       divergence_patience=self.patience if level == 0 else 0,
                       divergence_min_iterations=self.min_iterations, roi_enabled=self.rois is not None)
        if self.policy == "disabled":
            return raw, raw
        out = oc.uod(raw, lv.metadata, grid=self._grid(level), subset_stride=self.s, model=self.model,
                     policy=self.policy, median_size=self.median_size,
                     seed_mode=self.policy == "median" and level > 0,
                     permissions=None if self.rois is None else self.rois[level].links)
        return raw, out

    def register(self, frame: np.ndarray, levels_used: int | None = None,
                 shift: tuple[float, float] | None = None) -> tuple[np.ndarray, list[int]]:
        """One frame; `shift` = the frame's global translation (Fourier
        initialization)."""
        L = levels_used or self.L
        frames = [np.ascontiguousarray(frame, dtype=np.uint8)]
        for _ in range(1, L):
            frames.append(oc.reduce(frames[-1]))
        counters = [0, 0, 0, 0]
        c = L - 1
        seed = active = None
        if self.temporal:
            source = self.history
            if self.velocity:
                source, counters[2] = oc.temporal_predict(self.history, self.prev_history, self.ages,
                                                          self.prev_ages, model=self.model)
            links = self.temporal_links if c == self.L - 1 else None
            seed, active, weights = oc.transfer_seed(
                source, source_grid=self._grid(0), destination_grid=self._grid(c), source_scale=1.0,
                destination_scale=float(1 << c), subset_size=self.S, subset_stride=self.s, model=self.model,
                track_availability=self.fine_correction, return_weights=True, permissions=links)
            projected = weights > 0.0
            if links is not None:
                projected &= (np.asarray(links, np.uint32).ravel() & 16) != 0
            counters[0] = int(projected.sum())
            if self.search_radius:
                seed[weights == 0.0, self.status_at] = -1.0
            if self.fine_correction:
                seed[~projected, self.status_at] = -1.0
        selected = None if self.rois is None else self.rois[c].selected
        if self.global_shift:
            count = self.levels[c].grid_w * self.levels[c].grid_h
            seed = np.zeros((count, self.ss), np.float32)
            inv = np.float32(1.0 / (1 << c))
            seed[:, 0] = np.float32(shift[0]) * inv
            seed[:, 3] = np.float32(shift[1]) * inv
            active = np.ones(count, np.uint32) if selected is None else (selected != 0).astype(np.uint32)
        if self.search_radius and c == self.L - 1:
            seed, active, _ = oc.seed_search(
                self.reference_levels[c], frames[c], subset_size=self.S, subset_stride=self.s,
                radius=self.search_radius, model=self.model, seed=seed, only_missing=self.temporal,
                selected=selected, active=active, centered=self.global_shift)
        raws, outs = {}, {}
        raws[c], outs[c] = self._solve_level(c, frames[c], seed, active)
        for level in range(L - 2, -1, -1):
            seed, active = oc.transfer_seed(
                outs[level + 1], source_grid=self._grid(level + 1), destination_grid=self._grid(level),
                source_scale=float(1 << (level + 1)), destination_scale=float(1 << level), subset_size=self.S,
                subset_stride=self.s, model=self.model, track_availability=self.fine_correction,
                permissions=None if self.rois is None else self.rois[level].seed_links)
            if level == 0 and self.temporal and self.fine_correction:
                seed = oc.refine_temporal_seed(
                    seed, active, self.coarse_history, self.coarse_ages, self.history, self.ages,
                    source_grid=self._grid(1), destination_grid=self._grid(0), source_scale=2.0,
                    subset_size=self.S, subset_stride=self.s, model=self.model, max_age=self.max_age,
                    permissions=None if self.rois is None else self.rois[0].seed_links)
            raws[level], outs[level] = self._solve_level(level, frames[level], seed, active)
        if self.temporal:
            use_filtered = self.policy == "replace" and not self.velocity
            if self.velocity:
                oc.temporal_save_previous(self.history, self.ages, raws[0], outs[0], self.prev_history,
                                          self.prev_ages, model=self.model)
            accepted, expired = oc.temporal_merge(self.history, self.ages, raws[0], outs[0], model=self.model,
                                                  max_age=self.max_age, use_filtered=use_filtered)
            counters[1] = accepted
            counters[3] = expired if self.adaptive else 0
            if self.fine_correction:
                top = self.L - 1
                if top in raws:
                    raw_top, out_top = raws[top], outs[top]
                else:
                    raw_top = out_top = np.zeros_like(self.coarse_history)
                oc.temporal_merge(self.coarse_history, self.coarse_ages, raw_top, out_top, model=self.model,
                                  max_age=self.max_age, use_filtered=use_filtered)
        return outs[0], counters


def roi_tables(mask: np.ndarray | None, *, subset_size: int, subset_stride: int, levels: int,
               median_filter_size: int = 3, outlier_policy: str = "replace"):
    """The host ROI tables a full-pyramid engine uploads for `mask` (per-level
    selection, UOD links, coarse-to-fine seed permissions, and the temporal
    projection's permissions), from the package's ROI planner (whose plans
    are pinned to the reference's).  Returns (plans, rois, temporal_links),
    or (None, None, None) without a mask."""
    from live_dic_gb300.roi import integral, prepare_roi, reduce_mask, seed_permissions

    if mask is None:
        return None, None, None
    masks = [mask]
    for _ in range(1, levels):
        masks.append(reduce_mask(masks[-1]))
    plans = [prepare_roi(m, subset_size, subset_stride, median_filter_size=median_filter_size) for m in masks]
    prefix = integral(mask)
    rois = []
    for level, plan in enumerate(plans):
        links = None
        if level < levels - 1:
            links = np.ascontiguousarray(seed_permissions(
                plans[level + 1], plan, source_scale=1 << (level + 1), destination_scale=1 << level,
                size=subset_size, stride=subset_stride, reference_mask=mask, reference_prefix=prefix),
                dtype=np.uint32).ravel()
        rois.append(LevelRoi(np.ascontiguousarray(plan.selected, np.uint8).ravel(),
                             np.ascontiguousarray(plan.links_table(median_filter_size, outlier_policy)), links))
    temporal = np.ascontiguousarray(seed_permissions(
        plans[0], plans[-1], source_scale=1, destination_scale=1 << (levels - 1), size=subset_size,
        stride=subset_stride, reference_mask=mask, reference_prefix=prefix), dtype=np.uint32).ravel()
    return plans, rois, temporal


def float64_levels(reference: np.ndarray, *, subset_size: int, subset_stride: int, levels: int,
                   plans=None) -> tuple[list[LevelArrays], list[np.ndarray]]:
    """Per-level reference arrays from the float64 restatement of
    _reference_arrays on the integer pyramid of `reference` (windows a plan
    excludes get validity -3), and the level images."""
    images = [np.ascontiguousarray(reference, dtype=np.uint8)]
    for _ in range(1, levels):
        images.append(oc.reduce(images[-1]))
    out = []
    for level, img in enumerate(images):
        plane, inverse, metadata = rp.reference_arrays(img, subset_size=subset_size, subset_stride=subset_stride)
        h, w = img.shape
        gw, gh = 1 + (w - subset_size) // subset_stride, 1 + (h - subset_size) // subset_stride
        if plans is not None:
            meta = metadata.reshape(gw * gh, -1)
            meta[~plans[level].selected.ravel(), 1] = -3.0
        out.append(LevelArrays(w, h, gw, gh, plane, metadata, inverse))
    return out, images
