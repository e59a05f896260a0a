"""The full-pyramid oracle on its own (CPU, no GPU): float64 reference
preparation per level (oracle/reference_prep.py, pinned to the reference's
NumPy code) feeding the C oracle's per-frame pipeline over a short temporal
sequence; the composed oracle must recover the imposed field, which pins the
checker that the GPU pipeline is compared with bit for bit."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as oc
from oracle import reference_prep as rp
from oracle.pyramid_oracle import LevelArrays, PyramidOracle

W, H, S, ST = 192, 160, 21, 10


@pytest.fixture(scope="module")
def sequence():
    rng = np.random.default_rng(314)
    dots = 4000 * W * H // (512 * 512)
    cx, cy = rng.uniform(-10, W + 10, dots), rng.uniform(-10, H + 10, dots)
    sig, amp = rng.uniform(1.5, 3.0, dots), rng.uniform(0.3, 1.0, dots)

    def image(u0, v0, noise_seed):
        y, x = np.mgrid[0:H, 0:W].astype(np.float64)
        X, Y = x - u0, y - v0
        img = np.zeros((H, W))
        for k in range(dots):
            img += amp[k] * np.exp(-((X - cx[k]) ** 2 + (Y - cy[k]) ** 2) / (2 * sig[k] ** 2))
        img = 255.0 * (img - img.min()) / (img.max() - img.min() + 1e-12)
        img += np.random.default_rng(noise_seed).normal(0.0, 0.5, img.shape)
        return np.clip(np.rint(img), 0, 255).astype(np.uint8)

    ref = image(0.0, 0.0, 1)
    frames = [image(0.4 * k, -0.25 * k, 10 + k) for k in range(1, 4)]
    return ref, frames


def _levels(ref, count):
    levels, img = [], ref
    for level in range(count):
        plane, inverse, metadata = rp.reference_arrays(img, subset_size=S, subset_stride=ST)
        h, w = img.shape
        levels.append(LevelArrays(w, h, 1 + (w - S) // ST, 1 + (h - S) // ST, plane, metadata, inverse))
        img = oc.reduce(img)
    return levels


def test_pyramid_oracle_recovers_a_translation_sequence(sequence):
    oc.build()
    ref, frames = sequence
    levels = _levels(ref, 2)
    oracle = PyramidOracle(levels, subset_size=S, subset_stride=ST, iterations=(8, 16), tolerances=(5e-3, 5e-3),
                           lanes=16, temporal=True, velocity=True)
    gw, gh = levels[0].grid_w, levels[0].grid_h
    for k, frame in enumerate(frames, start=1):
        state, counters = oracle.register(frame)
        state = state.reshape(gh, gw, -1)[1:-1, 1:-1]   # border windows leave the frame
        ok = state[..., 6] >= 1
        assert ok.mean() > 0.95, (k, ok.mean())
        err = np.hypot(state[..., 0] - 0.4 * k, state[..., 3] + 0.25 * k)[ok]
        assert float(np.sqrt(np.mean(err ** 2))) < 0.02, k
        if k > 1:
            assert counters[0] > 0 and counters[1] > 0


def test_pyramid_oracle_with_roi_hole_and_first_frame_search(sequence):
    """The ROI and seed-search paths of the composed oracle: a circular hole
    excluded from every level (status -3, UOD and seed permissions from the
    host ROI plan), the integer ZNCC search on the coarsest level for the
    first frame and for windows the temporal projection leaves unseeded."""
    from live_dic_gb300.roi import integral, prepare_roi, reduce_mask, seed_permissions
    from oracle.pyramid_oracle import LevelRoi

    oc.build()
    ref, frames = sequence
    yy, xx = np.ogrid[:H, :W]
    mask = (xx - W / 2) ** 2 + (yy - H / 2) ** 2 >= 30.0 ** 2
    masks = [mask, reduce_mask(mask)]
    plans = [prepare_roi(m, S, ST) for m in masks]
    levels = _levels(ref, 2)
    for lv, plan in zip(levels, plans, strict=True):
        meta = lv.metadata.reshape(lv.grid_w * lv.grid_h, -1)
        meta[~plan.selected.ravel(), 1] = -3.0
    prefix = integral(mask)
    links0 = seed_permissions(plans[1], plans[0], source_scale=2, destination_scale=1, size=S, stride=ST,
                              reference_mask=mask, reference_prefix=prefix)
    temporal = seed_permissions(plans[0], plans[1], source_scale=1, destination_scale=2, size=S, stride=ST,
                                reference_mask=mask, reference_prefix=prefix)
    rois = [LevelRoi(plans[0].selected.astype(np.uint8).ravel(), plans[0].links_table(3, "replace"),
                     np.asarray(links0, np.uint32).ravel()),
            LevelRoi(plans[1].selected.astype(np.uint8).ravel(), plans[1].links_table(3, "replace"), None)]
    oracle = PyramidOracle(levels, subset_size=S, subset_stride=ST, iterations=(8, 16), tolerances=(5e-3, 5e-3),
                           lanes=16, temporal=True, velocity=True, rois=rois,
                           temporal_links=np.asarray(temporal, np.uint32).ravel(), search_radius=3,
                           reference_levels=[ref, oc.reduce(ref)])
    gw, gh = levels[0].grid_w, levels[0].grid_h
    selected = plans[0].selected
    assert not selected.all() and selected.mean() > 0.6
    for k, frame in enumerate(frames, start=1):
        state, counters = oracle.register(frame)
        state = state.reshape(gh, gw, -1)
        assert np.all(state[..., 6][~selected] == -3.0)
        inner = np.zeros_like(selected)
        inner[1:-1, 1:-1] = True
        ok = (state[..., 6] >= 1) & inner & selected
        assert ok.sum() > 0.9 * (inner & selected).sum(), (k, ok.sum())
        err = np.hypot(state[..., 0] - 0.4 * k, state[..., 3] + 0.25 * k)[ok]
        assert float(np.sqrt(np.mean(err ** 2))) < 0.02, k
        if k == 1:
            assert counters[0] == 0
        else:
            assert counters[0] > 0 and counters[1] > 0
