"""CPU pins of the oracle's spatial-seed restatement (spatial_seed.wgsl):
the affine frontier against the reference's own NumPy expectation
(test_affine_frontier.py:70-140) and hypothesis scoring on an exact
integer shift."""

from __future__ import annotations

import numpy as np

from oracle import oracle as oracle_c


def test_frontier_matches_reference_numpy_median():
    rng = np.random.default_rng(27)
    states = rng.normal(0, 0.1, (9, 8)).astype(np.float32)
    states[:, 0] += 2
    states[:, 3] -= 1
    states[:, 6] = 1
    states[4, 6] = 0
    permissions = np.full((3, 3), 511, np.uint32)
    seeds, active = oracle_c.affine_frontier(states.reshape(3, 3, 8), permissions, subset_stride=16)
    candidates = []
    for idx in range(9):
        if idx == 4:
            continue
        dx, dy = (1 - idx % 3) * 16, (1 - idx // 3) * 16
        p = states[idx].copy()
        p[0] += p[1] * dx + p[2] * dy
        p[3] += p[4] * dx + p[5] * dy
        candidates.append(p[:6])
    np.testing.assert_allclose(seeds[1, 1, :6], np.median(candidates, axis=0), atol=1e-6)
    assert active.sum() == 1 and active[1, 1]


def test_frontier_respects_permissions_and_acceptance():
    states = np.zeros((3, 4, 8), np.float32)
    states[1, 1, :6] = [1.0, 0.01, 0.0, -2.0, 0.0, 0.02]
    states[1, 1, 6] = 1.0
    permissions = np.full((3, 4), 511, np.uint32)
    permissions[1, 2] &= ~np.uint32(1 << 3)  # subset (1, 2) may not take its left neighbour
    seeds, active = oracle_c.affine_frontier(states, permissions, subset_stride=10)
    assert not active[1, 1] and not active[1, 2]
    assert active[0, 0] and active[2, 2] and active[0, 2]
    # first-order transport from (1,1) to (0,0): delta = (-10, -10)
    np.testing.assert_allclose(seeds[0, 0, :6], [1.0 - 0.1, 0.01, 0.0, -2.0 - 0.2, 0.0, 0.02], rtol=1e-6)


def test_choose_finds_the_neighbour_translation():
    rng = np.random.default_rng(5)
    ref = rng.integers(0, 256, (96, 96), dtype=np.uint8)
    tgt = np.roll(ref, shift=(-2, 3), axis=(0, 1))  # content moves by (+3, -2)
    S, st = 16, 16
    gh = gw = 1 + (96 - S) // st
    states = np.zeros((gh, gw, 8), np.float32)
    states[2, 2, 0], states[2, 2, 3], states[2, 2, 6] = 3.0, -2.0, 1.0
    permissions = np.full((gh, gw), 511, np.uint32)
    seeds, active, scores = oracle_c.spatial_choose(ref, tgt, states, permissions, subset_size=S, subset_stride=st)
    assert active[2, 3] and active[3, 3] and active[1, 1]
    np.testing.assert_array_equal(seeds[2, 3, [0, 3]], [3.0, -2.0])
    assert scores[2, 3, 1] > 0.999 and scores[2, 3, 0] < 0.5
    assert not active[2, 2]  # its own hypothesis is already the best
    _, median_only, _ = oracle_c.spatial_choose(ref, tgt, states, permissions, subset_size=S, subset_stride=st,
                                                candidate_mode=1)
    assert median_only[2, 3]
