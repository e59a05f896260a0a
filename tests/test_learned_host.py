"""Host-side logic of the learned seeding (no GPU): the consensus statement
that the device kernel follows (fit_consensus) and its tables."""

from __future__ import annotations

import numpy as np
import pytest

learned = pytest.importorskip("live_dic_gb300.learned")


def _lattice(lw, lh, pitch=64.0):
    gy, gx = np.mgrid[0:lh, 0:lw] * pitch
    node = np.stack([gx.ravel(), gy.ravel()], -1)
    return ((node - node.mean(0)) / 1000.0).astype(np.float32).astype(np.float64)


def test_tables_are_deterministic_and_in_range():
    a, b = learned.consensus_tables(510), learned.consensus_tables(510)
    for x, y in zip(a, b, strict=True):
        np.testing.assert_array_equal(x, y)
    singles, triples, probes = a
    assert singles.shape == (256,) and triples.shape == (128, 3) and probes.shape == (256,)
    assert len(set(probes.tolist())) == 256
    assert all(0 <= t.min() and t.max() < 510 for t in a)
    assert np.array_equal(learned.consensus_tables(100)[2], np.arange(100))


@pytest.mark.parametrize("outliers", [0.0, 0.3, 0.6])
def test_affine_field_recovered_through_outliers(outliers):
    rng = np.random.default_rng(int(outliers * 10) + 1)
    xy = _lattice(30, 17)
    n = len(xy)
    truth = np.stack([21.0 + 9.0 * xy[:, 0] - 4.0 * xy[:, 1], -13.0 + 2.0 * xy[:, 0] + 7.0 * xy[:, 1]], -1)
    t = truth + rng.normal(0.0, 0.5, truth.shape)
    bad = rng.random(n) < outliers
    t[bad] = rng.uniform(-45.0, 45.0, (int(bad.sum()), 2))
    t[5] = np.nan
    fitted = learned.fit_consensus(t, xy, learned.consensus_tables(n))
    assert np.isfinite(fitted).all()
    np.testing.assert_allclose(fitted, truth, atol=0.3)


def test_too_few_finite_nodes_return_the_input():
    xy = _lattice(3, 2)
    t = np.full((6, 2), np.nan)
    t[0] = (1.0, 2.0)
    t[3] = (1.5, 2.5)
    out = learned.fit_consensus(t, xy, learned.consensus_tables(6))
    np.testing.assert_array_equal(np.isnan(out), np.isnan(t))
