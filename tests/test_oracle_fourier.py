"""CPU pins of the Fourier initializer: the oracle and the product's window
choice against the reference's own FourierInitializer outputs
(tests/golden/fourier_vectors.npz, made by tests/golden/make_golden.py)."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from oracle import fourier_oracle

GOLDEN = Path(__file__).resolve().parent / "golden" / "fourier_vectors.npz"


@pytest.fixture(scope="module")
def fourier_golden():
    with np.load(GOLDEN) as g:
        return {k: g[k] for k in g.files}


@pytest.mark.parametrize("k", range(4))
def test_oracle_matches_reference(fourier_golden, k):
    g = fourier_golden
    mask = g[f"fourier_{k}_mask"] if bool(g[f"fourier_{k}_has_mask"]) else None
    est = fourier_oracle.estimate(g[f"fourier_{k}_ref"], g[f"fourier_{k}_tgt"], mask)
    assert list(est["window"]) == list(g[f"fourier_{k}_window"])
    accepted = est["peakScore"] >= 8.0 and est["overlap"] >= 0.25 and est["correlation"] >= 0.2
    assert accepted == bool(g[f"fourier_{k}_accepted"])
    if accepted:
        r = g[f"fourier_{k}_result"]
        assert (est["dx"], est["dy"]) == (int(r[0]), int(r[1]))
        np.testing.assert_allclose([est["peakScore"], est["overlap"], est["correlation"]], r[2:], rtol=1e-9)
