"""Test configuration: import paths, the `gpu` marker, oracle build."""

from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for path in (ROOT / "live-dic_gb300", ROOT, ROOT / "tests"):
    if str(path) not in sys.path:
        sys.path.insert(0, str(path))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libgbdic.so")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    from oracle import oracle as oracle_c

    oracle_c.build()
    yield


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(ROOT / "tests" / "golden" / "reference_vectors.npz")
