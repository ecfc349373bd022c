"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import importlib
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT), str(ROOT / "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


@pytest.fixture(scope="session")
def latpkg():
    """The engine package (lattice-dev_gb300)."""
    return importlib.import_module("lattice-dev_gb300")


@pytest.fixture(scope="session")
def engine(latpkg):
    """The loaded engine library: raises if it has not been built (no CPU fallback)."""
    latpkg.load_library()
    return latpkg


@pytest.fixture(scope="session")
def orc():
    import py_oracle
    py_oracle.load()
    return py_oracle


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))
