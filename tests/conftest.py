"""Shared pytest setup: markers, import paths and session fixtures.

Tests marked ``gpu`` need a CUDA device and the built library; everything
else runs on the CPU.  The oracle (oracle/) is test infrastructure and is
imported only here and in the test modules.
"""
import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
for p in (REPO / "atlas-engine_gb300", REPO / "oracle", REPO):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libatlas_rt.so")


@pytest.fixture(scope="session")
def native():
    """Builds (if needed) and loads libatlas_rt.so."""
    from atlas_rt import build as _b
    _b.build()
    from atlas_rt import _native
    return _native.lib()


@pytest.fixture(scope="session")
def ctx(native):
    import atlas_rt
    c = atlas_rt.Context(device=0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    import json
    d = REPO / "tests" / "golden"
    return np.load(d / "small_cases.npz"), json.loads((d / "digests.json").read_text())


@pytest.fixture(scope="session", autouse=True)
def _built_library():
    """The product library is built before any test (nvcc cross-compiles
    without a GPU); the oracle port is built with gcc."""
    from atlas_rt import build as _b
    _b.build()
    import pyoracle
    pyoracle.build_port()
