"""pytest configuration: the `gpu` marker and shared fixtures.

Tests marked `gpu` call the CUDA kernels through the C ABI and need an
sm_100-family GPU; everything else runs on the CPU (oracle checks against the
reference's golden vectors, host logic, library symbol checks).
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU; calls the C ABI")


@pytest.fixture(scope="session")
def native_lib():
    """Builds (if stale) and loads libphylo_gpu.so."""
    from phylocaml_gb300 import build, _native
    build.build()
    return _native.load()


@pytest.fixture(scope="session")
def ctx(native_lib):
    """A context on GPU 0.  A GPU test fails (not skips) when none is usable."""
    from phylocaml_gb300 import _native
    c = _native.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle
