import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "enkf-c_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load libenkfg.so; the GPU tests call through it."""
    import build
    build.build()
    import enkfg
    return enkfg


@pytest.fixture(scope="session")
def ctx(gpu_lib):
    c = gpu_lib.Enkfg(0)
    yield c
    c.close()
