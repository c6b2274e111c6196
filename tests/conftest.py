import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def srlib():
    """libsr.so, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    import vkscanlinepr_gb300 as sr
    sr.build()
    sr.lib()
    return sr


@pytest.fixture(scope="session")
def gpu(srlib):
    """Fails (does not skip) when no GPU is visible: -m gpu tests must run."""
    # sr_create on device 0 is the real probe; a tiny context is cheap
    r = srlib.ScanlineVGRasterizer()
    r.initialize(None, 8, 8)
    r.close()
    return srlib
