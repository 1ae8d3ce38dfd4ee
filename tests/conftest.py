import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and runs the CUDA kernels")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def snac_lib():
    """The compiled extension; GPU tests fail loudly (no CPU fallback) when it or the device is missing."""
    from snac_gb300 import capi
    L = capi.lib()
    n = capi.device_count()
    if n < 1:
        pytest.fail("no CUDA device visible to libsnac_gb300 (GPU tests need one)")
    return L
