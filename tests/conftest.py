import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libneofiz_gpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if stale) and loads the CUDA library; fails loudly when it cannot."""
    from neofiz_gb300 import build, _native
    build.build()
    return _native.api()


@pytest.fixture(scope="session")
def oracle_api():
    from oracle import oracle
    return oracle.api()
