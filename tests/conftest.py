import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def hfx_lib():
    """The CUDA library, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    from hyperfox_gb300 import build, capi
    if not os.path.exists(capi.LIB_PATH):
        build.build()
    return capi.load()
