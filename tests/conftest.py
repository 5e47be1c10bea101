import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libmepi_gb300.so)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the CUDA library; GPU tests fail loudly without it."""
    from mepinterp_gb300 import build, api
    build.build()
    return api.load_library()
