import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def native_lib():
    """The built adfwi_gb300 library (built in-tree on first use)."""
    from adfwi_gb300.build import build
    build()
    from adfwi_gb300 import _native
    return _native.lib()
