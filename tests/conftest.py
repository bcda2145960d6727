import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI)")


@pytest.fixture(scope="session")
def lib():
    """The built CUDA library (built on demand; GPU tests only)."""
    from eq_gb300 import build
    build.build()
    from eq_gb300 import _lib
    return _lib.load()
