import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def gpu_lib():
    """The in-tree CUDA library, built on first use; fails loudly when it cannot be loaded."""
    from opensurgsim_gb300 import build, _lib

    build.build()
    return _lib.load()
