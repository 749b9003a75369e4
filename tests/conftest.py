import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    """Path of the shared library, building it (and the spectral2d_run main
    program) in-tree if either is absent."""
    from spectral2d_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH) or not os.path.exists(build.DRIVER):
        build.build()
    return _lib.LIB_PATH


@pytest.fixture(scope="session")
def gpu_lib(built_lib):
    from spectral2d_gb300 import _lib
    return _lib.lib()
