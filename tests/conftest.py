import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA engine")
    config.addinivalue_line("markers", "slow: longer CPU tests")


def _have_gpu() -> bool:
    try:
        from clode_gb300 import _native as N
        import ctypes as C
        n = C.c_int(0)
        return N.lib.clode_device_count(C.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_available():
    return _have_gpu()


def pytest_collection_modifyitems(config, items):
    # GPU tests on a machine without a GPU fail loudly rather than skip: the
    # engine has no CPU path.  Select them with -m gpu only where a GPU exists.
    pass
