import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

# A checkout of the reference project, for the tests that read its own files
# (rule caches, the shipped sample, its prepared case): the TAILOR_REFERENCE
# environment variable names it; those tests skip when it is unset.
REFERENCE = Path(os.environ["TAILOR_REFERENCE"]) if os.environ.get("TAILOR_REFERENCE") else None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def has_gpu() -> bool:
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so")
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def gpu_lib():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from tailor_gb300 import build
    build.build()
    from tailor_gb300 import _lib
    return _lib.load()
