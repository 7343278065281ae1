import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _stale(lib, srcdir):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    for dp, _, fs in os.walk(srcdir):
        for f in fs:
            if f.endswith((".cu", ".cuh", ".cpp", ".h")) and os.path.getmtime(os.path.join(dp, f)) > t:
                return True
    return False


@pytest.fixture(scope="session", autouse=True)
def native_libs():
    """Builds the oracle and the GPU library when missing or out of date."""
    from oracle import build as ob
    ob.build()
    from rayna_gb300 import build as rb
    if any(_stale(lib, os.path.join(ROOT, d)) for lib in (rb.LIB, rb.LIB_EXACT)
           for d in (os.path.join("rayna_gb300", "csrc"), "include")):
        rb.build()
    yield


@pytest.fixture(scope="session")
def gpu_available():
    import ctypes as C
    from rayna_gb300 import _abi as A
    lib = A.load_library()
    h = C.c_void_p()
    st = lib.rg_create(None, C.byref(h))
    if st == A.RG_OK:
        lib.rg_destroy(h)
        return True
    return False
