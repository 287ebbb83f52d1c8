import ctypes
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: multi-GB cases")


@pytest.fixture(scope="session")
def E():
    import eithot_gb300
    return eithot_gb300


@pytest.fixture(scope="session")
def hostsim():
    import __graft_entry__ as g
    lib = ctypes.CDLL(g.build_hostsim())
    lib.hs_last_error.restype = ctypes.c_char_p
    I64P = ctypes.POINTER(ctypes.c_int64)
    IP = ctypes.POINTER(ctypes.c_int)
    lib.hs_transpose.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, I64P, IP, ctypes.c_size_t,
                                 ctypes.c_int, ctypes.c_double, ctypes.c_int]
    lib.hs_describe.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, I64P, IP, ctypes.c_size_t,
                                ctypes.c_int, ctypes.c_double, ctypes.c_int]
    return lib
