import ctypes as C
import ctypes.util
import glob
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session")
def oracle_built():
    """Compile the oracle (C restatement) once per session."""
    import pyoracle

    pyoracle.build()
    return True


@pytest.fixture(scope="session")
def gpu():
    """Build (if stale) and load the CUDA library; GPU tests need a GB300."""
    from ffea_ci_demo_gb300 import build, lib

    build.build()
    return lib.load()


@pytest.fixture(scope="session")
def device_free_bytes():
    """cudaMemGetInfo's free bytes of the current device, through the CUDA runtime the library links."""
    rt = None
    for c in ["libcudart.so.13", ctypes.util.find_library("cudart")] + sorted(
            glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        if not c:
            continue
        try:
            rt = C.CDLL(c)
            break
        except OSError:
            continue
    if rt is None:
        pytest.skip("libcudart not found")
    rt.cudaMemGetInfo.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    rt.cudaMemGetInfo.restype = C.c_int

    def free() -> int:
        f, t = C.c_size_t(), C.c_size_t()
        assert rt.cudaMemGetInfo(C.byref(f), C.byref(t)) == 0
        return f.value

    return free
