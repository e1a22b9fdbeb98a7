import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "stress-particle-sph_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def _has_gpu():
    """True when the CUDA runtime sees a device (checked without importing torch)."""
    import ctypes
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        n = ctypes.c_int(0)
        try:
            return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
        except Exception:
            return False
    return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU visible")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Build the host library and the oracle (and the CUDA library when possible)."""
    import sps_gb300
    import orc
    sps_gb300.build_host()
    orc.build()
    return True


@pytest.fixture(scope="session")
def built_gpu(built):
    import sps_gb300
    sps_gb300.build_cuda()
    return True
