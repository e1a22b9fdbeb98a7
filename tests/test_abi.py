"""The C-ABI libraries load and export every function their public headers declare.

No compute call is made, so this runs without a GPU: libsps_gb300.so (include/sps.h) is
cross-compiled for sm_103a and only loaded; libsph_host.so (include/sph_host.h) is host
code.
"""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"^[A-Za-z_][\w\s\*]*?\b((?:sps|sph)_\w+)\s*\(", re.M)


def declared(header):
    with open(os.path.join(ROOT, "include", header)) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)  # drop comments
    text = re.sub(r"//[^\n]*", "", text)
    names = sorted(set(DECL.findall(text)))
    return [n for n in names if not n.endswith("_t")]


def test_headers_declare_functions():
    assert "sps_step" in declared("sps.h")
    assert "sph_problem_read" in declared("sph_host.h")


@pytest.mark.parametrize("header,lib", [("sps.h", "libsps_gb300.so"),
                                        ("sps_surrogate.h", "libsps_gb300.so"),
                                        ("sph_host.h", "libsph_host.so")])
def test_library_exports_header(built, header, lib):
    import sps_gb300
    from sps_gb300 import build as _build
    if lib == "libsps_gb300.so":
        sps_gb300.build_cuda()  # nvcc cross-compiles without a GPU
    dll = C.CDLL(_build.lib_path(lib))
    missing = [n for n in declared(header) if not hasattr(dll, n)]
    assert not missing, missing


def test_params_layout_matches_binding(built):
    # the ctypes mirror of sps_params must have the C struct's size (a missing or reordered
    # field would shift every later one)
    import sps_gb300
    from sps_gb300 import _abi
    from sps_gb300 import build as _build
    sps_gb300.build_host()
    dll = C.CDLL(_build.lib_path("libsph_host.so"))
    dll.sph_sizeof_params.restype = C.c_int32
    assert dll.sph_sizeof_params() == C.sizeof(_abi.SpsParams)
