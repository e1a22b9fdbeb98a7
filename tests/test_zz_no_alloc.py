"""GPU: the allocation-free neighbour statistics entry point against the step's pair list.

sps_neighbour_stats_static (include/sps.h) counts, for every particle, the partners the
step's pair test accepts and sums their FP32 kernel values, with all device scratch in one
fixed array of the library instead of allocated memory.  Two calls in a row must each agree
with the pair list sps_dump_pairs returns after one step (the list is built from the
uploaded positions): neighbour counts and the pair count exactly, kernel sums to 1e-12
relative (the summation order inside a call is unspecified).  The file is collected last
so that the entry point also runs after every other test of the session.
"""
import ctypes as C

import numpy as np
import pytest

import cases
import sps_gb300
from sps_gb300 import _abi

pytestmark = pytest.mark.gpu


def _entry():
    f = sps_gb300.gpu_lib().sps_neighbour_stats_static
    f.argtypes = [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32,
                  C.c_double, C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                  C.POINTER(C.c_int64), C.c_char_p, C.c_int32]
    f.restype = C.c_int
    return f


def static_stats(x, h, skf, pi):
    n = len(h)
    deg = np.full(n, -1, np.int32)
    ws = np.full(n, np.nan)
    npairs = C.c_int64(-1)
    msg = C.create_string_buffer(256)
    rc = _entry()(n, x.ctypes.data_as(C.POINTER(C.c_double)),
                  h.ctypes.data_as(C.POINTER(C.c_double)), skf, pi, None,
                  deg.ctypes.data_as(C.POINTER(C.c_int32)), ws.ctypes.data_as(C.POINTER(C.c_double)),
                  C.byref(npairs), msg, 256)
    return rc, deg, ws, npairs.value, msg.value.decode()


def pair_list_stats(problem):
    """Neighbour counts and kernel sums from the pair list of the existing entry points."""
    ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                problem.params_copy(precision=_abi.SPS_PREC_FP64_PLAIN))
    ctx.upload_problem(problem)
    ctx.step(1, 0.0)
    p = ctx.dump_pairs()
    ctx.close()
    n = problem.ntotal2
    i, j = p["pair_i"] - 1, p["pair_j"] - 1
    w = p["w"].astype(np.float64)
    deg = np.bincount(i, minlength=n) + np.bincount(j, minlength=n)
    ws = np.bincount(i, weights=w, minlength=n) + np.bincount(j, weights=w, minlength=n)
    return deg, ws, len(i)


@pytest.mark.parametrize("make", [lambda: cases.bui_like(),
                                  lambda: cases.column(dx=0.004),
                                  lambda: cases.bui_like(width=1.0, height=0.5, dx=0.05, skf=2),
                                  lambda: cases.bui_like(width=1.0, height=0.5, dx=0.05, skf=3)],
                         ids=["bui_cubic", "column_cubic", "bui_gauss", "bui_quintic"])
def test_static_matches_pair_list(built_gpu, make):
    prob = make()
    deg_ref, ws_ref, np_ref = pair_list_stats(prob)
    x, h = prob.x.copy(), prob.hsml.copy()
    for call in range(2):  # two calls in a row share the scratch array
        rc, deg, ws, npairs, msg = static_stats(x, h, prob.params.skf, prob.params.pi)
        assert rc == _abi.SPS_OK, (call, rc, msg)
        np.testing.assert_array_equal(deg, deg_ref)
        assert npairs == np_ref, (call, npairs, np_ref)
        np.testing.assert_allclose(ws, ws_ref, rtol=1e-12, atol=0.0)


def test_static_limits(built_gpu):
    n = 65537  # SPS_STATIC_MAX_PARTICLES + 1
    x = np.zeros(2 * n)
    h = np.ones(n)
    rc, _, _, _, msg = static_stats(x, h, 1, np.pi)
    assert rc == _abi.SPS_ERR_CAPACITY and "65536" in msg, (rc, msg)
    rc, _, _, npairs, msg = static_stats(np.zeros(0), np.zeros(0), 1, np.pi)
    assert rc == _abi.SPS_OK and npairs == 0
    rc, _, _, _, msg = static_stats(np.zeros(4), np.array([1.0, 0.0]), 1, np.pi)
    assert rc == _abi.SPS_ERR_ARG and "smoothing length" in msg, (rc, msg)
    # two particles 1e6 smoothing lengths apart span far more cells than the scratch holds
    rc, _, _, _, msg = static_stats(np.array([0.0, 0.0, 1e6, 1e6]), np.ones(2), 1, np.pi)
    assert rc == _abi.SPS_ERR_CAPACITY and "cells" in msg, (rc, msg)
