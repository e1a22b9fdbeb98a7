"""GPU: the launch-shape autotuner (sps_autotune) changes speed only.

Tuning runs profiled steps at several block sizes and restores the state it started from,
so a run tuned first must equal, bit for bit, the same run untuned, in both forms and for
a batch.
"""
import numpy as np
import pytest

import cases
import sps_gb300
from sps_gb300 import _abi

pytestmark = pytest.mark.gpu

FIELDS = ("x", "vel", "stress", "rho", "intvars1", "displ", "f_drucker", "bc_or_not")


@pytest.mark.parametrize("precision", [_abi.SPS_PREC_FP64_PLAIN, _abi.SPS_PREC_FP32_FAST],
                         ids=["plain", "fp32"])
def test_tuned_run_equals_untuned(built_gpu, precision):
    p = cases.bui_like()
    out = []
    for tune in (True, False):
        ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", p.params_copy(precision=precision))
        ctx.upload_problem(p)
        if tune:
            chosen = sps_gb300.autotune(ctx, 2)
            assert set(chosen) == set(sps_gb300.context.TUNED_KERNELS)
            assert all(b in (64, 128, 256, 512) for b in chosen.values()), chosen
            assert chosen["derivs"] <= 256
        t = ctx.step(6, 0.0)
        t = ctx.step(6, t)
        out.append((t, ctx.download(), ctx.dump_pairs()))
        ctx.close()
    (ta, a, pa), (tb, b, pb) = out
    assert ta == tb
    for k in FIELDS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    for k in ("pair_i", "pair_j", "w"):
        np.testing.assert_array_equal(pa[k], pb[k], err_msg=k)


def test_tuned_batch_equals_untuned(built_gpu):
    probs = [cases.bui_like(), cases.bui_like(width=1.0, height=0.5, dx=0.05, dt=1.0e-4)]
    res = []
    for tune in (True, False):
        b = sps_gb300.Batch(probs, precision=_abi.SPS_PREC_FP32_FAST)
        b.upload_all()
        if tune:
            sps_gb300.autotune(b, 2)
        b.step(8)
        res.append([b.download(r) for r in range(len(probs))])
        b.close()
    for r in range(len(probs)):
        for k in FIELDS:
            np.testing.assert_array_equal(res[0][r][k], res[1][r][k], err_msg="%d %s" % (r, k))


@pytest.mark.parametrize("make", [lambda: cases.bui_like(),
                                  lambda: cases.bui_like(width=1.0, height=0.5, dx=0.05,
                                                         cspm=True, alpha=0.0, beta=0.0)],
                         ids=["walls_xsph_viscosity", "cspm"])
def test_lookahead_changes_nothing(built_gpu, make):
    # the FP32 neighbour sums load 1-8 neighbours before summing any, in the same order:
    # every look-ahead gives the same bits, so the autotuner may choose any
    p = make()
    res = []
    # and the bulk L2 prefetch of list entries is a hint: on or off, the same bits
    for interp, derivs, pf in ((4, 2, 0), (2, 2, 3), (2, 1, 1), (8, 4, 2)):
        ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                    p.params_copy(precision=_abi.SPS_PREC_FP32_FAST))
        sps_gb300.set_lookahead(ctx, interp, derivs)
        sps_gb300.set_prefetch(ctx, pf & 1, pf & 2)
        assert sps_gb300.lookahead(ctx) == {"interp": interp, "derivs": derivs}
        assert sps_gb300.prefetch(ctx) == {"interp": bool(pf & 1), "derivs": bool(pf & 2)}
        ctx.upload_problem(p)
        ctx.step(10, 0.0)
        res.append(ctx.download())
        ctx.close()
    for r in res[1:]:
        for k in FIELDS:
            np.testing.assert_array_equal(r[k], res[0][k], err_msg=k)
    ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                p.params_copy(precision=_abi.SPS_PREC_FP32_FAST))
    ctx.upload_problem(p)
    sps_gb300.autotune(ctx, 2)
    la = sps_gb300.lookahead(ctx)
    assert la["interp"] in (2, 4, 8) and la["derivs"] in (1, 2, 4), la
    with pytest.raises(sps_gb300.SpsError):
        sps_gb300.set_lookahead(ctx, 3, 2)
    ctx.close()
