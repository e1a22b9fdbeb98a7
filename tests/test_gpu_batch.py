"""GPU: batches of realisations (sps_create_batch) against the same problems run alone.

Each realisation of a batch keeps its own cell grid and pair-list bookkeeping, so after any
number of steps its pair list and its fields must be bit-identical to a context holding it
alone, in both arithmetic forms, although the batch advances all of them with one launch
per kernel.  The realisations differ in size, material and time step.
"""
import numpy as np
import pytest

import cases
import sps_gb300
from sps_gb300 import _abi

pytestmark = pytest.mark.gpu


def problems():
    return [cases.bui_like(),
            cases.column(dx=0.004, xsph=True, phi_deg=25.0, young=1.5e7, rho=2300.0,
                         cohesion=150.0),
            cases.bui_like(width=1.0, height=0.5, dx=0.05, young=3.0e6, tanphi=0.6, coh=2000.0,
                           dt=1.0e-4)]


FIELDS = ("x", "vel", "stress", "rho", "intvars1", "displ", "f_drucker")


@pytest.mark.parametrize("precision", [_abi.SPS_PREC_FP64_PLAIN, _abi.SPS_PREC_FP32_FAST],
                         ids=["plain", "fp32"])
def test_batch_matches_single_runs(built_gpu, precision):
    probs = problems()
    b = sps_gb300.Batch(probs, precision=precision)
    b.upload_all()
    b.step(7)
    times = b.step(8)
    for r, prob in enumerate(probs):
        ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                    prob.params_copy(precision=precision))
        ctx.upload_problem(prob)
        t = ctx.step(7, 0.0)
        t = ctx.step(8, t)
        assert t == times[r]
        one, many = ctx.download(), b.download(r)
        for k in FIELDS:
            np.testing.assert_array_equal(many[k], one[k], err_msg="realisation %d %s" % (r, k))
        p1, pb = ctx.dump_pairs(), b.dump_pairs(r)
        for k in ("pair_i", "pair_j", "pint_type", "w", "dwdx", "dwdy"):
            np.testing.assert_array_equal(pb[k], p1[k], err_msg="realisation %d %s" % (r, k))
        ctx.close()
    b.close()


def test_batch_rejects_mixed_flags(built_gpu):
    probs = [cases.bui_like(), cases.column(dx=0.004)]  # XSPH on / off
    with pytest.raises(sps_gb300.SpsError):
        sps_gb300.Batch(probs)
