"""GPU: the checks of sps_upload (done on the device, one host synchronisation) and the
download into caller-provided arrays."""
import numpy as np
import pytest

import cases
import sps_gb300
from sps_gb300 import _abi

pytestmark = pytest.mark.gpu


def _ctx(prob):
    return sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", prob.params_copy())


def test_rejected_upload_then_valid_upload(built_gpu):
    prob = cases.bui_like()
    ctx = _ctx(prob)
    st = prob.state()
    bad = dict(st)
    bad["itype"] = st["itype"].copy()
    bad["itype"][prob.nnode + 3] = 2  # a node among the stress-points
    with pytest.raises(sps_gb300.SpsError, match="itype"):
        ctx.upload(**bad)
    with pytest.raises(sps_gb300.SpsError):
        ctx.step(1, 0.0)  # the context holds no valid state
    nan = dict(st)
    nan["x"] = st["x"].copy()
    nan["x"][5] = np.nan
    with pytest.raises(sps_gb300.SpsError, match="non-finite"):
        ctx.upload(**nan)
    ctx.upload_problem(prob)
    ctx.step(4, 0.0)
    ref = _ctx(prob)
    ref.upload_problem(prob)
    ref.step(4, 0.0)
    cases.assert_bitwise(ctx.download(), ref.download(), prob.ntotal)
    ctx.close()
    ref.close()


def test_download_into_given_arrays(built_gpu):
    prob = cases.bui_like()
    ctx = _ctx(prob)
    ctx.upload_problem(prob)
    ctx.step(3, 0.0)
    want = ctx.download()
    out = {k: np.full_like(v, 7) for k, v in want.items()}
    got = ctx.download(out=out)
    assert got is out
    cases.assert_bitwise(got, want, prob.ntotal)
    with pytest.raises(ValueError):
        ctx.download(out=dict(out, rho=np.empty(3)))
    ctx.close()


def test_nonfinite_state_after_a_step(built_gpu):
    # a NaN stress is accepted by the upload (it checks positions and smoothing lengths
    # only); the step propagates it into velocities and positions, and the finiteness check
    # after the step reports SPS_ERR_NONFINITE.  The context stays usable: a valid upload
    # then steps exactly as the oracle does after the same sequence (the pair list's
    # bookkeeping carries over an upload in both, as the reference's linked list carries
    # over its steps)
    import orc
    prob = cases.bui_like()
    ctx = _ctx(prob)
    ref = orc.context(prob.params_copy())
    st = prob.state()
    st["stress"] = st["stress"].copy()
    st["stress"][4 * (prob.nnode + 7) + 1] = np.nan
    ctx.upload(**st)
    ref.upload(**st)
    with pytest.raises(sps_gb300.SpsError) as e:
        ctx.step(1, 0.0)
    assert e.value.rc == _abi.SPS_ERR_NONFINITE
    ref.step(1, 0.0)
    assert not np.isfinite(ref.download()["x"]).all()
    for c in (ctx, ref):
        c.upload_problem(prob)
        c.step(3, 0.0)
    cases.assert_bitwise(ctx.download(), ref.download(), prob.ntotal)
    ctx.close()
    ref.close()
