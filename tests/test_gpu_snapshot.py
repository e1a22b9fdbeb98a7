"""GPU: output snapshots (sps_snapshot / sps_snapshot_wait) and the writers fed from them.

A snapshot is staged on the device and copied out on a second stream while later steps run;
what it returns must be bit-identical to sps_download at the snapshot, and taking it must
not change the run (its free-surface refresh writes only what a download would)."""
import numpy as np
import pytest

import cases
import sps_gb300
from sps_gb300 import _abi

pytestmark = pytest.mark.gpu

KEYS = ("x", "vel", "stress", "rho", "intvars1", "displ", "f_drucker")


def _same(a, b, ntotal):
    cases.assert_bitwise(a, b, ntotal, KEYS)
    np.testing.assert_array_equal(a["bc_or_not"], b["bc_or_not"])


def _ctx(prob, precision):
    ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", prob.params_copy(precision=precision))
    ctx.upload_problem(prob)
    return ctx


@pytest.mark.parametrize("precision", [_abi.SPS_PREC_FP64_PLAIN, _abi.SPS_PREC_FP32_FAST],
                         ids=["plain", "fp32"])
def test_snapshot_equals_download(built_gpu, precision):
    prob = cases.bui_like()
    a, b, c = _ctx(prob, precision), _ctx(prob, precision), _ctx(prob, precision)
    t = a.step(6, 0.0)
    a.snapshot()
    t = a.step(9, t)  # runs while the snapshot copies out
    snap, step = a.snapshot_wait()
    assert step == 6
    b.step(6, 0.0)
    _same(snap, b.download(), prob.ntotal)
    # the run that took a snapshot continues exactly as one that did not
    c.step(15, 0.0)
    _same(a.download(), c.download(), prob.ntotal)
    # a second wait returns the same snapshot; a new snapshot replaces it
    again, step = a.snapshot_wait()
    assert step == 6
    _same(again, snap, prob.ntotal)
    a.snapshot()
    latest, step = a.snapshot_wait()
    assert step == 15
    _same(latest, c.download(), prob.ntotal)
    view, step = a.snapshot_view()
    assert step == 15
    _same(view, latest, prob.ntotal)
    for x in (a, b, c):
        x.close()


def test_snapshot_batch(built_gpu):
    probs = [cases.bui_like(), cases.bui_like(width=1.0, height=0.5, dx=0.05, dt=1.0e-4)]
    bat = sps_gb300.Batch(probs)
    bat.upload_all()
    bat.step(5)
    bat.snapshot()
    bat.step(4)
    for r, prob in enumerate(probs):
        snap, step = bat.snapshot_wait(r)
        assert step == 5
        _same(bat.snapshot_view(r)[0], snap, prob.ntotal)
        one = _ctx(prob, _abi.SPS_PREC_FP64_PLAIN)
        one.step(5, 0.0)
        _same(snap, one.download(), prob.ntotal)
        one.close()
    bat.close()


def test_snapshot_without_upload_is_an_error(built_gpu):
    prob = cases.bui_like()
    ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", prob.params_copy())
    with pytest.raises(sps_gb300.SpsError):
        ctx.snapshot()
    ctx.upload_problem(prob)
    with pytest.raises(sps_gb300.SpsError):
        ctx.snapshot_wait()
    ctx.close()


def test_snapshot_to_writer(built_gpu, tmp_path):
    """The output loop of the reference's driver: OutputMesh once, then OutputRes from a
    snapshot every few steps while the next steps run."""
    prob = cases.bui_like()
    ctx = _ctx(prob, _abi.SPS_PREC_FP64_PLAIN)
    prob.write_mesh(tmp_path)
    t, pending = 0.0, None
    for k in range(3):
        t_next = ctx.step(4, t)
        if pending is not None:
            f, step = ctx.snapshot_wait()
            prob.write_output(tmp_path, step, pending, f, hsml=prob.hsml)
        ctx.snapshot()
        pending, t = t_next, t_next
    f, step = ctx.snapshot_wait()
    prob.write_output(tmp_path, step, pending, f, hsml=prob.hsml)
    for s in (4, 8, 12):
        assert (tmp_path / ("nodes.csv.%06d" % s)).exists()
    res = (tmp_path / (prob.name + ".post.res")).read_text()
    assert res.count('Result "vel"') == 3
    ctx.close()


def test_surface_every_step_matches(built_gpu):
    """Downloads with the free surface after every step (the context then writes the list
    keys during the steps) give the same fields as one download at the end."""
    prob = cases.bui_like()
    a, b = _ctx(prob, _abi.SPS_PREC_FP64_PLAIN), _ctx(prob, _abi.SPS_PREC_FP64_PLAIN)
    t = 0.0
    for _ in range(6):
        t = a.step(1, t)
        fa = a.download()
    b.step(6, 0.0)
    _same(fa, b.download(), prob.ntotal)
    (na, sa), (nb, sb) = a.download_surface(), b.download_surface()
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(na, nb)
    a.close()
    b.close()
