"""The oracle's artificial_force (2_SPH_main_2018.f90:908-1016, Monaghan's artificial stress
over node-node pairs): a pairwise-antisymmetric force (total momentum conserved) that vanishes
when no node carries a tensile principal stress."""
import ctypes as C

import numpy as np

import cases
import orc


def _force(prob):
    ctx = orc.context(prob.params_copy())
    ctx.upload_problem(prob)
    ctx.step(1, 0.0)  # builds the pair list
    out = np.zeros(2 * prob.nnode)
    orc.lib().orc_artificial_force(ctx._h, out.ctypes.data_as(C.POINTER(C.c_double)))
    s = ctx.download()
    ctx.close()
    return out.reshape(-1, 2), s


def _tensile(s0):
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, art_stress=True)
    p.stress[:4 * p.ntotal] = np.tile(s0, p.ntotal)
    return p


def test_momentum_conserved_and_nonzero():
    p = _tensile([2e3, -1e3, 5e2, 3e2])
    f, _ = _force(p)
    m = p.mass[:p.nnode]
    total = (m[:, None] * f).sum(axis=0)
    scale = (m[:, None] * np.abs(f)).sum(axis=0)
    assert (scale > 0).all()
    assert (np.abs(total) <= 1e-12 * scale).all()


def test_compressive_state_has_no_force():
    p = _tensile([-2e3, -1e3, 5e2, -1e3])
    f, s = _force(p)
    # still compressive after one step: both principal stresses negative at every node
    st = s["stress"][:4 * p.nnode].reshape(-1, 4)
    c, r = 0.5 * (st[:, 0] + st[:, 1]), np.hypot(0.5 * (st[:, 0] - st[:, 1]), st[:, 2])
    assert (c + r < 0).all()
    assert not f.any()
