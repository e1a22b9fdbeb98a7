"""The oracle's outside approach (shift_stress_points and isolated_nodes,
2_SPH_main_2018.f90:244-398; the re-interpolation after a shift, :99-108): stress-points
attached to their nodes, placed again every shift_update steps."""
import numpy as np
import pytest

import cases
import orc

OUT = dict(sph_shift=True, vel_vector=False, shift_update=1, rx=1 / 3, ry=1 / 3, disp_tol=0.125)


def _run(p, nsteps):
    ctx = orc.context(p.params_copy())
    ctx.upload_problem(p)
    ctx.step(nsteps, 0.0)
    f = ctx.download()
    ctx.close()
    return f


def _offsets(p, f):
    nn, np_ = p.nnode, p.params.npoints
    x = f["x"].reshape(-1, 2)
    node = x[:nn]
    sp = x[nn:p.ntotal].reshape(nn, np_, 2)
    return sp - node[:, None, :], x


@pytest.mark.parametrize("npoints", [1, 2, 3])
def test_fixed_offsets_after_shift(npoints):
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, outside=OUT, npoints=npoints)
    assert p.params.npoints == npoints and p.nstress == npoints * p.nnode
    f = _run(p, 3)
    off, _ = _offsets(p, f)
    rx = ry = 0.05 / 3
    want = {1: [(rx, ry)], 2: [(rx, ry), (-rx, -rx)], 3: [(0, ry), (-rx, -ry), (rx, -ry)]}[npoints]
    on_node = np.all(np.abs(off) < 1e-12, axis=(1, 2))
    # nodes next to a wall moving fast, or with fewer than two node neighbours, hold their
    # stress-points; the rest carry the fixed offsets
    assert (~on_node).sum() > 0.5 * p.nnode
    np.testing.assert_allclose(off[~on_node], np.broadcast_to(want, off[~on_node].shape),
                               rtol=0, atol=1e-12)


def test_shift_every_other_step():
    o = dict(OUT, shift_update=2)
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, outside=o, npoints=1, xsph=False)
    f1 = _run(p, 1)  # itimestep 1: no shift, the points moved with their own velocity
    off1, _ = _offsets(p, f1)
    f2 = _run(p, 2)  # itimestep 2: shifted
    off2, _ = _offsets(p, f2)
    rx = 0.05 / 3
    moved = ~np.all(np.abs(off2) < 1e-12, axis=(1, 2))
    np.testing.assert_allclose(off2[moved][:, 0], np.full((moved.sum(), 2), [rx, rx]), atol=1e-12)
    assert np.abs(off1[moved][:, 0] - [rx, rx]).max() > 1e-12


def test_velocity_vector_points_along_velocity():
    o = dict(OUT, vel_vector=True, disp_tol=0.0)
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, outside=o, npoints=2)
    assert p.params.npoints == 2 and p.params.vel_vector == 1
    f = _run(p, 4)
    off, _ = _offsets(p, f)
    v = f["vel"].reshape(-1, 2)[:p.nnode]
    moved = ~np.all(np.abs(off) < 1e-12, axis=(1, 2)) & (np.hypot(v[:, 0], v[:, 1]) > 0)
    assert moved.sum() > 0
    # the two points are symmetric about the node, and (apart from the minimum offsets
    # dx/3 added to small components) lie along the velocity
    np.testing.assert_allclose(off[moved][:, 0], -off[moved][:, 1], atol=1e-12)
    dot = off[moved][:, 0, 0] * v[moved][:, 0] + off[moved][:, 0, 1] * v[moved][:, 1]
    assert (dot > 0).all()
