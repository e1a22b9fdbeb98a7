"""CPU pins of the oracle's get_nodes_on_free_surface (3_SPH_material_2018.f90:1135-1430).

A rectangular block on a floor with a left wall, one step from rest: the top and right
faces are free surface with outward unit normals, the interior and the particles next to
the walls are not, and the bc_or_not update marks exactly the surface particles with 2.
The reference's refined normal sums the perpendiculars of x_j - x_i over surface pairs
with the pair's own orientation, so on a flat face it leans by up to ~20 degrees; the
checks pin the outward direction, not the exact angle.
"""
import numpy as np

import cases
import orc


def test_block_surface(built):
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05)
    o = orc.context(p.params_copy())
    o.upload_problem(p)
    o.step(1, 0.0)
    normal, subset = o.download_surface()
    f = o.download()
    nt, nn = p.ntotal, p.nnode
    x = f["x"][:2 * nt].reshape(-1, 2)
    n = normal.reshape(-1, 2)
    dx = 0.05
    xs, ys = x[:nn, 0], x[:nn, 1]
    x0, x1, y0, y1 = xs.min(), xs.max(), ys.min(), ys.max()
    tol = 1e-3
    top = (np.abs(ys - y1) < tol) & (xs > x0 + 2 * dx) & (xs < x1 - 2 * dx)
    right = (np.abs(xs - x1) < tol) & (ys > y0 + 2 * dx) & (ys < y1 - 2 * dx)
    inner = (xs > x0 + 3 * dx) & (xs < x1 - 3 * dx) & (ys > y0 + 3 * dx) & (ys < y1 - 3 * dx)
    near_wall = (np.abs(ys - y0) < tol) & (xs > x0 + 2 * dx) & (xs < x1 - 2 * dx)
    assert top.sum() > 5 and right.sum() > 3 and inner.sum() > 10
    assert (subset[:nn][top] == 1).all() and (n[:nn][top][:, 1] > 0.8).all()
    assert (subset[:nn][right] == 1).all() and (n[:nn][right][:, 0] > 0.8).all()
    assert (subset[:nn][inner] == 2).all() and (n[:nn][inner] == 0).all()
    assert (subset[:nn][near_wall] == 2).all()
    on = subset == 1
    np.testing.assert_allclose(np.hypot(n[on, 0], n[on, 1]), 1.0, atol=1e-6)
    assert ((f["bc_or_not"] == 2) == on).all()
