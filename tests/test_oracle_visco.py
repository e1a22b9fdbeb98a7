"""The oracle's viscoplastic laws (plastic_terms with ncrit 1-4: Get_Vivel, invar09, yieldf09,
flowvp09, Get_Dmatx; 3_SPH_material_2018.f90:2165-2691) against their published forms:
Perzyna overstress flow g(F) df/dsigma with the Tresca, von Mises, Mohr-Coulomb and
Drucker-Prager yield functions in the Owen-Hinton invariant form, written here
independently in numpy."""
import ctypes as C
import math

import numpy as np
import pytest

import orc

ROOT3 = float(np.sqrt(np.float32(3.0)))  # the reference's sqrt(3.00) is an FP32 root
RAD = float(np.float32(0.017453292))


def props(ncrit, E=8e7, nu=0.25, Y=1.5e4, H=-8e5, phi=30.0, gamma=0.5, delta=1.0, n=1):
    p = np.zeros(20)
    p[:12] = [2, ncrit, E, nu, 1.0, 2000.0, Y, H, phi, gamma, delta, n]
    return p


def call(p, s, iv1=0.0, ntype_solid=2):
    v, g = np.zeros(4), np.zeros(4)
    P = C.POINTER(C.c_double)
    s = np.ascontiguousarray(s, dtype=np.float64)
    orc.lib().orc_viscoplastic(p.ctypes.data_as(P), ntype_solid, s.ctypes.data_as(P), iv1,
                               v.ctypes.data_as(P), g.ctypes.data_as(P))
    return v, g


def model(p, s, iv1=0.0, ntype_solid=2):
    """Published form: vivel = gamma phi(F/F0 - 1) dF/dsigma for F > F0 (and F/F0 - 1 >= 0.01)."""
    ncrit, E, nu, Y, H, phi, gamma, delta, n = (int(p[1]), p[2], p[3], p[6], p[7], p[8], p[9],
                                                  p[10], p[11])
    sm = (s[0] + s[1] + s[3]) / 3.0
    d = np.array([s[0] - sm, s[1] - sm, s[2], s[3] - sm])
    J2 = d[2] ** 2 + 0.5 * (d[0] ** 2 + d[1] ** 2 + d[3] ** 2)
    J3 = d[3] * (d[3] ** 2 - J2)
    se = math.sqrt(J2)
    st3 = 0.0 if se == 0 else max(-1.0, min(1.0, -3.0 * ROOT3 * J3 / (2.0 * J2 * se)))
    th = math.asin(st3) / 3.0
    sphi = math.sin(phi * RAD)
    F = {1: 2.0 * math.cos(th) * se, 2: ROOT3 * se,
         3: sm * sphi + se * (math.cos(th) - math.sin(th) * sphi / ROOT3),
         4: 6.0 * sm * sphi / (ROOT3 * (3.0 - sphi)) + se}[ncrit]
    F0 = Y * max(abs(Y + H * iv1) / abs(Y), float(np.float32(0.1)))
    v = np.zeros(4)
    if F > F0 and (F - F0) / F0 >= float(np.float32(0.01)):
        fn = (F - F0) / F0
        c = gamma * (fn ** delta if n == 1 else math.exp(delta * fn) - 1.0)
        a1 = np.array([1.0, 1.0, 0.0, 1.0])
        a2 = np.array([d[0], d[1], 2.0 * d[2], d[3]]) / (2.0 * se)
        a3 = np.array([d[1] * d[3] + J2 / 3, d[0] * d[3] + J2 / 3, -2 * d[2] * d[3],
                       d[0] * d[1] - d[2] ** 2 + J2 / 3])
        deg = abs(math.degrees(th))
        if ncrit == 1:
            c1, c2, c3 = (0.0, ROOT3, 0.0) if deg >= 29.0 else (
                0.0, 2 * math.cos(th) * (1 + math.tan(th) * math.tan(3 * th)),
                ROOT3 * math.sin(th) / (J2 * math.cos(3 * th)))
        elif ncrit == 2:
            c1, c2, c3 = 0.0, ROOT3, 0.0
        elif ncrit == 3:
            c1 = sphi / 3.0
            if deg >= 29.0:
                c2, c3 = 0.5 * ROOT3 * (1 - math.copysign(1.0, th) * c1), 0.0
            else:
                c2 = math.cos(th) * ((1 + math.tan(th) * math.tan(3 * th)) +
                                     c1 * (math.tan(3 * th) - math.tan(th)) * ROOT3)
                c3 = (ROOT3 * math.sin(th) + 3 * c1 * math.cos(th)) / (2 * J2 * math.cos(3 * th))
        else:
            c1, c2, c3 = 2 * sphi / (ROOT3 * (3 - sphi)), 1.0, 0.0
        v = c * (c1 * a1 + c2 * a2 + c3 * a3)
    if ntype_solid == 1:
        k = E / (1 - nu * nu)
        D = np.array([[k, k * nu, 0, 0], [k * nu, k, 0, 0], [0, 0, (1 - nu) * k / 2, 0],
                      [0, 0, 0, 0]])
    else:
        k = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
        q = k * nu / (1 - nu)
        D = np.array([[k, q, 0, q], [q, k, 0, q], [0, 0, (1 - 2 * nu) * k / (2 * (1 - nu)), 0],
                      [q, q, 0, k]])
    return v, -D @ v


def stresses(seed, n, scale=4e4):
    rng = np.random.default_rng(seed)
    s = rng.normal(0.0, scale, size=(n, 4))
    s[:, :2] -= scale  # mostly compressive, like the biaxial sample
    s[:, 3] = 0.25 * (s[:, 0] + s[:, 1])
    return s


@pytest.mark.parametrize("ncrit", [1, 2, 3, 4])
@pytest.mark.parametrize("flow", [dict(n=1, delta=1.0), dict(n=2, delta=1.5),
                                  dict(n=1, delta=2.0)], ids=["linear", "exp", "power"])
def test_law_matches_published_form(ncrit, flow):
    p = props(ncrit, **flow)
    for s in stresses(100 + ncrit, 400):
        for iv in (0.0, 3e-3, 0.5):  # hardening state, down to the 0.1 floor
            v, g = call(p, s, iv)
            vm, gm = model(p, s, iv)
            np.testing.assert_allclose(v, vm, rtol=1e-9, atol=1e-12 * (np.abs(vm).max() + 1))
            np.testing.assert_allclose(g, gm, rtol=1e-9, atol=1e-9 * (np.abs(gm).max() + 1))


def test_below_yield_is_elastic():
    p = props(2, Y=1e9)
    v, g = call(p, np.array([-1e4, -2e4, 3e3, -7.5e3]))
    assert not v.any() and not g.any()


def test_von_mises_flow_is_deviatoric_and_drucker_prager_dilates():
    s = np.array([-4e4, -1e4, 8e3, -1.25e4])
    v, _ = call(props(2), s)
    assert np.abs(v).max() > 0
    assert abs(v[0] + v[1] + v[3]) <= 1e-12 * np.abs(v).max()
    v4, _ = call(props(4), s)
    sphi = math.sin(30.0 * RAD)
    cons1 = 2 * sphi / (ROOT3 * (3 - sphi))
    # the volumetric rate is 3 cons1 times the Perzyna multiplier
    mult = v4[2] / (s[2] / math.sqrt(s[2] ** 2 + 0.5 * sum(
        (x - (s[0] + s[1] + s[3]) / 3) ** 2 for x in (s[0], s[1], s[3]))))
    np.testing.assert_allclose(v4[0] + v4[1] + v4[3], 3 * cons1 * mult, rtol=1e-12)


def test_plane_stress_matrix():
    s = np.array([-4e4, -1e4, 8e3, 0.0])
    s[3] = 0.25 * (s[0] + s[1])
    p = props(2)
    v, g = call(p, s, ntype_solid=1)
    vm, gm = model(p, s, ntype_solid=1)
    np.testing.assert_allclose(g, gm, rtol=1e-12)
    assert g[3] == 0.0


def test_softening_floor():
    # strong softening: the yield-surface size stops at a tenth of the initial one
    p = props(2, H=-1e9)
    s = np.array([-4e4, -1e4, 8e3, -1.25e4])
    v1, _ = call(p, s, 1.0)
    v2, _ = call(p, s, 10.0)
    np.testing.assert_array_equal(v1, v2)
