"""The host-side reader / particle generator (CPU only).

Every input set of the reference's examples must parse, and the generated counts, masses
and dummy layout must follow the reference's formulas
(example_problems/soil_failure_bui_et_al_2008/3_SPH_material_2018.f90:431-461, :682-733,
:795-879).  The example inputs are the copies under tests/golden/example_problems.
"""
import math

import numpy as np
import pytest

import cases
import examples
import orc
import sps_gb300


@pytest.mark.parametrize("rel", examples.example_sets())
def test_reference_inputs_parse(built, rel):
    p = examples.load(rel)
    par = p.params
    assert par.nnode > 0 and p.ntotal2 >= p.ntotal
    assert len(p.blocks) >= 1 and p.blocks[0]["dt"] > 0
    # the source copy's constants: the Drucker-Prager copy's header carries ntype_solid,
    # the others' (code/, strain localisation, vertical cut) do not and are plane strain
    if rel.startswith("soil_failure"):
        assert par.cspm_det_min == float(np.float32(1e-7)) and par.bc_nodes_only == 0
    else:
        assert par.ntype_solid == 2
        assert par.cspm_det_min == float(np.float32(1e-3)) and par.bc_nodes_only == 1


def test_example_sets_present():
    sets = examples.example_sets()
    assert len(sets) == 16
    for fam in ("soil_failure_bui_et_al_2008", "strain_localisation_in_soil_sample",
                "vertical_slope"):
        assert any(s.startswith(fam) for s in sets)


@pytest.mark.parametrize("rel", examples.example_sets())
def test_reference_inputs_step_on_oracle(built, rel):
    # two steps of every set on the oracle with its copy's constants: the set-up path and
    # the options each set turns on (BCs, CSPM, viscoplasticity, outside approach, standard
    # SPH) run and keep the state finite
    p = examples.load(rel)
    o = orc.context(p.params_copy(**examples.overrides(rel)))
    o.upload_problem(p)
    o.step(2, 0.0)
    f = o.download()
    assert np.isfinite(f["x"]).all() and np.isfinite(f["vel"]).all()
    assert np.isfinite(f["stress"][:4 * p.ntotal]).all()
    o.close()


def test_own_steps_follow_the_driver_loop(built):
    # code/1_SPH_2018.f90:72-88: up to maxtimestep steps, leaving after the step whose FP64
    # time first exceeds time_end
    lengths = {r: examples.own_steps(examples.load(r)) for r in examples.example_sets()}
    assert lengths["soil_failure_bui_et_al_2008/inside_approach/SP1"] == 10
    assert lengths["strain_localisation_in_soil_sample/SP1"] == 2101
    assert lengths["vertical_slope/SP1"] == 2001
    assert lengths["soil_failure_bui_et_al_2008/standard_sph"] == 16667


def test_bui_counts_and_masses(built):
    # the Drucker-Prager example's layout: 4 x 2 m block at dx 0.1, inside approach
    p = cases.bui_like()
    ndivx, ndivy = int(4.0 / 0.1 + 1.0), int(2.0 / 0.1 + 1.0)
    assert p.nnode == ndivx * ndivy == 861
    assert p.nstress == (ndivx - 1) * (ndivy - 1) == 800
    # walls: LHS (-0.1 .. 2.1) and floor (-0.3 .. 9) at FP32 spacing, three rows each
    f = np.float32
    nd = int((f(2.1) - f(-0.1)) / f(0.1) + f(1.0)) + int((f(9.0) - f(-0.3)) / f(0.1) + f(1.0))
    assert p.params.ndummy2 == nd and p.params.ndummy == 3 * nd
    rho, dx = 1850.0, 0.1
    area = ((rho * dx) * dx) / 8.0
    m = p.mass
    X = p.x.reshape(-1, 2)
    nn = p.nnode
    corner = [k for k in range(nn) if X[k, 0] in (0.0, 4.0) and X[k, 1] in (0.0, 2.0)]
    assert all(m[k] == 2 * area for k in corner)
    interior = (X[:nn, 0] > 0) & (X[:nn, 0] < 4.0) & (X[:nn, 1] < 2.0)
    assert np.all(m[:nn][interior] == 8 * area)  # bottom row counts as interior (:522-526)
    assert np.all(m[nn:p.ntotal] == 8 * area)
    # stress-points at the cell centres, offset by dx/2 in both directions (:567-568)
    Xs = X[nn:p.ntotal]
    assert np.allclose(Xs[:, 0] % dx, dx / 2) and np.allclose(Xs[:, 1] % dx, dx / 2)
    # dummy coordinates are FP32 values and masses FP32 dx^2 * rho
    Xd = X[p.ntotal:]
    assert np.all(Xd == Xd.astype(np.float32).astype(np.float64))
    assert np.all(m[p.ntotal:] == float(np.float32(dx) * np.float32(dx)) * rho)
    # the innermost layer comes first and carries its wall's position
    wp = p.wall_position[p.ntotal:p.ntotal + p.params.ndummy2]
    assert np.all(wp == np.float32(-0.1))


def test_elastic_constants(built):
    p = cases.bui_like()
    E, nu = 1.8e6, 0.3
    K = E / (3 * (1 - 2 * nu))
    G = E / (2 * (1 + nu))
    assert p.params.D11 == float(np.float32(4.0) / np.float32(3.0)) * G + K
    assert p.params.D12 == -(float(np.float32(2.0) / np.float32(3.0)) * G) + K
    assert p.params.D33 == G
    assert p.params.pi == float(np.float32(math.pi))


def test_boundary_condition_tables(built):
    p = cases.bc_case()
    par = p.params
    assert par.no_bcs == 6
    bl = np.ctypeslib.as_array(par.bc_list, shape=(8 * par.no_bcs,)).reshape(-1, 8)
    twopi = np.float32(np.float32(math.acos(0.0)) * np.float32(4.0)) / np.float32(360.0)
    assert bl[2, 6] == 30.0 * float(twopi)
    info = p.bc_info.reshape(-1, 8)
    X = p.x.reshape(-1, 2)
    left = np.nonzero(X[:p.ntotal, 0] == 0.0)[0]
    assert np.all(p.bc_or_not[left] == 1)
    assert np.all(info[left, 1] >= 2)
    # the nodal BC lands in the row of its variable (bc_var + 2)
    node = 2 * (int(round(1.0 / 0.05)) + 1) + 5 - 1
    assert info[node, 3] == 6 and p.bc_or_not[node] == 1


def test_conflicting_nodal_bc_is_an_error(built):
    inp, dat, pts = _bc_texts()
    bad = dat.replace("nber of nodes with BCs\n0", "nber of nodes with BCs\n2\nnode bc\n1 1\n1 4")
    with pytest.raises(ValueError):
        sps_gb300.Problem.from_text(inp, bad, pts)


def _bc_texts():
    pts = "geom_type\n1\nx\n0 0.2 0 0.2 0.05\ny\n0 0 0.2 0.2 0.05\ndummy\nF\n"
    dat = ("1\nt\nndimn\n2\nh\n2 4 1\nm\n1 1 12 1e7 0.3 1. 2000 1 0 0 1 1 1\nt\n0.5 0 0 0 0 0 0 0\n"
           "ic\n0\nBC\n4 0\nbc\n1 5 1 0 0 0 0 0\n2 6 1 0 0 0 0 0\n3 1 1 0 0 0 0 0\n4 5 1 1 0 0 0 0\n"
           "seg\n0\nnber of nodes with BCs\n0\nic_tcurve\n1\nn\n1 10\np\n2\nt\n0 1\n1 1\n"
           "dom\n-1 -1 1 1\nIC\n2\na\n0\nb\n0\nc\n0\nd\n0\ne\n0\nf\n0\nflags\n2 2 1 1 F T F\n"
           "d\nF F\ndamp\n0\nab\n0 0\ng\n0\no\nx\n1 1 1 1 1 1 1 0 0 0\n")
    inp = ("p\nt\nf\nT F F\ni\nT\nn\n1\ns\n1.2\nt\n1e-5,1,10\np\n1,1,1\ne\n-1,1,1\n")
    return inp, dat, pts


def test_reader_errors(built):
    inp, dat, pts = _bc_texts()
    with pytest.raises(ValueError):
        sps_gb300.Problem.from_text(inp, dat[:200], pts)  # truncated .dat
    with pytest.raises(ValueError):
        sps_gb300.Problem.from_text(inp, dat.replace("2 2 1 1 F T F", "2 2 1 x F T F"), pts)


def test_column_k0(built):
    p = cases.column(dx=0.004)
    st = p.stress.reshape(-1, 4)[:p.ntotal]
    X = p.x.reshape(-1, 2)[:p.ntotal]
    depth = np.maximum(0.10 - X[:, 1], 0)
    assert np.allclose(st[:, 1], -2650 * 9.81 * depth)
    assert np.allclose(st[:, 0], 0.5 * st[:, 1]) and np.all(st[:, 2] == 0)


def test_slope_generator(built):
    # extents are snapped to the lattice; these are multiples of dx
    p = sps_gb300.Problem.slope(Lf=2.0, Hf=0.5, Ls=0.45, Hs=1.0, dx=0.05)
    X = p.x.reshape(-1, 2)
    nn = p.nnode
    # the slope block sits on the foundation with a vertical face at x = Ls
    above = X[:nn, 1] > 0.5 + 1e-9
    assert np.all(X[:nn][above, 0] <= 0.45 + 1e-9) and above.any()
    # total mass equals rho * area (each node a quarter cell per adjacent cell)
    area = 2.0 * 0.5 + 0.45 * 1.0
    assert abs(p.mass[:nn].sum() - 1850.0 * area) < 1e-6 * 1850 * area
    assert abs(p.mass[nn:p.ntotal].sum() - 1850.0 * area) < 1e-6 * 1850 * area


def test_biaxial_generator(built):
    # 0.05 x 0.10 m at 2 mm: 26 x 51 nodes, 25 x 50 stress-points, no dummies
    p = sps_gb300.Problem.biaxial(dx=0.002, confining=50e3, q_ratio=0.5, phi_deg=35.0,
                                  cohesion=2e3)
    assert (p.nnode, p.nstress, p.ntotal2) == (26 * 51, 25 * 50, 26 * 51 + 25 * 50)
    nn = p.nnode
    X = p.x.reshape(-1, 2)[:p.ntotal]
    bi = p.bc_info.reshape(-1, 8)[:p.ntotal]
    top, bot = X[:, 1] == X[:nn, 1].max(), X[:, 1] == 0.0
    side = (X[:, 0] == 0.0) | (X[:, 0] == X[:nn, 0].max())
    # the segments catch exactly the outer node rows and columns (stress-points sit inside)
    assert np.array_equal(p.bc_or_not[:p.ntotal] == 1, top | bot | side)
    assert not (top | bot | side)[nn:].any()
    bcs = lambda m: {frozenset(r[2:2 + r[1]]) for r in bi[m]}
    assert bcs(top & ~side) == {frozenset({1, 2})} and bcs(bot & ~side) == {frozenset({1, 3})}
    assert bcs(side & ~top & ~bot) == {frozenset({4, 5})}
    assert bcs(top & side) == {frozenset({1, 2, 4, 5})}
    bl = np.asarray(p.params.bc_list[0:40]).reshape(5, 8)
    # (var, time curve, a1): vx = 0 and vy = -/+ v on the platens, sxx = -p and sxy = 0
    assert [tuple(r[1:4]) for r in bl] == [(5, 1, 0), (6, 1, -0.05), (6, 1, 0.05),
                                           (1, 2, -50e3), (3, 2, 0)]
    # initial stress: half way (in axial excess) from the confining state to the cone
    st = p.stress.reshape(-1, 4)[:p.ntotal]
    t = math.tan(math.radians(35.0))
    root = math.sqrt(9 + 12 * t * t)
    alpha, kc = t / root, 3 * 2e3 / root
    s = st[0]
    mean = (s[0] + s[1] + s[3]) / 3
    j2 = 0.5 * ((s[0] - mean) ** 2 + (s[1] - mean) ** 2 + (s[3] - mean) ** 2) + s[2] ** 2
    f = math.sqrt(j2) + alpha * 3 * mean - kc
    assert abs(f - (-0.5) * (3 * alpha * 50e3 + kc)) < 1e-6 * 50e3
    assert np.all(st == st[0])
