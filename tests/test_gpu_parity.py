"""GPU parity: the CUDA FP64 plain path against the CPU oracle, through the C-ABI.

The plain path sums every neighbour term in the reference's linked-list walk order and
repeats its FP32 roundings, so it must equal the oracle bit for bit (tolerance 0) on every
downloaded field, step after step.
"""
import numpy as np
import pytest

import cases
import orc
import sps_gb300
from sps_gb300 import _abi

pytestmark = pytest.mark.gpu


def _gpu_ctx(problem, **over):
    p = problem.params_copy(precision=_abi.SPS_PREC_FP64_PLAIN, **over)
    return sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", p)


def _orc_ctx(problem, **over):
    return orc.context(problem.params_copy(**over))


def _compare(problem, nsteps, chunks=None, pairs=True, **over):
    g = _gpu_ctx(problem, **over)
    o = _orc_ctx(problem, **over)
    tg, to = cases.run_pair(problem, nsteps, [g, o], chunks)
    assert tg == to
    if pairs:
        pg, po = g.dump_pairs(), o.dump_pairs()
        for k in ("pair_i", "pair_j", "pint_type"):
            np.testing.assert_array_equal(pg[k], po[k], err_msg=k)
        for k in ("w", "dwdx", "dwdy"):
            np.testing.assert_array_equal(pg[k].view(np.int32), po[k].view(np.int32), err_msg=k)
    fg, fo = g.download(), o.download()
    cases.assert_bitwise(fg, fo, problem.ntotal)
    np.testing.assert_array_equal(fg["bc_or_not"], fo["bc_or_not"])
    (ng, sg), (no, so) = g.download_surface(), o.download_surface()
    np.testing.assert_array_equal(sg, so, err_msg="subset")
    same = (ng.view(np.int64) == no.view(np.int64)) | (np.isnan(ng) & np.isnan(no))
    assert same.all(), ("surface normal", np.nonzero(~same)[0][:10])
    return fg


def test_pairs_first_step(built_gpu):
    p = cases.bui_like()
    _compare(p, 1)


def test_bui_like_steps(built_gpu):
    # cohesive Drucker-Prager block, XSPH, artificial viscosity, wall dummies
    p = cases.bui_like()
    f = _compare(p, 10, chunks=[1, 2, 7])
    assert np.isfinite(f["stress"]).all()


def test_bui_like_finer_trapezoid(built_gpu):
    p = cases.bui_like(width=1.0, height=0.5, dx=0.02, xsph=False, alpha=0.0, beta=0.0,
                       dt=4e-5)
    _compare(p, 25, chunks=[5, 20])


def test_column_k0(built_gpu):
    # granular column with a K0 stress state (plastic from the first return on)
    p = cases.column(dx=0.004)
    _compare(p, 30, chunks=[10, 20])


def test_leaving_the_domain(built_gpu):
    # Check_Out_Domain (2_SPH_main_2018.f90:1186-1192): the block moves right at 1 m/s and
    # its right-hand columns cross xmax = 1.0005 m within the run; a particle that leaves
    # is excluded from the cell grid and the pair search for good (the floor ends under
    # the block, so no wall particle starts outside)
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, dt=5e-5, floor_to=1.0,
                       domain=(-10, -10, 1.0005, 41))
    p.vel[0:2 * p.ntotal:2] = 1.0
    f = _compare(p, 30, chunks=[10, 20])
    x = f["x"].reshape(-1, 2)[:p.ntotal, 0]
    assert (x > 1.0005).sum() >= 10  # the right-hand column of nodes left


def test_damping_and_ramped_gravity(built_gpu):
    # gravity_force (3_SPH_material_2018.f90:2809-2870) with DampingTG = 50 and the gravity
    # factor ramped from 0 to 1 over 10 ms by its time curve, on the plastic block
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, dt=5e-5, damping=50.0,
                       gravity_curve=((0, 0.01, 500), (0, 1, 1)))
    f = _compare(p, 40, chunks=[15, 25])
    q = cases.bui_like(width=1.0, height=0.5, dx=0.05, dt=5e-5)
    o = _orc_ctx(q)
    o.upload_problem(q)
    o.step(40, 0.0)
    assert not np.array_equal(o.download()["vel"], f["vel"])  # the terms act


def test_cspm_cont_density(built_gpu):
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, cspm=True, cont_density=True, sle=2,
                       dt=5e-5)
    _compare(p, 12, chunks=[4, 8])


def test_plane_stress_quintic(built_gpu):
    p = cases.bui_like(width=1.0, height=0.6, dx=0.05, skf=3, ntype_solid=1, dt=5e-5)
    _compare(p, 8)


def test_boundary_conditions(built_gpu):
    p = cases.bc_case()
    _compare(p, 20, chunks=[7, 13])
    p = cases.bc_case(plastic=True, cspm=False, xsph=True)
    _compare(p, 20, chunks=[20])


def test_biaxial_platens(built_gpu):
    # biaxial sample: rough platens driven by ramped segment velocity BCs, side stress BCs,
    # cohesionless Drucker-Prager (plastic near the platens within the run)
    p = sps_gb300.Problem.biaxial(dx=0.002, platen_v=0.5, t_ramp=2e-5)
    f = _compare(p, 40, chunks=[15, 25])
    assert (f["intvars1"] > 0).any()


def test_stress_free_surface(built_gpu):
    # ifsigman = 1: free-surface nodes away from the walls get zero normal and shear
    # traction after every BC application (apply_stress_free)
    p = cases.bc_case(plastic=True, cspm=False, xsph=True)
    f = _compare(p, 20, chunks=[5, 15], ifsigman=1)
    assert (f["bc_or_not"] == 2).any()


def _visco(ncrit, **kw):
    # an initial deviatoric stress above the yield surface of each law, a Perzyna fluidity
    # small enough for the explicit step to stay stable, and softening as in the
    # strain-localisation example
    base = dict(plastic=True, cspm=False, ncrit=ncrit, hards=-8e5, phi_deg=30.0, gamma=0.5,
                delta=1.0, nflow=1, yield_stress={1: 1.5e4, 2: 1.5e4, 3: 1e3, 4: 1e3}[ncrit])
    base.update(kw)
    p = cases.bc_case(**base)
    p.stress[:4 * p.ntotal] = np.tile([-4e4, -1e4, 5e3, -1.25e4], p.ntotal)  # initial stress
    return p


@pytest.mark.parametrize("ncrit", [2, 4])
def test_viscoplastic_bitwise(built_gpu, ncrit):
    # von Mises and Drucker-Prager viscoplasticity with Perzyna n = 1, delta = 1: no
    # transcendental function is evaluated, so the path is bit-exact
    p = _visco(ncrit)
    f = _compare(p, 20, chunks=[6, 14])
    o = _orc_ctx(p)
    o.upload_problem(p)
    o.step(20, 0.0)
    assert (o.download()["intvars1"][p.nnode:] > 0).any()  # plastic flow took place


def _close(problem, nsteps, rtol):
    g = _gpu_ctx(problem)
    o = _orc_ctx(problem)
    cases.run_pair(problem, nsteps, [g, o])
    fg, fo = g.download(), o.download()
    for k in ("x", "vel", "stress", "intvars1"):
        a, b = fg[k], fo[k]
        if k == "stress":
            a, b = a[:4 * problem.ntotal], b[:4 * problem.ntotal]
        scale = np.abs(b).max() + 1e-300
        assert np.abs(a - b).max() <= rtol * scale, (k, np.abs(a - b).max() / scale)
    return fo


@pytest.mark.parametrize("ncrit,extra", [(1, {}), (3, {}), (2, dict(nflow=2, delta=1.5)),
                                         (4, dict(delta=2.0))],
                         ids=["tresca", "mohr_coulomb", "vm_exp_flow", "dp_power_flow"])
def test_viscoplastic_close(built_gpu, ncrit, extra):
    # Tresca and Mohr-Coulomb read the Lode angle through asin, sin, cos and tan, and the
    # other Perzyna forms call exp or pow: CUDA's and the host libm's results may differ in
    # the last bit, so these are compared with a relative tolerance of 1e-9
    p = _visco(ncrit, **extra)
    fo = _close(p, 20, 1e-9)
    assert (fo["intvars1"][p.nnode:] > 0).any()


def _tensile(**kw):
    # a cohesive block with a tensile initial stress (admissible: below the tension-cut
    # apex), so that the nodes' principal tensile stresses drive the artificial force
    p = cases.bui_like(art_stress=True, **kw)
    p.stress[:4 * p.ntotal] = np.tile([2e3, -1e3, 5e2, 3e2], p.ntotal)
    return p


@pytest.mark.parametrize("precision", ["plain", "fp32"])
def test_artificial_stress_close(built_gpu, precision):
    # artificial_force calls atan, cos, sin and pow: CUDA's and the host libm's results may
    # differ in the last bit, so the plain path is compared at 1e-10 relative; the FP32
    # form at its own accuracy
    p = _tensile()
    if precision == "plain":
        fo = _close(p, 12, 1e-10)
    else:
        g = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                  p.params_copy(precision=_abi.SPS_PREC_FP32_FAST))
        o = _orc_ctx(p)
        cases.run_pair(p, 12, [g, o])
        fg, fo = g.download(), o.download()
        for k in ("x", "vel"):
            scale = np.abs(fo[k]).max() + 1e-300
            assert np.abs(fg[k] - fo[k]).max() <= 1e-4 * scale, k
    # the force acts: the run differs from the same run without it
    q = cases.bui_like()
    q.stress[:4 * q.ntotal] = p.stress[:4 * p.ntotal]
    o2 = _orc_ctx(q)
    o2.upload_problem(q)
    o2.step(12, 0.0)
    assert not np.array_equal(o2.download()["vel"], fo["vel"])


OUTSIDE = dict(sph_shift=True, vel_vector=False, shift_update=1, rx=1 / 3, ry=1 / 3,
               disp_tol=0.125)


@pytest.mark.parametrize("npoints,extra", [
    (1, {}), (2, {}), (3, {}), (2, dict(vel_vector=True, disp_tol=0.0)),
    (2, dict(vel_vector=True, disp_tol=0.5, shift_update=2)),
    (1, dict(sph_shift=False, shift_update=3))],
    ids=["np1", "np2", "np3", "vel_vector", "vel_vector_tol", "no_reinterp"])
def test_outside_approach(built_gpu, npoints, extra):
    # stress-points attached to their nodes and placed again every shift_update steps,
    # with the re-interpolation at the start of the following step (plain: bit-exact)
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, outside=dict(OUTSIDE, **extra),
                       npoints=npoints)
    _compare(p, 12, chunks=[5, 7])


def test_outside_approach_fp32(built_gpu):
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, outside=OUTSIDE, npoints=2)
    g = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                              p.params_copy(precision=_abi.SPS_PREC_FP32_FAST))
    o = _orc_ctx(p)
    cases.run_pair(p, 12, [g, o])
    fg, fo = g.download(), o.download()
    for k in ("x", "vel"):
        scale = np.abs(fo[k]).max() + 1e-300
        assert np.abs(fg[k] - fo[k]).max() <= 1e-4 * scale, k


def test_standard_sph(built_gpu):
    p = cases.standard_sph()
    _compare(p, 6)


def test_gauss_kernel_close(built_gpu):
    # skf = 2 calls exp(): CUDA's and the host libm's may differ in the last bit, so this
    # case is compared with a relative tolerance of 1e-10 instead of bitwise
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05, skf=2, dt=5e-5)
    g = _gpu_ctx(p)
    o = _orc_ctx(p)
    cases.run_pair(p, 5, [g, o])
    fg, fo = g.download(), o.download()
    for k in ("x", "vel", "stress"):
        a, b = fg[k], fo[k]
        if k == "stress":
            a, b = a[:4 * p.ntotal], b[:4 * p.ntotal]
        scale = np.abs(b).max() + 1e-300
        assert np.abs(a - b).max() <= 1e-10 * scale, k


def test_capacity_error(built_gpu):
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05)
    g = _gpu_ctx(p, max_neighbours=16)
    g.upload_problem(p)
    with pytest.raises(sps_gb300.SpsError) as e:
        g.step(1, 0.0)
    assert e.value.rc == _abi.SPS_ERR_CAPACITY


def test_unsupported_options(built_gpu):
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05)
    cam_clay = cases.bc_case(plastic=True, ncrit=5)
    with pytest.raises(sps_gb300.SpsError, match="Cam Clay"):
        _gpu_ctx(cam_clay)
    weak = _visco(2, yield_stress=1e-4)  # invar09 stops below 0.001
    with pytest.raises(sps_gb300.SpsError):
        _gpu_ctx(weak)
    for over in (dict(inside_approach=0), dict(skf=7)):  # inside_approach 0: no npoints
        with pytest.raises(sps_gb300.SpsError):
            _gpu_ctx(p, **over)


def test_step_before_upload(built_gpu):
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05)
    g = _gpu_ctx(p)
    with pytest.raises(sps_gb300.SpsError) as e:
        g.step(1, 0.0)
    assert e.value.rc == _abi.SPS_ERR_STATE


def test_corrected_division_matches_ieee(built_gpu):
    # the plain path divides by densities and smoothing lengths through exact reciprocals
    # (Markstein correction); it must reproduce the IEEE quotient bit for bit
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05)
    g = _gpu_ctx(p)
    assert sps_gb300.selftest_division(g, 200_000_000, seed=12345) == 0


def test_integer_pipe_conversions_match_hardware(built_gpu):
    # the FP32 form converts its records with integer operations on the bit patterns; they
    # must round exactly as the hardware conversions
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05)
    g = _gpu_ctx(p)
    assert sps_gb300.selftest_convert(g, 100_000_000, seed=777) == 0


def test_fp32_cone_certification_is_sound(built_gpu):
    # both forms skip the FP64 stress return for stresses that an FP32 evaluation with
    # error bounds certifies inside the cone; no certified stress may be one that either
    # FP64 return would change, including stresses within 1e-9 of the cone
    p = cases.bui_like(width=1.0, height=0.5, dx=0.05)
    g = _gpu_ctx(p)
    bad, certified = sps_gb300.selftest_cone(g, 100_000_000, seed=4242)
    assert bad == 0, bad
    assert certified > 30_000_000, certified  # most stresses are certified
