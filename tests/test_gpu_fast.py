"""GPU: the FP32 form against the FP64 plain form (and the oracle) on the same inputs.

The FP32 form must keep the pair set bit-exact (same neighbour search) and stay within
stated relative errors of the FP64 plain path:
    stress   relative L2 <= 1e-4, relative Linf <= 1e-3
    velocity relative L2 <= 1e-4
    displacement relative L2 <= 1e-4
(relative L2 = ||a - b||_2 / ||b||_2 over nodes and stress-points; Linf relative to max|b|).
"""
import numpy as np
import pytest

import cases
import sps_gb300
from sps_gb300 import _abi

pytestmark = pytest.mark.gpu


def rel_errors(a, b):
    d = a - b
    l2 = np.linalg.norm(d) / max(np.linalg.norm(b), 1e-300)
    li = np.abs(d).max() / max(np.abs(b).max(), 1e-300)
    return l2, li


def run(problem, prec, nsteps, chunks=None):
    ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", problem.params_copy(precision=prec))
    ctx.upload_problem(problem)
    t = 0.0
    for c in chunks or [nsteps]:
        t = ctx.step(c, t)
    return ctx, t


def chaos_floor(problem, nsteps, rel=2.0 ** -24, seed=5):
    """Relative L2 stress difference between two FP64 plain runs whose initial stresses
    differ by a random relative perturbation of size `rel` (default: half an FP32 ulp, the
    rounding the FP32 form applies to every neighbour value): the sensitivity of the
    problem itself.  The Drucker-Prager loading test `f >= 0 and df >= 0` switches on
    rounding noise for particles on the yield surface, so plastic runs amplify any
    perturbation; no arithmetic that is not bit-exact can agree with the plain form
    more closely than this."""
    st = problem.state()
    rng = np.random.default_rng(seed)
    pert = st["stress"] * (1.0 + rel * rng.uniform(-1.0, 1.0, st["stress"].shape))
    out = []
    for s_ in (st["stress"], pert):
        ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                    problem.params_copy(precision=_abi.SPS_PREC_FP64_PLAIN))
        d = dict(st)
        d["stress"] = s_
        ctx.upload(**d)
        ctx.upload_bcs(problem.bc_or_not, problem.bc_info)
        ctx.step(nsteps, 0.0)
        out.append(ctx.download()["stress"][:4 * problem.ntotal])
    return rel_errors(out[1], out[0])[0]


def compare(problem, nsteps, tol_s=1e-4, tol_v=1e-4, tol_d=1e-4, tol_linf=1e-3):
    cf, tf = run(problem, _abi.SPS_PREC_FP32_FAST, nsteps)
    cp, tp = run(problem, _abi.SPS_PREC_FP64_PLAIN, nsteps)
    assert tf == tp
    ff, fp = cf.download(), cp.download()
    nt, nn = problem.ntotal, problem.nnode
    s_l2, s_li = rel_errors(ff["stress"][:4 * nt], fp["stress"][:4 * nt])
    v_l2, _ = rel_errors(ff["vel"][:2 * nt], fp["vel"][:2 * nt])
    d_l2, _ = rel_errors(ff["displ"], fp["displ"])
    assert s_l2 <= tol_s, ("stress L2", s_l2)
    assert s_li <= tol_linf, ("stress Linf", s_li)
    assert v_l2 <= tol_v, ("velocity L2", v_l2)
    assert d_l2 <= tol_d, ("displacement L2", d_l2)
    return cf, cp, dict(stress_l2=s_l2, stress_linf=s_li, vel_l2=v_l2, displ_l2=d_l2)


def test_fast_pairs_identical(built_gpu):
    p = cases.bui_like()
    # after three steps the positions of the two forms differ slightly; the pair set
    # must still be the same (the lattice is far from the support radius)
    cf, _ = run(p, _abi.SPS_PREC_FP32_FAST, 3)
    cp, _ = run(p, _abi.SPS_PREC_FP64_PLAIN, 3)
    a, b = cf.dump_pairs(), cp.dump_pairs()
    np.testing.assert_array_equal(a["pair_i"], b["pair_i"])
    np.testing.assert_array_equal(a["pair_j"], b["pair_j"])
    np.testing.assert_array_equal(a["pint_type"], b["pint_type"])
    # kernel values are compared on the first step, where the positions are identical
    cf, _ = run(p, _abi.SPS_PREC_FP32_FAST, 1)
    cp, _ = run(p, _abi.SPS_PREC_FP64_PLAIN, 1)
    a, b = cf.dump_pairs(), cp.dump_pairs()
    # the FP32 form forms r and q = r/h in double-float (no cancellation of 2 - q near the
    # edge of the support) and the polynomial in FP32: every value within a few FP32 ulps
    # of the FP64 evaluation rounded to FP32 (about half of them identical)
    for k in ("w", "dwdx", "dwdy"):
        same = a[k].view(np.int32) == b[k].view(np.int32)
        assert same.mean() >= 0.25, (k, same.mean())
        np.testing.assert_allclose(a[k], b[k], rtol=6e-7, atol=1e-30)


def test_fast_column(built_gpu):
    # cohesionless column with K0 stress: plastic from the first step, so the run is
    # sensitive to rounding; the FP32 form must stay within 3x the sensitivity of the FP64
    # plain run to an FP32-sized perturbation of its initial stress
    p = cases.column(dx=0.004)
    floor = chaos_floor(p, 200)
    floor64 = chaos_floor(p, 200, rel=2.0 ** -52)
    tol = max(1e-4, 3.0 * floor)
    _, _, err = compare(p, 200, tol_s=tol, tol_v=tol, tol_d=tol, tol_linf=1.0)
    print("column 200 steps: sensitivity to FP32-sized noise %.3g, to FP64-sized noise %.3g, "
          "FP32 form %s" % (floor, floor64, err))


def test_fast_bui_like(built_gpu):
    p = cases.bui_like()
    compare(p, 100)


def test_fast_cspm_bcs(built_gpu):
    compare(cases.bc_case(), 60)
    compare(cases.bui_like(width=1.0, height=0.5, dx=0.05, cspm=True, dt=5e-5), 60)


@pytest.mark.parametrize("make,nsteps", [(lambda: cases.column(dx=0.004), 30),
                                         (lambda: cases.bui_like(), 20)],
                         ids=["column", "bui_like"])
def test_fast_surface_detection_fp32(built_gpu, make, nsteps):
    # the FP32 form's on-demand free-surface detection in FP32 against its exact detection
    # on the same state: nothing in the step reads it here, so every other field is
    # bit-identical; flags may differ only at the scan region's edge, and the normals of
    # particles flagged alike agree to FP32 rounding of their sums
    p = make()
    out = []
    for exact in (True, False):
        ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                    p.params_copy(precision=_abi.SPS_PREC_FP32_FAST))
        sps_gb300.set_surface_detection(ctx, exact)
        ctx.upload_problem(p)
        t = 0.0
        for _ in range(nsteps):  # a download after every step, as an output loop does
            t = ctx.step(1, t)
            f = ctx.download()
        out.append((f, ctx.download_surface()))
    (fe, (ne, se)), (ff, (nf, sf)) = out
    for k in ("x", "vel", "stress", "rho", "intvars1", "displ", "f_drucker"):
        np.testing.assert_array_equal(fe[k].view(np.int64), ff[k].view(np.int64), err_msg=k)
    nt = p.ntotal
    differ = (fe["bc_or_not"] != ff["bc_or_not"]).sum() + (se != sf).sum()
    assert differ <= max(2, nt // 2000), differ
    assert (se == 1).sum() > 0
    both = (se == 1) & (sf == 1)
    ne2, nf2 = ne.reshape(-1, 2)[both], nf.reshape(-1, 2)[both]
    cosang = (ne2 * nf2).sum(axis=1)
    assert np.all(cosang > 1.0 - 1e-6), cosang.min()


def test_fast_pair_dump_after_replayed_steps(built_gpu):
    # the FP32 form gathers its lists straight from the cell stencil and builds the half
    # lists only when they are asked for (sps_dump_pairs, the exact detection's keyed
    # lists): after steps replayed from a graph, with or without a detection after each,
    # the dump is the last step's pair list, the same as a context that never downloaded
    p = cases.column(dx=0.004)
    dumps = []
    for every_step in (True, False):
        ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                    p.params_copy(precision=_abi.SPS_PREC_FP32_FAST))
        sps_gb300.set_surface_detection(ctx, True)
        ctx.upload_problem(p)
        t = 0.0
        for _ in range(12):
            t = ctx.step(1, t)
            if every_step:
                ctx.download()
        dumps.append(ctx.dump_pairs())
        ctx.close()
    for k in ("pair_i", "pair_j", "pint_type", "w", "dwdx", "dwdy"):
        np.testing.assert_array_equal(dumps[0][k], dumps[1][k], err_msg=k)
