"""Parameterised problem generators for the tests (reference input format, own values).

Each generator writes input.txt / <name>.dat / <name>.pts text in the format the
Drucker-Prager example reads (example_problems/soil_failure_bui_et_al_2008/
3_SPH_material_2018.f90 problem_input_data and Read_2DMesh) and parses it with the
product's reader, so every case goes through the same set-up path as a reference input.
"""
import numpy as np

import sps_gb300


def _fmt(v):
    return repr(float(v))


def bui_like(width=4.0, height=2.0, dx=0.1, young=1.8e6, poiss=0.3, rho=1850.0,
             tanphi=0.466308, coh=5000.0, xsph=True, cspm=False, alpha=0.1, beta=0.1,
             damping=0.0, dt=1.5e-4, sml=1.2, skf=1, cont_density=False, sle=1,
             ntype_solid=2, npoints=1, floor_to=9.0, ntype_eco=2, ncrit=12,
             output_flags="1 1 1 1 1 1 1 0 0 0", art_stress=False, outside=None,
             domain=(-10, -10, 41, 41), gravity_curve=((0, 1, 500), (1, 1, 1))):
    """Cohesive soil block on a floor with a left wall: the layout of the Drucker-Prager
    example (inside approach, three dummy rows) with every parameter adjustable.
    domain: xmin, ymin, xmax, ymax of the domain box (Check_Out_Domain); gravity_curve:
    the times and factors of the gravity time curve."""
    pts = "\n".join([
        "geom_type", "1", "x1 x2 x3 x4 dx",
        "0.0 %s 0.0 %s %s" % (_fmt(width), _fmt(width), _fmt(dx)),
        "y1 y2 y3 y4 dy",
        "0 0 %s %s %s" % (_fmt(height), _fmt(height), _fmt(dx)),
        "dummy nodes", "T", "number_of_walls", "2",
        "wall_1 - LHS wall", "id position x1 x2",
        "1 %s %s %s" % (_fmt(-dx), _fmt(-dx), _fmt(height + dx)),
        "wall_2 - bottom wall", "id position x1 x2",
        "2 %s %s %s" % (_fmt(-dx), _fmt(-3 * dx), _fmt(floor_to)), ""])
    L = lambda b: "T" if b else "F"
    dat = "\n".join([
        "1", "generated test case", "ndimn", "2", "ntype_solid nstre nmats",
        "%d 4 1" % ntype_solid,
        "mater. eco law E Poiss b rho yield H ? gamma delta n",
        "1 %d %d %s %s 1. %s 2000. 0 0. 5. 1. 1" % (ntype_eco, ncrit, _fmt(young), _fmt(poiss),
                                                  _fmt(rho)),
        "tan(phi) cohesion",
        "%s %s 0 0 0 0 0 0 0 0" % (_fmt(tanphi), _fmt(coh)),
        "ic_unks", "0", "BC's: nprer Sigman=0", "0 0", "segments", "0", "nodes", "0",
        "ic_tcurve", "1", "ntcurves mpts", "1 100", "pts in curve 1",
        str(len(gravity_curve[0])), "times and factors",
        " ".join(_fmt(v) for v in gravity_curve[0]), " ".join(_fmt(v) for v in gravity_curve[1]),
        "xmin domain xmax domain", " ".join(_fmt(v) for v in domain),
        "Initial conditions index", "2", "s11", "0", "s22", "0", "s12", "0", "s33", "0", "w1", "0",
        "v2", "0", "pa_sph nnps sle skf cspm update_x XSPH",
        "2 2 %d %d %s T %s" % (sle, skf, L(cspm), L(xsph)),
        "summ dens cont dens", "F %s" % L(cont_density), "damping", _fmt(damping), "alpha beta",
        "%s %s" % (_fmt(alpha), _fmt(beta)), "ic_grav", "1", "gx gy timecurve factor",
        "0 -9.81 1 1.", "output values", "sxx syy sxy szz ux uy strain rho sml disp_10",
        output_flags, ""])
    # outside approach: dict(sph_shift, vel_vector, shift_update, rx, ry, disp_tol), the
    # line of the outside-approach example's input.txt
    shift = [] if outside is None else [
        "SPH_shifting vel_vector shift_update rx_factor ry_factor disp_tol",
        "%s %s %d %s %s %s" % (L(outside["sph_shift"]), L(outside["vel_vector"]),
                               outside["shift_update"], _fmt(outside["rx"]), _fmt(outside["ry"]),
                               _fmt(outside["disp_tol"]))]
    inp = "\n".join([
        "problem name", "gen", "SP_SPH art_stress particle_shift", "T %s F" % L(art_stress),
        "inside_approach", "T" if outside is None else "F", "number of stress points",
        str(npoints)] + shift + ["smoothing length factor",
        _fmt(sml), "time step, time for end, max number of time steps",
        "%s,2.5,10" % _fmt(dt), "print, save, plot", "1,1,1", "if end of simulation:", "-1,1,1",
        ""])
    return sps_gb300.Problem.from_text(inp, dat, pts)


def bc_case(width=0.5, height=1.0, dx=0.05, young=8e7, poiss=0.25, rho=2000.0, dt=1e-5,
            plastic=False, cspm=True, xsph=False, sml=1.2, ncrit=12, yield_stress=5e5,
            hards=0.0, phi_deg=0.0, gamma=50.0, delta=1.0, nflow=1, ntype_solid=2):
    """Biaxial-style sample without walls and with segment and nodal boundary conditions,
    a time-curve platen velocity, a sinusoidal lateral stress and a time-curve stress,
    in the style of the strain-localisation example's input.  ncrit 12: Drucker-Prager
    (tan phi 0.7, c 100 Pa); ncrit 1-4: the viscoplastic laws with the yield stress,
    hardening modulus, friction angle and Perzyna parameters given."""
    pts = "\n".join([
        "geom_type", "1", "x1 x2 x3 x4 dx",
        "0 %s 0 %s %s" % (_fmt(width), _fmt(width), _fmt(dx)),
        "y1 y2 y3 y4 dy",
        "0 0 %s %s %s" % (_fmt(height), _fmt(height), _fmt(dx)),
        "dummy_nodes", "F", ""])
    W, H = _fmt(width), _fmt(height)
    law = ["tan(phi) cohesion", "0.7 100.0 0 0 0 0 0 0"] if ncrit in (5, 12) else []
    dat = "\n".join([
        "1", "bc test", "ndimn", "2", "ntype_solid nstre nmats", "%d 4 1" % ntype_solid,
        "mater. eco law E Poiss b rho yield H fi gamma delta n",
        "1 %d %d %s %s 1. %s %s %s %s %s %s %d" % (
            2 if plastic else 1, ncrit, _fmt(young), _fmt(poiss), _fmt(rho),
            _fmt(yield_stress), _fmt(hards), _fmt(phi_deg), _fmt(gamma), _fmt(delta), nflow)
    ] + law + [
        "ic_unks", "0", "no. of BC's Sigman=0", "6 0",
        "nber var t_variation a1 a0 w fi Tf",
        "1 5 1 0 0 0 0 0",
        "2 6 1 0 0 0 0 0",
        "3 1 0 -2.e4 -1.e4 900. 30. 0.001",
        "4 3 1 0 0 0 0 0",
        "5 6 1 -0.05 0 0 0 0",
        "6 2 2 -3.e4 0 0 0 0",
        "nber of segment with BCs", "7", "x1 y1 x2 y2 BC",
        "0. 0. 0. %s 1" % H,
        "0. 0. 0. %s 4" % H,
        "0. %s %s %s 5" % (H, W, H),
        "%s 0. %s %s 3" % (W, W, H),
        "%s 0. %s %s 4" % (W, W, H),
        "0. 0. %s 0. 1" % W,
        "0. 0. %s 0. 2" % W,
        "nber of nodes with BCs", "1", "node bc", "%d 6" % (2 * (int(round(height / dx)) + 1) + 5),
        "ic_tcurve", "1", "ntcurves mpts", "2 100", "pts in curve 1", "5",
        "Curve 1 times and factors", "0. 0.00005 0.00005 0.2 1", "0 1 1 1 1",
        "pts in curve 2", "4", "Curve 2 times and factors", "0. 0.00005 0.00051 1",
        "1.0 1.0 1.0 1.0", "xmin domain xmax domain", "-1 -1 41 41",
        "Initial conditions index", "2", "s11", "0", "s22", "0", "s12", "0", "s33", "0", "w1", "0",
        "v2", "0", "pa_sph nnps sle skf cspm update_x XSPH",
        "2 2 1 1 %s T %s" % ("T" if cspm else "F", "T" if xsph else "F"),
        "summ dens cont dens", "F F", "damping", "0", "alpha beta", "0.0 0.0", "ic_grav", "0",
        "output values", "sxx syy sxy szz ux uy strain rho sml disp_10",
        "0 0 1 0 1 1 1 0 0 0", ""])
    inp = "\n".join([
        "problem name", "bc", "SP_SPH art_stress particle_shift", "T F F", "inside_approach",
        "T", "number of stress points", "1", "smoothing length factor", _fmt(sml),
        "time step", "%s,0.021,10" % _fmt(dt), "print, save, plot", "100,100,100", "end",
        "-1,1,1", ""])
    return sps_gb300.Problem.from_text(inp, dat, pts)


def standard_sph(width=1.0, height=0.5, dx=0.05, dt=5e-5):
    """Standard SPH (SP_SPH = F): stress-points coincide with the nodes."""
    pts = "\n".join([
        "geom_type", "1", "x1 x2 x3 x4 dx", "0 %s 0 %s %s" % (_fmt(width), _fmt(width), _fmt(dx)),
        "y1 y2 y3 y4 dy", "0 0 %s %s %s" % (_fmt(height), _fmt(height), _fmt(dx)),
        "dummy nodes", "T", "number_of_walls", "1", "wall_2 - bottom wall", "id position x1 x2",
        "2 %s %s %s" % (_fmt(-dx), _fmt(-3 * dx), _fmt(3 * width)), ""])
    dat = bui_like_dat_text()
    inp = "\n".join([
        "problem name", "std", "SP_SPH art_stress particle_shift", "F F F",
        "smoothing length factor", "1.2", "time step", "%s,2.5,10" % _fmt(dt),
        "print, save, plot", "1,1,1", "end", "-1,1,1", ""])
    return sps_gb300.Problem.from_text(inp, dat, pts)


def bui_like_dat_text():
    return "\n".join([
        "1", "std", "ndimn", "2", "ntype_solid nstre nmats", "2 4 1",
        "mater. eco law E Poiss b rho yield H ? gamma delta n",
        "1 2 12 1.8e06 0.3 1. 1850 2000. 0 0. 5. 1. 1", "tan(phi) cohesion",
        "0.466308 5000 0 0 0 0 0 0", "ic_unks", "0", "BC's", "0 0", "segments", "0", "nodes", "0",
        "ic_tcurve", "1", "curves", "1 100", "pts", "3", "times", "0 1 500", "1 1 1", "domain",
        "-10 -10 41 41", "IC", "2", "s11", "0", "s22", "0", "s12", "0", "s33", "0", "w1", "0",
        "v2", "0", "flags", "2 2 1 1 F T F", "dens", "F F", "damping", "0", "alpha beta",
        "0.1 0.1", "ic_grav", "1", "g", "0 -9.81 1 1.", "output", "x", "1 1 1 1 1 1 1 0 0 0", ""])


def column(dx=0.004, **kw):
    """The granular column collapse workload (K0 stress) at a test-sized spacing."""
    return sps_gb300.Problem.column(dx=dx, **kw)


def run_pair(problem, nsteps, contexts, chunks=None):
    """Upload a problem into each context and advance them in the same step chunks."""
    chunks = chunks or [nsteps]
    times = []
    for ctx in contexts:
        ctx.upload_problem(problem)
        t = 0.0
        for c in chunks:
            t = ctx.step(c, t)
        times.append(t)
    return times


def fields(ctx):
    return ctx.download()


def assert_bitwise(a, b, ntotal=None,
                   keys=("x", "vel", "stress", "rho", "intvars1", "displ", "f_drucker")):
    """Bitwise equality of downloaded fields.  The stress of dummy particles (ids above
    ntotal) is excluded: the reference writes it only as pair-local scratch inside
    get_derivatives (node--dummy pairs copy the node's stress into the dummy) and never
    reads it elsewhere, so the GPU path does not materialise it."""
    for k in keys:
        x, y = a[k], b[k]
        if k == "stress" and ntotal is not None:
            x, y = x[:4 * ntotal], y[:4 * ntotal]
        same = (x.view(np.int64) == y.view(np.int64)) | (np.isnan(x) & np.isnan(y))
        if not same.all():
            idx = np.nonzero(~same)[0]
            raise AssertionError("%s differs at %d entries, first %s: %r vs %r" % (
                k, len(idx), idx[:5], x[idx[:5]], y[idx[:5]]))
