"""The reference's example input sets (tests/golden/example_problems, copied from the
reference by tests/golden/make_example_inputs.py) and how each is run.

Every set is run with the constants of the source copy it ships with (the two options of
sps_params that no input file carries):
  - soil_failure_bui_et_al_2008/*: the reader's values for its header (CSPM threshold
    (double)1e-07f, Normal_BCs over nodes and stress-points);
  - strain_localisation_in_soil_sample/*: the reader's values for the header without
    ntype_solid ((double)1e-03f, nodes only: its 3_SPH_material_2018.f90:1664
    `do ipoin = 1,nnode`);
  - vertical_slope/*: (double)1e-03f, and Normal_BCs over 1..ntotal (its
    3_SPH_material_2018.f90:1664 `do ipoin = 1,ntotal`).

A set runs for its own length: the driver loop of code/1_SPH_2018.f90:72-88 takes steps
until maxtimestep, and leaves after the step whose FP64 `time` first exceeds time_end.
"""
import glob
import os

import numpy as np

import sps_gb300

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "golden", "example_problems")

# checkpoints besides the end of the run: step 10 (the Drucker-Prager sets' own length)
# and step 100 (the first hundred steps of a run)
CHECKPOINTS = (10, 100)


def example_sets():
    """Relative paths of the input sets (a directory holding input.txt, .dat and .pts)."""
    return sorted(os.path.relpath(os.path.dirname(p), ROOT)
                  for p in glob.glob(ROOT + "/**/input.txt", recursive=True)
                  if glob.glob(os.path.join(os.path.dirname(p), "*.dat")))


# the granular column collapse at its stated size (0.20 x 0.10 m at dx 2 mm: 5151 velocity +
# 5000 stress particles, K0 = 0.5, three dummy rows on the floor and the left wall), run
# for its stated 2000 steps
COLUMN = "column_collapse_dx2mm"
COLUMN_STEPS = 2000


def load(rel):
    if rel == COLUMN:
        return sps_gb300.Problem.column(dx=0.002)
    return sps_gb300.Problem.from_dir(os.path.join(ROOT, rel))


def overrides(rel):
    """sps_params fields of the source copy that `rel` belongs to."""
    if rel.startswith("vertical_slope"):
        return dict(bc_nodes_only=0)
    return {}


def own_steps(problem):
    """Steps the reference driver takes on the first (dt, time_end, maxtimestep) block."""
    if problem.name == "column":
        return COLUMN_STEPS
    b = problem.blocks[0]
    dt, t_end, nmax = b["dt"], b["time_end"], b["maxtimestep"]
    t = 0.0
    for k in range(1, nmax + 1):
        t = t + dt
        if t > t_end:
            return k
    return nmax


def checkpoints(problem):
    n = own_steps(problem)
    return sorted({c for c in CHECKPOINTS if c < n} | {n})


FIELDS = ("x", "vel", "stress", "rho", "intvars1", "displ", "f_drucker", "bc_or_not")


def run_oracle(rel):
    """Oracle run of one input set (a spawned worker process runs this): the fields at
    each checkpoint while the state stays finite, and the pair list and free-surface
    arrays of the last finite checkpoint.  Returns (checkpoints reached, {step: fields},
    pairs, (normal, subset), seconds)."""
    import time
    import orc
    p = load(rel)
    ctx = orc.context(p.params_copy(**overrides(rel)))
    ctx.upload_problem(p)
    t0 = time.time()
    out, done, t = {}, 0, 0.0
    reached = []
    pairs = surf = None
    for c in checkpoints(p):
        t = ctx.step(c - done, t)
        done = c
        f = ctx.download()
        f = {k: np.array(f[k]) for k in FIELDS}
        finite = all(np.isfinite(f[k]).all() for k in ("x", "vel")) and \
            np.isfinite(f["stress"][:4 * p.ntotal]).all()
        if not finite:
            break
        out[c] = f
        reached.append(c)
        pairs = {k: np.array(v) for k, v in ctx.dump_pairs().items()}
        n, s = ctx.download_surface()
        surf = (np.array(n), np.array(s))
    ctx.close()
    return reached, out, pairs, surf, time.time() - t0
