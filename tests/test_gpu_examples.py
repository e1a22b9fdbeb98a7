"""GPU parity on the reference's own example inputs and on the column collapse at its
stated size: the FP64 plain path against the CPU oracle, bit for bit (tolerance 0).

Each set runs for its own length (examples.own_steps: 10 steps for the Drucker-Prager
sets, 2101 for the strain-localisation sample, 2001 for the vertical cut, 16,667 for the
standard-SPH soil failure) and the column collapse for its 2000 steps; every downloaded
field is compared at steps 10 and 100 and at the end, the pair list and the free-surface
arrays at the end.  The oracle runs in spawned worker processes (one per set, started
before any set is compared) while the GPU runs the sets one after another.
"""
import multiprocessing as mp
import os
import sys

import numpy as np
import pytest

import cases
import examples
import sps_gb300
from sps_gb300 import _abi

pytestmark = pytest.mark.gpu

# The vertical cut with two stress-points per cell diverges: its velocities grow from
# 4e-4 m/s at step 10 to 1e6 m/s at step 15 and overflow to NaN by step 160 in the
# oracle.  Its smoothing length is 0.8 dx (support 1.6 dx) and each cell's two points sit
# at the thirds of its diagonal triangles (3_SPH_material_2018.f90 Read_2DMesh, npoints 2).
# It is compared at the checkpoints the oracle reaches with a finite state (steps 10 and
# 100); the GPU is not stepped into the overflow.  The set does not move its particles
# (update_x is off), so the cell grid and the pair search never see the large values.
DIVERGES = {"vertical_slope/SP2"}

SETS = examples.example_sets() + [examples.COLUMN]


def _init_worker(paths):
    for p in paths:
        if p not in sys.path:
            sys.path.insert(0, p)


@pytest.fixture(scope="module")
def oracle_runs(built):
    """One spawned oracle process per set, all submitted at once (largest first)."""
    paths = [p for p in sys.path if p.endswith(("stress-particle-sph_gb300", "oracle", "tests"))]
    ctx = mp.get_context("spawn")
    pool = ctx.Pool(min(len(SETS), os.cpu_count() or 1), initializer=_init_worker,
                    initargs=(paths,))
    cost = {}
    for rel in SETS:
        p = examples.load(rel)
        cost[rel] = p.ntotal2 * examples.own_steps(p)
    runs = {rel: pool.apply_async(examples.run_oracle, (rel,))
            for rel in sorted(SETS, key=lambda r: -cost[r])}
    yield runs
    pool.close()
    pool.join()


@pytest.mark.parametrize("rel", SETS)
def test_example_bitwise(built_gpu, oracle_runs, rel):
    reached, ofields, opairs, osurf, secs = oracle_runs[rel].get(timeout=1800)
    p = examples.load(rel)
    want = examples.checkpoints(p)
    if rel in DIVERGES:
        assert reached and reached != want, "expected the oracle's run to overflow"
    else:
        assert reached == want, (reached, want)
    g = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                              p.params_copy(precision=_abi.SPS_PREC_FP64_PLAIN,
                                            **examples.overrides(rel)))
    g.upload_problem(p)
    t, done = 0.0, 0
    for c in reached:
        t = g.step(c - done, t)
        done = c
        f = g.download()
        try:
            cases.assert_bitwise(f, ofields[c], p.ntotal)
            np.testing.assert_array_equal(f["bc_or_not"], ofields[c]["bc_or_not"])
        except AssertionError as e:
            raise AssertionError("%s, step %d: %s" % (rel, c, e))
    pg = g.dump_pairs()
    for k in ("pair_i", "pair_j", "pint_type"):
        np.testing.assert_array_equal(pg[k], opairs[k], err_msg=k)
    for k in ("w", "dwdx", "dwdy"):
        np.testing.assert_array_equal(pg[k].view(np.int32), opairs[k].view(np.int32), err_msg=k)
    ng, sg = g.download_surface()
    np.testing.assert_array_equal(sg, osurf[1], err_msg="subset")
    same = (ng.view(np.int64) == osurf[0].view(np.int64)) | (np.isnan(ng) & np.isnan(osurf[0]))
    assert same.all(), "surface normal"
    g.close()
