"""Multi-process host logic of bench.py (replicas, no data-path collective), on CPU.

Two gloo ranks each advance their own oracle replica of a small problem and time it; the
job time is the max over ranks and the throughput counts every rank's particles.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import time
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    for p in (ROOT, os.path.join(ROOT, "stress-particle-sph_gb300"), os.path.join(ROOT, "oracle"),
              os.path.join(ROOT, "tests")):
        sys.path.insert(0, p)
    import bench
    import cases
    import orc
    r, w, dist = bench.dist_init("gloo")
    assert (r, w) == (rank, world)
    prob = cases.bui_like(width=1.0, height=0.5, dx=0.05)
    ctx = orc.context(prob.params_copy())
    ctx.upload_problem(prob)
    bench.barrier(dist)
    t0 = time.perf_counter()
    ctx.step(2 + rank, 0.0)  # ranks do different amounts of work
    el = time.perf_counter() - t0
    mx = bench.reduce_max(dist, el)
    q.put((rank, el, mx, prob.nnode + prob.nstress))
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_rank_replicas(built):
    import multiprocessing as mp
    import socket
    pytest.importorskip("torch")
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    els = [e for _, e, _, _ in res]
    maxes = {m for _, _, m, _ in res}
    assert len(maxes) == 1 and abs(maxes.pop() - max(els)) < 1e-12
