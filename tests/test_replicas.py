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


def test_partition_by_size(built):
    import sps_gb300
    sizes = [60000, 2000, 35000, 35000, 12000, 9000, 58000, 4000, 21000]
    for n in (1, 2, 3, 4):
        parts = sps_gb300.partition_by_size(sizes, n)
        assert len(parts) == n
        assert sorted(i for q in parts for i in q) == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in q) for q in parts]
        # greedy largest-first: no rank exceeds the mean by more than the largest item
        assert max(loads) - sum(loads) / n <= max(sizes)
        assert parts == sps_gb300.partition_by_size(sizes, n)  # deterministic
    # 60k, 58k, 35k, 35k, 21k, ... placed in turn on the lighter rank: 118k on each
    assert sps_gb300.partition_by_size(sizes, 2) == [[0, 1, 3, 4, 5], [2, 6, 7, 8]]


def _batch_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    for p in (ROOT, os.path.join(ROOT, "stress-particle-sph_gb300"), os.path.join(ROOT, "oracle"),
              os.path.join(ROOT, "tests")):
        sys.path.insert(0, p)
    import numpy as np
    import bench
    import cases
    import orc
    r, w, dist = bench.dist_init("gloo")
    probs = [cases.bui_like(width=wd, height=0.5, dx=0.05) for wd in (1.0, 0.6, 0.8, 0.4, 1.2)]
    mine, idx = bench.shard(probs, dist)
    # each rank advances its own realisations; nothing crosses ranks but the totals
    digest = []
    for p in mine:
        ctx = orc.context(p.params_copy())
        ctx.upload_problem(p)
        ctx.step(2, 0.0)
        digest.append(float(np.abs(ctx.download()["stress"]).sum()))
    total = bench.reduce_sum(dist, sum(p.nnode + p.nstress for p in mine))
    q.put((rank, idx, digest, total))
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_rank_batch_shards(built):
    import multiprocessing as mp
    import socket
    pytest.importorskip("torch")
    import cases
    import orc
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_batch_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    probs = [cases.bui_like(width=wd, height=0.5, dx=0.05) for wd in (1.0, 0.6, 0.8, 0.4, 1.2)]
    # the shards cover the batch once, and the summed count is the whole batch's
    assert sorted(i for _, idx, _, _ in res for i in idx) == list(range(len(probs)))
    assert res[0][3] == res[1][3] == sum(p.nnode + p.nstress for p in probs)
    # a realisation advanced on its rank equals the same realisation advanced alone
    import numpy as np
    for _, idx, digest, _ in res:
        for i, d in zip(idx, digest):
            c = orc.context(probs[i].params_copy())
            c.upload_problem(probs[i])
            c.step(2, 0.0)
            assert d == float(np.abs(c.download()["stress"]).sum())
