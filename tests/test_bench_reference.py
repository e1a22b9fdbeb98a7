"""bench.py --impl reference on CPU: the replica count, one run of two replicas of a small
slope, and the launch under torchrun, where rank 0 alone runs and prints."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402

SMALL = ["--impl", "reference", "--dx", "0.2", "--steps", "1", "--warmup", "1"]


def _lines(out):
    return [json.loads(s) for s in out.splitlines() if s.startswith("{")]


def test_replicas_bounded_by_cores_and_memory():
    n2 = 2_012_175  # the 1.2 cm slope's particle slots
    per = bench.REF_BYTES_FIXED + bench.REF_BYTES_PER_PARTICLE * n2
    assert bench.reference_replicas(n2, 16, None) == 16
    assert bench.reference_replicas(n2, 16, 1 << 50) == 16
    # 60% of the memory holds five replicas
    assert bench.reference_replicas(n2, 16, int(5 * per / 0.6) + 1) == 5
    assert bench.reference_replicas(n2, 4, int(5 * per / 0.6) + 1) == 4
    # never fewer than one
    assert bench.reference_replicas(n2, 16, 0) == 1
    assert bench.reference_replicas(n2, 0, None) == 1


def test_host_memory_available():
    a = bench.host_memory_available()
    assert a is None or a > 0


def test_reference_arm_two_replicas():
    out = subprocess.run([sys.executable, "bench.py"] + SMALL + ["--ref-replicas", "2"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    (line,) = _lines(out.stdout)
    assert line["impl"] == "reference"
    assert line["config"]["replicas"] == 2 and line["cpu_baseline"]["cores"] == 2
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    n = line["config"]["particles"]
    # value = replicas * particles * steps / the slowest replica's time
    el = line["ms_per_step"] * line["steps"] / 1e3
    assert abs(line["value"] - 2 * n * line["steps"] / el) <= 0.01 * line["value"] + 1.0


def test_reference_arm_under_torchrun():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                          "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
                          "--master-port", str(port), "bench.py", "--gpus", "2"] + SMALL +
                         ["--ref-replicas", "1"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = _lines(out.stdout)
    assert len(lines) == 1  # rank 0 alone prints
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2
