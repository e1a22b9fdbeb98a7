#!/usr/bin/env python3
"""bench.py -- particle-steps/s of the Stress-Particle SPH step on GB300.

Workload (the configuration the headline metric is quoted on): a 10 m vertical slope
(block 4.4 m x 10 m) on a 20 m x 5 m foundation, spacing 1.2 cm -> about 1.00M velocity
particles + 1.00M stress-points, Drucker-Prager soil (rho 1850, E 20 MPa, nu 0.3,
phi 30 deg, c 10 kPa), K0 stress, gravity ramped in over 0.05 s, dt = 0.1 h / sqrt(E/rho).
A "step" is one call of the reference's time_integration (neighbour search + RK4 +
position update) over the whole particle set.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value  = (N_v + N_s) * K * ranks / max-over-ranks device time of K graph-launched steps
         (CUDA events on the context's own stream; state resident in HBM, working set
         larger than L2).
e2e    = the same metric through the C-ABI with host buffers: every step uploads the
         state from pinned host memory (sps_upload), advances one step (sps_step) and
         downloads the fields (sps_download).
--impl reference times the CPU restatement of the reference's step (the oracle; the
         Fortran reference cannot be compiled on either machine) on the same workload, as
         independent single-threaded replicas (the reference's step is single-threaded),
         one per host core as far as the host memory allows, for a bounded number of steps
         (min(K, 2) after min(W, 1) warm-up); value = all replicas' particle-steps over
         the slowest replica's time.

The headline runs the FP32 form with the learned Drucker-Prager surrogate installed
(trained first, on the GPU, on tuples captured from coarse runs of the same slope with
seeded material draws); the FP32 form without it and the FP64 plain form are timed beside
it on the same workload, and the errors of both FP32 runs against the plain run are
reported after the same number of steps.
"""
import argparse
import json
import os
import queue
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "stress-particle-sph_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "particle-steps/s at 1M particles: FP64 plain vs FP32+surrogate at stated error"
SLOPE = dict(Lf=20.0, Hf=5.0, Ls=4.4, Hs=10.0, young=20e6, poiss=0.3, rho=1850.0, phi_deg=30.0,
             cohesion=10e3, k0=0.5, t_ramp=0.05)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-replicas", type=int, default=0,
                    help="reference arm: single-threaded replicas of the workload run side "
                         "by side (0: one per core, bounded by the host memory)")
    ap.add_argument("--precision", default="fast", choices=["plain", "fast"])
    ap.add_argument("--dx", type=float, default=0.012)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-size", type=int, default=256)
    ap.add_argument("--error-steps", type=int, default=0,
                    help="instead of timing: advance the FP64 plain and the FP32 forms this "
                         "many steps side by side and report their relative errors")
    ap.add_argument("--error-times", default="",
                    help="with --error-steps: comma-separated simulated times (s) at which the "
                         "errors are also reported (the step whose time first reaches each)")
    ap.add_argument("--error-at", type=float, default=0.01,
                    help="simulated time (s) at which the run also reports the errors of the "
                         "FP32 form, with and without the surrogate, and of the 2^-52 floor "
                         "against the FP64 plain form, from fresh contexts (0: skip)")
    ap.add_argument("--steady-steps", type=int, default=500,
                    help="steps with the network before the settled with/without comparison "
                         "(0: skip)")
    ap.add_argument("--surrogate-tol", type=float, default=1e-6)
    ap.add_argument("--surrogate-gate", type=float, default=0.5,
                    help="answered fraction below which a step runs without the network "
                         "(sps_surrogate_gate; 0 keeps the network on in every step)")
    ap.add_argument("--workload", default="slope", choices=["slope", "column-batch", "biaxial"],
                    help="slope: the headline (one 2M-particle slope); column-batch: the "
                         "combined form (batched columns, FP32 + surrogate vs FP64 plain); "
                         "biaxial: the surrogate's biaxial sample")
    ap.add_argument("--columns", type=int, default=16)
    ap.add_argument("--combined-steps", type=int, default=2000,
                    help="column-batch, biaxial: steps of the FP32 + surrogate and FP64 "
                         "plain runs before their fields are compared")
    return ap.parse_args()


def dist_init(backend):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch.distributed as dist
    dist.init_process_group(backend=backend)
    return dist.get_rank(), dist.get_world_size(), dist


def reduce_max(dist, v, device=None):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = max(smax, float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp64_peak_tflops():
    """FP64 throughput of cuBLAS DGEMM on this GPU (the FP64 pipe's practical ceiling)."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e30
    for _ in range(3):
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


# material ranges of the surrogate's training runs (stratified draws bracket the slope's)
SURR_RANGES = dict(phi_deg=(26.0, 34.0), cohesion=(6e3, 14e3), young=(14e6, 26e6),
                   poiss=(0.27, 0.33), rho=(1800.0, 1900.0), k0=(0.42, 0.58))


def train_surrogate(seed=0, nruns=6, dx=0.08, nsteps=2000, every=20, max_tuples=4000000,
                    schedule=((10, 2e-3), (6, 5e-4), (4, 1e-4)), make=None, ranges=None,
                    geometry="slope geometry"):
    """Capture tuples from coarse FP32 runs of a geometry (default: the slope) with seeded
    materials and train the network on the GPU; returns (net, envelope, summary).
    make(dx, material) builds one training problem; ranges are the material draws."""
    import numpy as np
    import sps_gb300
    from sps_gb300 import _abi
    from sps_gb300 import surrogate as sg
    if make is None:
        def make(dx, mat):
            return sps_gb300.Problem.slope(dx=dx, **dict(SLOPE, **mat))
    ranges = SURR_RANGES if ranges is None else ranges
    w0 = time.perf_counter()
    runs = []
    for mat in sg.stratified_materials(ranges, nruns, seed):
        prob = make(dx, mat)
        runs.append(sg.sample_run(prob, _abi.SPS_PREC_FP32_FAST, nsteps, every))
    data = np.concatenate(runs)
    captured = len(data)
    w1 = time.perf_counter()
    idx = np.random.default_rng(seed).permutation(len(data))[:max_tuples]
    nhold = min(20000, len(data) // 10)
    hold, train = data[idx[:nhold]], data[idx[nhold:]]
    net = sg.Mlp(batch=4096, seed=seed + 1)
    net.set_data(train)
    loss = net.fit(schedule)
    w2 = time.perf_counter()
    y = net.predict(hold[:, :sg.NIN])
    t = hold[:, sg.NIN:].astype(np.float64)
    held = float(np.linalg.norm(y - t) / max(np.linalg.norm(t), 1e-300))
    summary = {"tuples": int(len(train)), "captured": int(captured), "runs": nruns,
               "runs_desc": "%s at dx %.3g m, %d steps, one step in %d captured, "
                            "stratified draws of %s" % (geometry, dx, nsteps, every, ranges),
               "capture_s": round(w1 - w0, 2), "train_s": round(w2 - w1, 2),
               "epochs": int(len(loss)), "schedule": [list(x) for x in schedule],
               "loss_first_epoch": float(loss[0]),
               "loss_last_epoch": float(loss[-1]), "heldout_rel_l2": round(held, 4),
               "network": "14-128-128-128-4 SiLU, BF16 weights/activations, FP32 accumulate"}
    return net, sg.Envelope.of(train), summary


def batch_problems(n=256, seed=0):
    """Seeded 2D slopes: height U[2,10] m, face angle U[30,70] deg, U[2k,60k] velocity
    particles each (spacing from the area), phi U[20,40] deg, c U[0,20] kPa, E U[10,50] MPa,
    nu 0.3, rho U[1800,2000]; foundation half the height deep, crest half the height wide."""
    import numpy as np
    import sps_gb300
    rng = np.random.default_rng(seed)
    out, desc = [], []
    for _ in range(n):
        H, face, nt = rng.uniform(2, 10), rng.uniform(30, 70), rng.uniform(2000, 60000)
        phi, coh, E, rho = (rng.uniform(20, 40), rng.uniform(0, 20e3), rng.uniform(10e6, 50e6),
                            rng.uniform(1800, 2000))
        run = H / np.tan(np.radians(face))
        Hf, Ls = 0.5 * H, 0.5 * H
        Lf = Ls + run + H
        area = Lf * Hf + Ls * H + 0.5 * H * run
        dx = float(np.sqrt(area / nt))
        out.append(sps_gb300.Problem.slope(Lf=Lf, Hf=Hf, Ls=Ls, Hs=H, dx=dx, young=E, poiss=0.3,
                                           rho=rho, phi_deg=phi, cohesion=coh, k0=0.5,
                                           t_ramp=0.05, face_deg=face))
    return out


def shard(probs, dist):
    """This rank's share of a batch of realisations (partitioned by particle count, no
    exchange between ranks) and their indices; the whole batch on one rank."""
    import sps_gb300
    if dist is None:
        return probs, list(range(len(probs)))
    mine = sps_gb300.partition_by_size([p.nnode + p.nstress for p in probs],
                                       dist.get_world_size())[dist.get_rank()]
    return [probs[i] for i in mine], mine


def reduce_sum(dist, v, device=None):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_batch(args, dist, local):
    """The batched-realisations workload: one FP32 context holding every slope (under
    torchrun, this rank's share of them)."""
    import numpy as np
    import sps_gb300
    from sps_gb300 import _abi
    w0 = time.perf_counter()
    probs, _ = shard(batch_problems(args.batch_size), dist)
    b = sps_gb300.Batch(probs, precision=_abi.SPS_PREC_FP32_FAST)
    b.upload_all()
    tuned = sps_gb300.autotune(b, 2)
    w1 = time.perf_counter()
    b.step(max(args.warmup, 1))
    _, ms, clk = timed_steps(b, args.steps, None, dist, local)
    n = reduce_sum(dist, sum(p.nnode + p.nstress for p in probs), device="cuda")
    nv = reduce_sum(dist, sum(p.nnode for p in probs), device="cuda")
    # two realisations against contexts holding them alone (bit-identical fields)
    same = {}
    done = max(args.warmup, 1) + args.steps
    for r in (0, len(probs) // 2):
        ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                    probs[r].params_copy(precision=_abi.SPS_PREC_FP32_FAST))
        ctx.upload_problem(probs[r])
        ctx.step(done, 0.0)
        a, bb = ctx.download(), b.download(r)
        same[str(r)] = bool(all(np.array_equal(a[k], bb[k]) for k in ("x", "vel", "stress")))
        ctx.close()
    b.close()
    return {"realisations": args.batch_size, "realisations_per_rank": len(probs),
            "particles": int(n), "velocity_particles": int(nv),
            "value": round(n * args.steps / (ms * 1e-3), 1), "unit": "particle-steps/s",
            "ms_per_step": round(ms / args.steps, 4), "steps": args.steps,
            "setup_s": round(w1 - w0, 2), "precision": "fp32 form", "autotuned_blocks": tuned,
            "bit_identical_to_single_runs": same, "clocks": clk,
            "workload": batch_problems.__doc__.split("\n")[0]}


# the combined form: batched granular columns of the column-collapse material, friction
# drawn per column; the surrogate is trained on coarse columns that bracket the draws
COLUMN = dict(width=0.5, height=0.25, young=5.84e6, poiss=0.3, rho=2650.0, cohesion=0.0, k0=0.5)
COLUMN_SURR_RANGES = dict(phi_deg=(19.0, 35.0), k0=(0.42, 0.58))


def column_batch_problems(n=16, dx=0.001, seed=0):
    """Granular columns 0.5 m wide x 0.25 m high at dx 1 mm (125,751 velocity + 125,000
    stress particles each), left wall and a 2 m floor, rho 2650, E 5.84 MPa, nu 0.3, c 0,
    K0 0.5, phi U[19,35] deg per column."""
    import numpy as np
    import sps_gb300
    rng = np.random.default_rng(seed)
    phis = rng.uniform(19.0, 35.0, n)
    return [sps_gb300.Problem.column(dx=dx, phi_deg=float(p), **COLUMN) for p in phis], phis


def three_arms(args, make, n, net, env, training, dist, local):
    """The FP32 form with the surrogate installed, the FP64 plain form and the FP32 form
    alone on the same problem(s) (n: the particles of the whole job, all ranks): each is
    timed over args.steps graph-launched steps after the warm-up, then advances to
    args.combined_steps steps in all, and its fields are downloaded (one dict per
    realisation).  make(precision) -> uploaded context."""
    import torch
    from sps_gb300 import _abi
    from sps_gb300 import surrogate as sg
    import sps_gb300
    nlong = max(args.combined_steps, max(args.warmup, 1) + args.steps)
    arms, fields, surr = {}, {}, None
    for name, prec, use in (("fp32_surrogate", _abi.SPS_PREC_FP32_FAST, True),
                            ("fp64_plain", _abi.SPS_PREC_FP64_PLAIN, False),
                            ("fp32", _abi.SPS_PREC_FP32_FAST, False)):
        b = make(prec)
        if use:
            sg.install(b, net, tol=args.surrogate_tol, envelope=env)
            sg.set_gate(b, args.surrogate_gate)
        sps_gb300.autotune(b, 2)
        single = not isinstance(b, sps_gb300.Batch)
        t = b.step(max(args.warmup, 1), 0.0) if single else b.step(max(args.warmup, 1))
        if use:
            sg.stats(b, reset=True)
        t, ms, clk = timed_steps(b, args.steps, t if single else None, dist, local)
        arms[name] = {"value": round(n * args.steps / (ms * 1e-3), 1),
                      "ms_per_step": round(ms / args.steps, 4), "clocks": clk}
        rest = nlong - max(args.warmup, 1) - args.steps
        t = b.step(rest, t) if single else b.step(rest)
        torch.cuda.synchronize()
        fields[name] = [b.download()] if single else \
            [b.download(r) for r in range(len(b.problems))]
        arms[name]["simulated_s"] = t if single else b.times[0]
        if use:
            loading, answered, outside, rejected = sg.stats(b)
            lf = max(loading, 1)
            surr = {"tol": args.surrogate_tol, "training": training,
                    "loading_evaluations": loading, "answered_frac": round(answered / lf, 6),
                    "outside_envelope_frac": round(outside / lf, 6),
                    "fallback_rate": round(1.0 - answered / lf, 6) if loading else None}
        b.close()
    return arms, fields, surr


# the biaxial sample: the surrogate is trained on coarse samples with seeded materials and
# faster platens (plastic within the captured steps)
BIAXIAL = dict(width=0.05, height=0.10, young=50e6, poiss=0.25, rho=2000.0, phi_deg=35.0,
               cohesion=0.0, platen_v=0.05, t_ramp=1e-4)
BIAXIAL_SURR_RANGES = dict(phi_deg=(30.0, 40.0), young=(40e6, 60e6), poiss=(0.22, 0.28),
                           rho=(1900.0, 2100.0))


def run_biaxial(args):
    """The surrogate's own configuration: a biaxial sample 0.05 m x 0.10 m at dx 0.1 mm
    (501,501 velocity + 500,000 stress particles), rough platens closing at 0.05 m/s each,
    cohesionless Drucker-Prager (phi 35 deg, E 50 MPa, nu 0.25, rho 2000).  The network is
    trained on the GPU on up to 20M tuples captured from eight coarse samples (dx 1 mm,
    platens 0.5 m/s, 12,000 steps, one in ten captured) with seeded material draws; then the
    FP32 form with it, the FP64 plain form and the FP32 form alone are timed and compared."""
    import numpy as np
    import torch
    import sps_gb300
    rank, world, dist = dist_init("nccl")
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    sps_gb300.build_all()
    w0 = time.perf_counter()
    prob = sps_gb300.Problem.biaxial(dx=1e-4, **BIAXIAL)
    n = prob.nnode + prob.nstress
    net, env, training = train_surrogate(
        dx=0.001, nruns=8, nsteps=12000, every=10, max_tuples=20000000,
        make=lambda dx, m: sps_gb300.Problem.biaxial(dx=dx, **dict(
            BIAXIAL, platen_v=0.5, t_ramp=2e-5, **m)),
        ranges=BIAXIAL_SURR_RANGES, geometry="biaxial sample 0.05 x 0.10 m, platens 0.5 m/s")
    setup_s = time.perf_counter() - w0

    def single(prec):
        c = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", prob.params_copy(precision=prec))
        c.upload_problem(prob)
        return c

    # every rank runs a replica of the sample
    arms, fields, surr = three_arms(args, single, n * world, net, env, training, dist, local)
    nlong = max(args.combined_steps, max(args.warmup, 1) + args.steps)
    b = fields["fp64_plain"][0]
    nt = prob.ntotal
    errors = {"after_steps": nlong, "time_s": arms["fp64_plain"]["simulated_s"],
              "reference": "FP64 plain GPU path (bit-identical to the CPU oracle)"}
    for arm in ("fp32_surrogate", "fp32"):
        a, e = fields[arm][0], {}
        for k, sl in (("stress", slice(0, 4 * nt)), ("vel", slice(0, 2 * nt)),
                      ("displ", slice(None))):
            l2, li = rel_errors(a[k][sl], b[k][sl])
            e[k + "_rel_l2"], e[k + "_rel_linf"] = l2, li
        errors[arm] = e
    errors["plastic_stress_points_plain"] = int((b["intvars1"][prob.nnode:nt] > 0).sum())
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": arms["fp32_surrogate"]["value"],
            "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": arms["fp32_surrogate"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (generated biaxial sample, no dataset)",
            "config": {"workload": "biaxial sample 0.05 x 0.10 m at dx 0.1 mm, %d velocity + "
                                   "%d stress particles, platens 0.05 m/s"
                                   % (prob.nnode, prob.nstress),
                       "precision": "fp32 neighbour sums (Kahan), fp64 state and stress "
                                    "return, learned flow rule with exact fallback",
                       "l2": "state and pair tables larger than L2; no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "arms": arms, "surrogate": surr, "error_vs_plain": errors,
            "setup_s": round(setup_s, 1)}))


def run_combined(args):
    """The combined form: a batch of granular columns advanced by the FP32 form with the
    surrogate (exact fallback) and by the FP64 plain form, both as one batch context with a
    graph-launched step; particle-steps/s of each, the fallback rate, and the runout and
    field errors of the FP32 run against the plain run after the same steps."""
    import numpy as np
    import torch
    import sps_gb300
    from sps_gb300 import _abi
    from sps_gb300 import surrogate as sg
    rank, world, dist = dist_init("nccl")
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    sps_gb300.build_all()
    w0 = time.perf_counter()
    probs, phis = column_batch_problems(args.columns)
    probs, mine = shard(probs, dist)
    phis = [phis[i] for i in mine]
    n = reduce_sum(dist, sum(p.nnode + p.nstress for p in probs), device="cuda")
    nv_all = int(reduce_sum(dist, sum(p.nnode for p in probs), device="cuda"))
    net, env, training = train_surrogate(
        dx=0.005, make=lambda dx, m: sps_gb300.Problem.column(dx=dx, **dict(COLUMN, **m)),
        ranges=COLUMN_SURR_RANGES, geometry="column 0.5 x 0.25 m")
    setup_s = time.perf_counter() - w0

    def batch(prec):
        b = sps_gb300.Batch(probs, precision=prec)
        b.upload_all()
        return b

    arms, fields, surr = three_arms(args, batch, n, net, env, training, dist, local)
    nlong = max(args.combined_steps, max(args.warmup, 1) + args.steps)
    errors = {"after_steps": nlong, "time_s": arms["fp64_plain"]["simulated_s"],
              "reference": "FP64 plain GPU path (bit-identical to the CPU oracle)"}
    for arm in ("fp32_surrogate", "fp32"):
        per, pooled = [], {k: [0.0, 0.0] for k in ("stress", "vel", "displ")}
        for r, p in enumerate(probs):
            a, b = fields[arm][r], fields["fp64_plain"][r]
            nt, nn = p.nnode + p.nstress, p.nnode
            row = {"phi_deg": round(float(phis[r]), 3)}
            # runout: the front of the velocity particles (largest x) beyond the column
            fa, fb = float(a["x"][0:2 * nn:2].max()), float(b["x"][0:2 * nn:2].max())
            row["runout_plain_m"] = fb - COLUMN["width"]
            row["runout_abs_err_m"] = abs(fa - fb)
            for k, sl in (("stress", slice(0, 4 * nt)), ("vel", slice(0, 2 * nt)),
                          ("displ", slice(None))):
                d = a[k][sl] - b[k][sl]
                pooled[k][0] += float(np.dot(d, d))
                pooled[k][1] += float(np.dot(b[k][sl], b[k][sl]))
                row[k + "_rel_l2"] = float(np.linalg.norm(d) /
                                           max(np.linalg.norm(b[k][sl]), 1e-300))
            per.append(row)
        errors[arm] = {"pooled": {k + "_rel_l2": float(np.sqrt(v[0] / max(v[1], 1e-300)))
                                  for k, v in pooled.items()},
                       "max_runout_abs_err_m": max(r["runout_abs_err_m"] for r in per),
                       "per_column": per}
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": arms["fp32_surrogate"]["value"],
            "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": arms["fp32_surrogate"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (generated column geometry, no dataset)",
            "config": {"workload": "combined form: %d granular columns in one batch context "
                                   "per rank, %d particles (%d velocity) in all; %s"
                                   % (args.columns, n, nv_all,
                                      column_batch_problems.__doc__.split("\n")[0]),
                       "precision": "fp32 neighbour sums (Kahan), fp64 state and stress "
                                    "return, learned flow rule with exact fallback",
                       "l2": "state and pair tables larger than L2; no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "arms": arms, "surrogate": surr, "error_vs_plain": errors,
            "setup_s": round(setup_s, 1)}))


def workload(dx):
    import sps_gb300
    return sps_gb300.Problem.slope(dx=dx, **SLOPE)


def workload_name(prob, dx):
    return ("vertical slope 10 m (block 4.4 x 10 m) on a 20 x 5 m foundation, dx %.4g m, "
            "%d velocity + %d stress particles + %d wall dummies" % (dx, prob.nnode, prob.nstress,
                                                                     prob.ntotal2 - prob.ntotal))


# algorithmic bytes per target entry / particle for the roofline of each kernel class
# (FP64 plain layout): a neighbour entry is 16 B; per-particle state is counted once.
def kernel_bytes(name, prob, deg, fast=False):
    nn, ns, n2 = prob.nnode, prob.nstress, prob.ntotal2
    ent = 16.0
    # the node-node list is read by the derivative sums only for artificial viscosity
    visc = prob.params.alpha > 0 or prob.params.beta > 0
    if fast and name == "derivs":
        # entries + one 16 B record per neighbour-visible particle + per-particle FP64
        # state read/written once (SP: v, s, grad_u, RHS1, RKs, fdp, RKd; node: v, RHS2, RKv)
        return ent * deg["cross"] + (ent * deg["same_nodes"] if visc else 0) + \
            16 * (nn + ns) + ns * (16 + 32 + 32 + 32 + 64 + 16 + 16) + nn * (16 + 16 + 32 + 16)
    if fast and name == "interp":
        # the compact {id, W} entries (8 B) of the gathered lists
        return 8.0 * deg["cross"] + 16 * nn + 32 * ns + ns * 16 + nn * 40
    if name == "derivs":
        # entries + SP (v,s,m,rho,grad_u w, RHS1 w, RKs rw, fdp rw, RKd rw) + node terms
        return ent * deg["cross"] + ns * (16 + 32 + 16 + 32 + 32 + 64 + 16 + 16) + \
            nn * (16 + 32 + 16 + 16 + 32 + 16) + (ent * deg["same_nodes"] if visc else 0)
    if name == "interp":
        return ent * deg["cross"] + ns * (16 + 16) + nn * (40 + 16 + 16)
    if name == "half":
        return n2 * (4 * 8 + 8) + ent * deg["pairs"]
    if fast and name == "gather":
        # the FP32 form's direct lists: entries written (the same-kind lists' only when a
        # step kernel reads them) and the compact {id, W} copy of the cross entries (8 B),
        # and per particle its sorted record (16 + 8 B), its own offsets (20 B), ids, type,
        # realisation and cell (16 B), counts (12 B), target (4 B)
        p = prob.params
        same_written = p.xsph or p.art_stress or p.alpha > 0 or p.beta > 0
        return ent * (deg["cross"] + (deg["same"] if same_written else 0)) + \
            8.0 * deg["cross"] + n2 * 76
    if name == "lists":
        # entries written (the same-kind lists' only when a step kernel reads them: XSPH,
        # artificial viscosity or stress), and the creators' half-list entries read,
        # counted as half an entry per list entry (each pair's entry serves two lists)
        p = prob.params
        same_written = p.xsph or p.art_stress or p.alpha > 0 or p.beta > 0
        return ent * (deg["cross"] + (deg["same"] if same_written else 0)) + \
            0.5 * ent * (deg["cross"] + deg["same"])
    return None


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch group of the FP32
# form on the full-size slope (dx 0.012 m), from one ncu pass over the first timed stage
# (profiles/dram_traffic_fp32_slope_2M.md); the neighbour sums' group is the stress-point
# and the node launch of one stage, the gather's the two target kinds and the remaining
# positions.  Valid for that workload and this code state only.
NCU_TRAFFIC_FULL = {"derivs": 337793792 + 22539776 + 388249856 + 26990592,
                    "interp": 176712704 + 8054784 + 178151168 + 22437632,
                    "gather": 100680704 + 339088640 + 101198848 + 336080384 + 8663552}
NCU_TRAFFIC_SOURCE = ("ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum (1 pass), "
                      "FP32 form, this slope at dx 0.012 m, first timed stage")


def timed_steps(ctx, nsteps, t, dist, local, mark=False):
    """Device time (ms, max over ranks) of nsteps graph-launched steps on the context's
    own stream; clocks sampled meanwhile.  t: the start time (None for a batch, which keeps
    its own times).  mark: bracket the steps with cudaProfilerStart/Stop, so that a
    profiler started with --profile-from-start off captures exactly these launches."""
    import torch
    import sps_gb300
    stream = torch.cuda.ExternalStream(sps_gb300.stream_of(ctx))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(local)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    if mark:
        torch.cuda.cudart().cudaProfilerStart()
    e0.record(stream)
    t = ctx.step(nsteps) if t is None else ctx.step(nsteps, t)
    e1.record(stream)
    e1.synchronize()
    if mark:
        torch.cuda.cudart().cudaProfilerStop()
    clk = clocks.stop()
    torch.cuda.synchronize()
    barrier(dist)
    ms = reduce_max(dist, e0.elapsed_time(e1), device="cuda")
    return t, ms, clk


def rel_errors(a, b):
    import numpy as np
    d = a - b
    return (float(np.linalg.norm(d) / max(np.linalg.norm(b), 1e-300)),
            float(np.abs(d).max() / max(np.abs(b).max(), 1e-300)))


def e2e_through_abi(ctx, prob, nparticles, args, dist, world):
    """The metric end to end through the C-ABI with host buffers: every step uploads the
    state from pinned host memory, advances one step and brings the result to the host."""
    import numpy as np
    import torch
    st = prob.state()
    pinned = {}
    for k, v in st.items():
        tt = torch.empty(v.size, dtype=torch.float64 if v.dtype == np.float64 else torch.int32,
                         pin_memory=True)
        a = tt.numpy()
        a[:] = v
        pinned[k] = (tt, a)
    h2d = sum(a.nbytes for _, a in pinned.values())
    outs = {}
    for k, v in ctx.download().items():
        tt = torch.empty(v.size, dtype=torch.float64 if v.dtype == np.float64 else torch.int32,
                         pin_memory=True)
        outs[k] = (tt, tt.numpy())
    out = {k: a for k, (_, a) in outs.items()}
    d2h = sum(a.nbytes for a in out.values())
    inputs = {k: a for k, (_, a) in pinned.items()}
    ctx.upload(**inputs)
    torch.cuda.synchronize()

    def e2e_sync():
        te = 0.0
        for _ in range(args.e2e_steps):
            ctx.upload(**inputs)
            te = ctx.step(1, te)
            ctx.download(out=out)

    def e2e_pipelined():
        # the result of step k copies out to pinned host memory on the second stream while
        # step k+1's inputs copy in and step k+1 runs; the host reads it in place
        te = 0.0
        for k in range(args.e2e_steps):
            ctx.upload(**inputs)
            te = ctx.step(1, te)
            if k:
                ctx.snapshot_view()
            ctx.snapshot()
        ctx.snapshot_view()

    runs = {}
    for name, fn in (("sync", e2e_sync), ("pipelined", e2e_pipelined)):
        fn()  # warm-up (first-touch of the snapshot buffers)
        barrier(dist)
        w0 = time.perf_counter()
        fn()
        w1 = time.perf_counter()
        runs[name] = reduce_max(dist, w1 - w0, device="cuda")
    return {"value": round(nparticles * args.e2e_steps * world / runs["pipelined"], 1),
            "unit": "particle-steps/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "steps": args.e2e_steps,
            "path": "every step: sps_upload from pinned host arrays, sps_step(1), "
                    "sps_snapshot of the result (free surface, device pack in the download "
                    "layout, copy to pinned host memory on a second stream overlapping the "
                    "next step's upload and step), sps_snapshot_view of it on the host",
            "sync": {"value": round(nparticles * args.e2e_steps * world / runs["sync"], 1),
                     "path": "sps_upload + sps_step(1) + sps_download into pinned arrays"}}


def run_ours(args):
    import numpy as np
    import torch
    import sps_gb300
    from sps_gb300 import _abi

    rank, world, dist = dist_init("nccl")
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    sps_gb300.build_all()
    prob = workload(args.dx)
    nparticles = prob.nnode + prob.nstress
    fast = args.precision == "fast"
    prec = _abi.SPS_PREC_FP32_FAST if fast else _abi.SPS_PREC_FP64_PLAIN
    use_surr = fast and not args.no_surrogate
    surr = None
    e2e_settled = None
    if use_surr:
        from sps_gb300 import surrogate as sg
        net, env, training = train_surrogate()
    ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", prob.params_copy(precision=prec))
    ctx.upload_problem(prob)
    if use_surr:
        sg.install(ctx, net, tol=args.surrogate_tol, envelope=env)
        sg.set_gate(ctx, args.surrogate_gate)
    tuned = sps_gb300.autotune(ctx, 2)  # launch shapes; the state is restored
    if fast:
        tuned = dict(tuned, lookahead=sps_gb300.lookahead(ctx),
                     l2_prefetch=sps_gb300.prefetch(ctx))
    t = ctx.step(max(args.warmup, 1), 0.0)  # warm-up (also instantiates the step graph)
    kps = sps_gb300.kernels_per_step(ctx)
    if use_surr:
        sg.stats(ctx, reset=True)
        g0 = sg.gate_stats(ctx)
    t, ms_max, clk = timed_steps(ctx, args.steps, t, dist, local, mark=True)
    value = nparticles * args.steps * world / (ms_max * 1e-3)
    nsteps_done = max(args.warmup, 1) + args.steps
    f_head = ctx.download()  # the headline run's fields after nsteps_done steps
    # per-kernel profile of two steps (events around every kernel, no graph), right after
    # the timed steps, in their configuration
    t, prof = sps_gb300.profile_steps(ctx, 2, t)
    pairs = ctx.dump_pairs()
    pt = np.bincount(pairs["pint_type"], minlength=10)
    deg = {"cross": 2 * int(pt[1]) + int(pt[6] + pt[9]), "same": 2 * int(pt[2] + pt[3]),
           "same_nodes": 2 * int(pt[3]), "pairs": len(pairs["pair_i"])}
    top = max(prof, key=lambda k: prof[k][0])
    top_ms, top_n = prof[top]
    per_launch_ms = top_ms / top_n
    peaks, peak_kind = measured_peaks()
    b = kernel_bytes(top, prob, deg, fast)
    full_size = fast and abs(args.dx - 0.012) < 1e-12
    roof = None
    if b is not None:
        ach = b / (per_launch_ms * 1e-3) / 1e9
        # a profiled region holds the launches of one phase: the neighbour sums launch once
        # for the stress-point targets and once for the node targets, back to back
        label = {"derivs": "k_fderivs<1> + k_fderivs<2>" if fast else "k_derivs (both kinds)",
                 "interp": "k_finterp<1> + k_finterp<2>" if fast else "k_interp (both kinds)",
                 "gather": "k_fgather<1> + k_fgather<2> + k_fgather_rest"}
        roof = {"kernel": label.get(top, "k_" + top), "bound": "hbm", "achieved": round(ach, 1),
                "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                "frac": round(ach / peaks.get("hbm_gbs"), 4),
                "traffic": NCU_TRAFFIC_FULL[top] if full_size and top in NCU_TRAFFIC_FULL
                else None,
                "traffic_source": NCU_TRAFFIC_SOURCE if full_size and top in NCU_TRAFFIC_FULL
                else None,
                "peak_kind": peak_kind, "algorithmic_bytes_per_launch": int(b),
                "per_launch_ms": round(per_launch_ms, 4), "launches_per_step": top_n / 2,
                "launch": "one RK stage's stress-point and node launches together"
                if top in label else "one launch",
                "share_of_step": round(top_ms / sum(v[0] for v in prof.values()), 3)}
    alg_bytes = {k: int(v) for k in prof for v in [kernel_bytes(k, prob, deg, fast)]
                 if v is not None}
    try:
        f64 = fp64_peak_tflops()
    except Exception:
        f64 = None

    if use_surr:
        loading, answered, outside, rejected = sg.stats(ctx)
        g1 = sg.gate_stats(ctx)
        lf = max(loading, 1)
        surr = {"tol": args.surrogate_tol,
                "drift_test": "dt |grad f : (D:e + Gs)| / sqrt(J2) <= tol",
                "training": training,
                "gate": {"min_answered": args.surrogate_gate, "max_period": 1024,
                         "timed_steps_with_network": g1[0] - g0[0],
                         "timed_steps_without": g1[1] - g0[1]},
                "timed_loading_evaluations_with_network": loading,
                "answered_frac": round(answered / lf, 6),
                "outside_envelope_frac": round(outside / lf, 6),
                "drift_rejected_frac": round(rejected / lf, 6),
                "fallback_rate": round(1.0 - answered / lf, 6)}
        # the same context without the network (same launch shapes, state and size), then
        # the network installed again for the rest of the run
        sg.install(ctx, None)
        t = ctx.step(2, t)
        t, ms_n, _ = timed_steps(ctx, args.steps, t, dist, local)
        surr["same_context_without_network"] = {
            "value": round(nparticles * args.steps * world / (ms_n * 1e-3), 1),
            "ms_per_step": round(ms_n / args.steps, 4)}
        surr["speed_with_over_without"] = round(ms_n / ms_max, 4)
        sg.install(ctx, net, tol=args.surrogate_tol, envelope=env)
        sg.set_gate(ctx, args.surrogate_gate)
        # the same comparison once the gate has settled: 500 steps with the network first
        # (its tries are then hundreds of steps apart), then the timed steps with and
        # without it from the same state
        if args.steady_steps > 0:
            t = ctx.step(args.steady_steps, t)
            g2 = sg.gate_stats(ctx)
            t, ms_s, _ = timed_steps(ctx, args.steps, t, dist, local)
            g3 = sg.gate_stats(ctx)
            sg.install(ctx, None)
            t = ctx.step(2, t)
            t, ms_s0, _ = timed_steps(ctx, args.steps, t, dist, local)
            surr["settled"] = {
                "after_steps": args.steady_steps, "ms_per_step_with": round(ms_s / args.steps, 4),
                "ms_per_step_without": round(ms_s0 / args.steps, 4),
                "timed_steps_with_network": g3[0] - g2[0],
                "speed_with_over_without": round(ms_s0 / ms_s, 4)}
            sg.install(ctx, net, tol=args.surrogate_tol, envelope=env)
            sg.set_gate(ctx, args.surrogate_gate)
            # the end-to-end loop with the gate settled too (installing restarts it: its
            # tries would otherwise fall into the few timed steps); each step uploads the
            # problem's state again, the gate runs on
            t = ctx.step(args.steady_steps, t)
            g4 = sg.gate_stats(ctx)
            e2e_settled = e2e_through_abi(ctx, prob, nparticles, args, dist, world)
            e2e_settled["steps_with_network"] = sg.gate_stats(ctx)[0] - g4[0]

    plain = None
    errors = None
    if fast:
        # the FP64 plain form on the same workload, advanced by the same number of steps
        cp = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                   prob.params_copy(precision=_abi.SPS_PREC_FP64_PLAIN))
        cp.upload_problem(prob)
        tp = cp.step(max(args.warmup, 1), 0.0)
        tp, ms_p, _ = timed_steps(cp, args.steps, tp, dist, local)
        plain = {"value": round(nparticles * args.steps * world / (ms_p * 1e-3), 1),
                 "ms_per_step": round(ms_p / args.steps, 4), "dtype": "f64"}
        ff, fp = f_head, cp.download()
        nt = prob.ntotal

        def errs(a, b):
            sl2, sli = rel_errors(a["stress"][:4 * nt], b["stress"][:4 * nt])
            vl2, vli = rel_errors(a["vel"][:2 * nt], b["vel"][:2 * nt])
            dl2, dli = rel_errors(a["displ"], b["displ"])
            return {"after_steps": nsteps_done, "time_s": t,
                    "stress_rel_l2": sl2, "stress_rel_linf": sli, "vel_rel_l2": vl2,
                    "vel_rel_linf": vli, "displ_rel_l2": dl2, "displ_rel_linf": dli,
                    "reference": "FP64 plain GPU path (bit-identical to the CPU oracle)"}
        errors = errs(ff, fp)
        if use_surr:
            # the FP32 form without the surrogate, same workload and steps
            cn = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                       prob.params_copy(precision=_abi.SPS_PREC_FP32_FAST))
            cn.upload_problem(prob)
            cn.step(nsteps_done, 0.0)
            surr["fp32_without_surrogate"] = {"error_vs_plain": errs(cn.download(), fp)}
            cn.close()
        _, prof_p = sps_gb300.profile_steps(cp, 1, tp)
        plain["kernel_ms_per_step"] = {k: round(v[0], 4) for k, v in sorted(
            prof_p.items(), key=lambda kv: -kv[1][0])[:6]}

    # end to end through the C-ABI with pinned host buffers (with the surrogate: measured
    # above, once its gate had settled; re-installing the network restarts the gate, whose
    # first tries would otherwise fall into the few timed steps)
    e2e = e2e_settled if e2e_settled is not None else \
        e2e_through_abi(ctx, prob, nparticles, args, dist, world)
    if fast:
        cp.upload_problem(prob)
        plain["e2e"] = e2e_through_abi(cp, prob, nparticles, args, dist, world)
        cp.close()

    batch = None
    if fast and not args.no_batch:
        batch = run_batch(args, dist, local)

    fixed = None
    if fast and rank == 0 and args.error_at > 0:
        m = steps_to_time(prob, args.error_at)
        w0 = time.perf_counter()
        rows, counters = error_rows(args, prob, [m], net if use_surr else None,
                                    env if use_surr else None)
        fixed = dict(rows[0], wall_s=round(time.perf_counter() - w0, 1),
                     reference="FP64 plain GPU path (bit-identical to the CPU oracle)",
                     floor="FP64 plain from initial stresses perturbed by 2^-52 relative")
        if counters is not None:
            fixed["surrogate"] = counters

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 1), "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms_max / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if fast else "f64",
            "data": "synthetic (generated slope geometry, no dataset)",
            "config": {"workload": workload_name(prob, args.dx),
                       "precision": ("fp32 neighbour sums (Kahan), fp64 state and stress return"
                                     if fast else "fp64 plain (reference rounding)"),
                       "particles": nparticles, "pairs": deg["pairs"],
                       "l2": "state and pair tables (%.1f GB) larger than L2; no flush" % (
                           (prob.ntotal2 * (3 * 48 * 16 + 400)) / 1e9),
                       "surrogate": ("learned Drucker-Prager flow rule, exact fallback "
                                     "(tol %g)" % args.surrogate_tol if use_surr else "off"),
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "free_surface": "the timed steps skip get_nodes_on_free_surface, which "
                                       "nothing in this workload's step reads; e2e detects it "
                                       "for every step's output (in FP32 in the FP32 form)"},
            "plain": plain, "error_vs_plain": errors, "error_at_fixed_time": fixed,
            "surrogate": surr, "batch": batch,
            "e2e": e2e, "gpu_launches": int(kps * args.steps), "roofline": roof,
            "autotuned_blocks": tuned, "algorithmic_bytes_per_launch": alg_bytes,
            "fp64": None if f64 is None else {"dgemm_peak_tflops": round(f64, 2)},
            "kernel_ms_per_step": {k: round(v[0] / 2, 4) for k, v in sorted(
                prof.items(), key=lambda kv: -kv[1][0])},
            "cpu_baseline": cpu, "clocks": clk,
        }
        print(json.dumps(line))


def cpu_sample(seconds_target=20.0):
    """The oracle (single-threaded restatement of the reference step) on a coarser slope of
    the same geometry and material, timed for a bounded number of steps."""
    import orc
    import sps_gb300
    dx = 0.06
    prob = sps_gb300.Problem.slope(dx=dx, **SLOPE)
    ctx = orc.context(prob.params_copy())
    ctx.upload_problem(prob)
    t = ctx.step(1, 0.0)
    steps, el = 0, 0.0
    while el < seconds_target and steps < 200:
        w0 = time.perf_counter()
        t = ctx.step(1, t)
        el += time.perf_counter() - w0
        steps += 1
    n = prob.nnode + prob.nstress
    return n * steps / el, "oracle (C restatement, 1 thread) on the same slope at dx %.3g m: " \
        "%d velocity + %d stress particles, %d steps in %.1f s" % (dx, prob.nnode, prob.nstress,
                                                                   steps, el), steps


def cpu_baseline(args):
    v, sample, _ = cpu_sample()
    return {"value": round(v, 1), "unit": "particle-steps/s", "cores": 1, "kind": "port",
            "sample": sample}


# peak resident memory of one oracle replica per particle slot (ntotal2): 2.46 GB measured
# for the 2.01M-slot slope, interpreter included; rounded up
REF_BYTES_PER_PARTICLE = 1500
REF_BYTES_FIXED = 200 << 20


def host_memory_available():
    """Bytes this process may still allocate: MemAvailable from /proc/meminfo, lowered to
    the cgroup's remaining limit (v2 memory.max - memory.current, or v1
    memory.limit_in_bytes - memory.usage_in_bytes) where one is set.  None if unknown."""
    avail = None
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    avail = int(line.split()[1]) * 1024
    except OSError:
        pass
    for lim_f, cur_f in (("/sys/fs/cgroup/memory.max", "/sys/fs/cgroup/memory.current"),
                         ("/sys/fs/cgroup/memory/memory.limit_in_bytes",
                          "/sys/fs/cgroup/memory/memory.usage_in_bytes")):
        try:
            lim = open(lim_f).read().strip()
            cur = int(open(cur_f).read().strip())
        except (OSError, ValueError):
            continue
        if lim.isdigit() and int(lim) < (1 << 60):
            left = max(0, int(lim) - cur)
            avail = left if avail is None else min(avail, left)
        break
    return avail


def reference_replicas(ntotal2, cores, avail):
    """How many single-threaded replicas of the reference step run side by side: one per
    core, as many as fit in 60% of the available memory at the measured footprint per
    particle slot, at least one."""
    n = max(1, cores)
    if avail is not None:
        per = REF_BYTES_FIXED + REF_BYTES_PER_PARTICLE * ntotal2
        n = min(n, int(0.6 * avail) // per)
    return max(1, n)


def _ref_replica(dx, warm, steps, barrier, q):
    """One realisation of the workload on one core (a spawned process): warm-up steps,
    then the timed steps, started together with the other replicas at the barrier."""
    try:
        import orc
        prob = workload(dx)
        ctx = orc.context(prob.params_copy())
        ctx.upload_problem(prob)
        t = ctx.step(warm, 0.0) if warm else 0.0
        barrier.wait(timeout=1800)
        w0 = time.perf_counter()
        ctx.step(steps, t)
        q.put(("ok", time.perf_counter() - w0, prob.nnode + prob.nstress))
    except BaseException as e:  # reported to the parent, which fails the run
        barrier.abort()
        q.put(("error", repr(e), 0))


def run_reference(args):
    """The reference's CPU implementation of the step on the same workload as the GPU arm:
    the oracle (the C restatement of the reference's single-threaded Fortran step; no
    Fortran compiler exists on either machine) on the full slope.  The step is single-
    threaded, so the host's cores are used as independent replicas of the workload, one
    per core (bounded by the host memory), which start their timed steps together; the
    value is all replicas' particle-steps over the slowest replica's time.  A step takes
    about a minute, so the timed steps are bounded: min(warmup, 1) untimed and
    min(steps, 2) timed."""
    rank, world, dist = dist_init("gloo")
    if rank != 0:
        return
    import multiprocessing as mp
    import orc
    orc.build()
    import sps_gb300
    sps_gb300.build_host()
    prob = workload(args.dx)
    n = prob.nnode + prob.nstress
    name = workload_name(prob, args.dx)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    reps = args.ref_replicas or reference_replicas(prob.ntotal2, cores or 1, host_memory_available())
    del prob
    warm, steps = min(args.warmup, 1), max(1, min(args.steps, 2))
    ctx = mp.get_context("spawn")
    barrier, q = ctx.Barrier(reps), ctx.Queue()
    procs = [ctx.Process(target=_ref_replica, args=(args.dx, warm, steps, barrier, q))
             for _ in range(reps)]
    for p in procs:
        p.start()
    res, deadline = [], time.time() + 3600
    try:
        while len(res) < reps:
            try:
                res.append(q.get(timeout=5))
            except queue.Empty:
                # a replica that ended without reporting (killed, crashed) fails the run
                dead = [p.exitcode for p in procs if p.exitcode not in (None, 0)]
                if dead or time.time() > deadline:
                    barrier.abort()
                    raise RuntimeError("reference replica ended without a result (exit codes "
                                       "%s)" % dead if dead else "reference replicas timed out")
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.terminate()
    bad = [r[1] for r in res if r[0] != "ok"]
    if bad:
        raise RuntimeError("reference replica failed: " + bad[0])
    el = max(r[1] for r in res)
    v = reps * n * steps / el
    sample = ("oracle (C restatement of the reference step; single-threaded, as the reference "
              "runs) on the same workload, %d replica(s) on %d host core(s), one each: %d untimed "
              "+ %d timed steps per replica, slowest replica %.3g s"
              % (reps, cores, warm, steps, el))
    line = {
        "metric": METRIC, "value": round(v, 1), "unit": "particle-steps/s", "n_gpus": world,
        "steps": steps, "warmup": warm, "ms_per_step": round(1e3 * el / steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (generated slope geometry, no dataset)", "impl": "reference",
        "config": {"workload": name,
                   "precision": "fp64 (reference mixed precision)",
                   "particles": n, "same_as_gpu_arm": True, "replicas": reps,
                   "bounded": "steps limited to min(K, 2) after min(W, 1) warm-up (about a "
                              "minute per step on one core)"},
        "cpu_baseline": {"value": round(v, 1), "unit": "particle-steps/s", "cores": reps,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(v, 1), "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def steps_to_time(prob, ts):
    """The step whose FP64 time (a sum of dt, as the step loop adds it) first reaches ts."""
    tt, k = 0.0, 0
    while tt < ts:
        tt += prob.params.dt_sph
        k += 1
    return k


def error_rows(args, prob, marks, net=None, env=None):
    """Relative L2 / Linf errors against the FP64 plain form at the given step counts, for
    the FP32 form, the FP32 form with the surrogate (when a network is given) and the
    "floor": the FP64 plain form again, from initial stresses perturbed by a relative 2^-52
    (one FP64 rounding), i.e. how far two runs that differ by rounding drift apart.  Returns
    (rows, surrogate counters or None)."""
    import numpy as np
    import sps_gb300
    from sps_gb300 import _abi
    arms = [("plain", _abi.SPS_PREC_FP64_PLAIN), ("fp32", _abi.SPS_PREC_FP32_FAST),
            ("floor", _abi.SPS_PREC_FP64_PLAIN)]
    if net is not None:
        from sps_gb300 import surrogate as sg
        arms.append(("fp32_surrogate", _abi.SPS_PREC_FP32_FAST))
    ctxs = {}
    for name, prec in arms:
        ctxs[name] = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps",
                                           prob.params_copy(precision=prec))
        st = prob.state()
        if name == "floor":
            rng = np.random.default_rng(1)
            st["stress"] = st["stress"] * (1.0 + 2.0 ** -52 * rng.uniform(-1, 1, st["stress"].shape))
        ctxs[name].upload(**st)
        ctxs[name].upload_bcs(prob.bc_or_not, prob.bc_info)
        if name == "fp32_surrogate":
            sg.install(ctxs[name], net, tol=args.surrogate_tol, envelope=env)
            sg.set_gate(ctxs[name], args.surrogate_gate)
    nt = prob.ntotal
    out, done, t = [], 0, {k: 0.0 for k in ctxs}
    for m in sorted(marks):
        for name, c in ctxs.items():
            t[name] = c.step(m - done, t[name])
        done = m
        b = ctxs["plain"].download()
        row = {"steps": m, "time_s": t["plain"]}
        for arm in [a for a, _ in arms if a != "plain"]:
            a = ctxs[arm].download()
            for k, sl in (("stress", slice(0, 4 * nt)), ("vel", slice(0, 2 * nt)),
                          ("displ", slice(None))):
                l2, li = rel_errors(a[k][sl], b[k][sl])
                row[arm + "_" + k + "_rel_l2"] = l2
                row[arm + "_" + k + "_rel_linf"] = li
        out.append(row)
    counters = None
    if net is not None:
        c = ctxs["fp32_surrogate"]
        loading, answered, outside, rejected = sg.stats(c)
        counters = {"steps_with_and_without_network": sg.gate_stats(c),
                    "loading_evaluations_with_network": loading, "answered": answered}
    for c in ctxs.values():
        c.close()
    return out, counters


def run_errors(args):
    """FP32 form (optionally with the surrogate) against the FP64 plain form over a long
    run of the slope workload, with relative L2 / Linf errors at checkpoints."""
    import sps_gb300
    sps_gb300.build_all()
    prob = workload(args.dx)
    net = env = None
    if not args.no_surrogate:
        net, env, training = train_surrogate()
    n = args.error_steps
    marks = {max(1, n * k // 20) for k in range(1, 21)}
    for ts in [float(v) for v in args.error_times.split(",") if v.strip()]:
        marks.add(min(n, steps_to_time(prob, ts)))
    w0 = time.perf_counter()
    out, counters = error_rows(args, prob, marks, net, env)
    extra = {}
    if counters is not None:
        extra["surrogate"] = dict({"tol": args.surrogate_tol, "training": training}, **counters)
    print(json.dumps({"error_run": dict({"workload": workload_name(prob, args.dx),
                                         "reference": "FP64 plain GPU path (bit-identical to "
                                                      "the CPU oracle)",
                                         "checkpoints": out,
                                         "wall_s": round(time.perf_counter() - w0, 1)}, **extra)}))


def main():
    args = parse()
    if args.error_steps > 0:
        run_errors(args)
        return
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "column-batch":
        run_combined(args)
    elif args.workload == "biaxial":
        run_biaxial(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
