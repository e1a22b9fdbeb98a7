"""sps_run (csrc/host/sps_run.cpp), the reference's main program over the C-ABI, on CPU.

The driver is linked here against a fake of the step library (the same C-ABI: it keeps the
uploaded state, advances time_sph by dt_sph, counts the steps and can return an error at a
chosen step), so that its loop -- the input's blocks, the FP32 output-cadence counters,
the stop at time_end, OutputRes / Out_print_sph and the error paths -- is checked without
a GPU against a restatement of code/1_SPH_2018.f90:50-106.  The real build is run once to
check that it refuses cleanly when no CUDA device is visible.
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
SRC = os.path.join(ROOT, "stress-particle-sph_gb300", "csrc", "host", "sps_run.cpp")
SP1 = os.path.join(ROOT, "tests", "golden", "example_problems", "soil_failure_bui_et_al_2008",
                   "inside_approach", "SP1")

FAKE = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sps.h"
struct sps_ctx {
  sps_params p;
  int n2, nt, nn;
  double *x, *vel, *stress, *rho, *iv1, *fdp, *x00;
  int *bc;
  long steps, fail_at;
  char err[128];
};
static double* dup(const double* s, size_t n) {
  double* d = (double*)calloc(n ? n : 1, sizeof(double));
  if (s) memcpy(d, s, n * sizeof(double));
  return d;
}
int sps_create(const sps_params* p, sps_ctx** out) {
  sps_ctx* c = (sps_ctx*)calloc(1, sizeof(sps_ctx));
  c->p = *p;
  c->nn = p->nnode;
  c->nt = p->nnode + p->nstress;
  c->n2 = c->nt + p->ndummy;
  const char* f = getenv("FAKE_FAIL_AT");
  c->fail_at = f ? atol(f) : 0;
  fprintf(stderr, "fake: create precision %d bc_nodes_only %d cspm_det_min %.17g\n",
          p->precision, p->bc_nodes_only, p->cspm_det_min);
  *out = c;
  return SPS_OK;
}
int sps_upload(sps_ctx* c, const double* x, const double* vel, const double* stress,
               const double* mass, const double* rho, const double* hsml, const int32_t* itype,
               const double* iv1, const double* fdp, const double* x00) {
  c->x = dup(x, 2 * c->n2); c->vel = dup(vel, 2 * c->n2); c->stress = dup(stress, 4 * c->n2);
  c->rho = dup(rho, c->n2); c->iv1 = dup(iv1, c->nt); c->fdp = dup(fdp, c->nt);
  c->x00 = dup(x00, 2 * c->n2);
  return SPS_OK;
}
int sps_upload_bcs(sps_ctx* c, const int32_t* bc, const int32_t* info) {
  c->bc = (int*)calloc(c->nt, sizeof(int));
  memcpy(c->bc, bc, c->nt * sizeof(int));
  return SPS_OK;
}
int sps_step(sps_ctx* c, int32_t n, double* t) {
  for (int k = 0; k < n; k++) {
    c->steps++;
    if (c->fail_at && c->steps == c->fail_at) {
      snprintf(c->err, sizeof c->err, "fake: non-finite state after step %ld", c->steps);
      return SPS_ERR_NONFINITE;
    }
    *t = *t + c->p.dt_sph;
    c->x[2 * (c->nn - 1)] += 1.0;  /* the last node moves 1 m a step */
  }
  return SPS_OK;
}
int sps_download(sps_ctx* c, double* x, double* vel, double* stress, double* rho,
                 double* iv1, double* displ, int32_t* bc, double* fdp) {
  if (x) memcpy(x, c->x, 2 * c->n2 * sizeof(double));
  if (vel) memcpy(vel, c->vel, 2 * c->n2 * sizeof(double));
  if (stress) memcpy(stress, c->stress, 4 * c->n2 * sizeof(double));
  if (rho) memcpy(rho, c->rho, c->n2 * sizeof(double));
  if (iv1) memcpy(iv1, c->iv1, c->nt * sizeof(double));
  if (fdp) memcpy(fdp, c->fdp, c->nt * sizeof(double));
  if (bc) memcpy(bc, c->bc, c->nt * sizeof(int));
  if (displ)
    for (int i = 0; i < 2 * c->nn; i++) displ[i] = c->x[i] - c->x00[i];
  return SPS_OK;
}
int sps_last_error(sps_ctx* c, char* buf, int32_t len) {
  snprintf(buf, len, "%s", c ? c->err : "fake: no context");
  return SPS_OK;
}
void sps_destroy(sps_ctx* c) {
  fprintf(stderr, "fake: %ld steps\n", c->steps);
  free(c->x); free(c->vel); free(c->stress); free(c->rho); free(c->iv1); free(c->fdp);
  free(c->x00); free(c->bc); free(c);
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    """sps_run linked against the fake step library and the real host library."""
    import sps_gb300
    host = sps_gb300.build_host()
    d = tmp_path_factory.mktemp("fake")
    (d / "fake.c").write_text(FAKE)
    subprocess.run(["gcc", "-O1", "-fPIC", "-shared", "-I" + INCLUDE, "-o",
                    str(d / "libsps_gb300.so"), str(d / "fake.c")], check=True)
    exe = d / "sps_run"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-I" + INCLUDE,
                    "-o", str(exe), SRC, "-L" + str(d), "-L" + os.path.dirname(host),
                    "-lsps_gb300", "-lsph_host",
                    "-Wl,-rpath," + str(d) + ":" + os.path.dirname(host)],
                   check=True)
    return str(exe)


def problem_dir(tmp_path, blocks):
    """SP1's input set with its run-control lines replaced by `blocks`:
    [(dt, time_end, maxtimestep, print, save, plot)]."""
    d = tmp_path / "prob"
    shutil.copytree(SP1, d)
    text = (d / "input.txt").read_text().splitlines()
    k = text.index("time step, time for end, max number of time steps")
    run = []
    for dt, t_end, nmax, pr, sv, pl in blocks:
        run += ["time step, time for end, max number of time steps",
                "%r,%r,%d" % (dt, t_end, nmax), "print, save, plot", "%d,%d,%d" % (pr, sv, pl)]
    run += ["if end of simulation:", "-1,1,1", ""]
    (d / "input.txt").write_text("\n".join(text[:k] + run) + "\n")
    return str(d)


def expected(blocks):
    """code/1_SPH_2018.f90:50-106: the steps taken, the steps whose results OutputRes writes
    and those Out_print_sph prints.  The cadence counters are FP32 (`real`)."""
    time, its, plots, prints = 0.0, 0, [], []
    for dt, t_end, nmax, pr, _, pl in blocks:
        plots.append(its)  # OutputRes at the start of the block
        tp, tl = np.float32(pr * dt), np.float32(pl * dt)
        rp = rl = np.float32(0.0)
        for _ in range(nmax):
            rp = np.float32(np.float64(rp) + dt)
            rl = np.float32(np.float64(rl) + dt)
            its += 1
            time = time + dt
            if time > t_end:
                break
            if rl >= tl:
                plots.append(its)
                rl = np.float32(0.0)
            if rp >= tp:
                prints.append(its)
                rp = np.float32(0.0)
    return its, plots, prints


def run(driver, pdir, out, *extra, env=None):
    os.makedirs(out, exist_ok=True)
    return subprocess.run([driver, pdir, "-o", str(out)] + list(extra), capture_output=True,
                          text=True, timeout=300, env=dict(os.environ, **(env or {})))


def outputs(out):
    return sorted(int(f.split(".")[-1]) for f in os.listdir(out) if f.startswith("nodes.csv."))


def printed(out):
    text = open(os.path.join(out, "output.txt")).read()
    return [int(m) for m in re.findall(r"time step_sph is (\d+)", text)], text


@pytest.mark.parametrize("blocks", [
    # one block: print every 2 steps, plot every 3, ended by time_end before maxtimestep
    [(0.00015, 0.0024, 40, 2, 1, 3)],
    # two blocks with the same dt: time and the step count carry over
    [(0.00015, 0.0015, 5, 3, 1, 2), (0.00015, 0.003, 4, 1, 1, 1)],
    # the standard_sph example's dt and cadence: the FP32 counters reach 100 dt only after
    # 101 steps, so the reference writes steps 101, 202, ... (not 100, 200)
    [(0.00015, 2.5, 250, 100, 1, 100)],
], ids=["one_block", "two_blocks", "fp32_counters"])
def test_loop_and_cadence(driver, tmp_path, blocks):
    r = run(driver, problem_dir(tmp_path, blocks), tmp_path / "out")
    assert r.returncode == 0, r.stderr
    its, plots, prints = expected(blocks)
    if blocks[0][3] == 100:
        assert plots == [0, 101, 202] and prints == [101, 202]
    assert "fake: %d steps" % its in r.stderr
    assert outputs(tmp_path / "out") == sorted(set(plots))
    got, text = printed(tmp_path / "out")
    assert got == prints
    # Out_print_sph: time_sph after the step and the last node's position (the fake moves it
    # 1 m a step)
    dt = blocks[0][0]
    x0 = None
    for it, line in zip(got, [l for l in text.splitlines() if "time step_sph is" in l]):
        t = float(re.search(r"time_sph = (\S+)", line).group(1))
        assert t == pytest.approx(it * dt, rel=1e-12)
    xs = [float(l.split()[0]) for l in text.splitlines()[3::5]]
    if len(xs) >= 2:
        x0 = xs[0] - got[0]
        assert xs == pytest.approx([x0 + it for it in got])


def test_options_reach_the_params(driver, tmp_path):
    blocks = [(0.00015, 2.5, 2, 1, 1, 1)]
    r = run(driver, problem_dir(tmp_path, blocks), tmp_path / "out", "--fast",
            "--bc-nodes-only", "1", "--cspm-det-min", "0.001")
    assert r.returncode == 0, r.stderr
    assert "precision 1 bc_nodes_only 1 cspm_det_min 0.001" in r.stderr
    r = run(driver, problem_dir(tmp_path / "b", blocks), tmp_path / "out2")
    assert "precision 0 " in r.stderr


def test_block_with_another_dt_is_refused(driver, tmp_path):
    blocks = [(0.00015, 2.5, 3, 1, 1, 1), (0.0003, 2.5, 3, 1, 1, 1)]
    r = run(driver, problem_dir(tmp_path, blocks), tmp_path / "out")
    assert r.returncode == 1
    assert "block 2 has dt" in r.stderr and "fake: 3 steps" in r.stderr


def test_step_error_is_reported(driver, tmp_path):
    blocks = [(0.00015, 2.5, 10, 1, 1, 1)]
    r = run(driver, problem_dir(tmp_path, blocks), tmp_path / "out", env={"FAKE_FAIL_AT": "4"})
    assert r.returncode == 1
    assert "sps_step failed (-5): fake: non-finite state after step 4" in r.stderr
    # the results of steps 0-3 were written, nothing after the failing step
    assert outputs(tmp_path / "out") == [0, 1, 2, 3]


def test_usage_and_bad_input(driver, tmp_path):
    assert subprocess.run([driver], capture_output=True).returncode == 2
    assert subprocess.run([driver, SP1, "--bc-nodes-only", "2"],
                          capture_output=True).returncode == 2
    r = subprocess.run([driver, str(tmp_path / "missing")], capture_output=True, text=True)
    assert r.returncode == 1 and "sps_run:" in r.stderr


def test_real_build_refuses_without_a_device(tmp_path):
    import sps_gb300
    exe = sps_gb300.build.build_driver()
    r = subprocess.run([exe, SP1, "-o", str(tmp_path)], capture_output=True, text=True,
                       timeout=120, env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode == 1
    assert "sps_create failed (-3)" in r.stderr
