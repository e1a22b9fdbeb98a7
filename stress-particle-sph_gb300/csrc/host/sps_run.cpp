// sps_run.cpp -- the reference's main program (code/1_SPH_2018.f90:30-106) over the C-ABI,
// for a caller without a Fortran compiler.
//
//   sps_run <problem_dir> [-o <out_dir>] [--fast] [--bc-nodes-only 0|1]
//           [--cspm-det-min <x>]
//
// Reads the problem directory (input.txt, <name>.dat, <name>.pts) with sph_problem_read,
// uploads its state into a step context and runs the input's (dt, time_end, maxtimestep)
// blocks as the Fortran loop does:
//   - OutputRes at the start of every block (files numbered by itimestep_sph);
//   - per step: the FP32 cadence counters t_plot_reset / t_print_reset advance by dt (an
//     FP64 sum rounded to FP32, as `real` variables are in 6_SPH_time_vars_2018.f90:31-36),
//     sps_step advances time_sph (time_integration + time_sph = time_sph + dt_sph), and
//     the run leaves the block once time > time_end (after that step, before its output);
//   - out_plot (OutputRes) when t_plot_reset >= time_plot, out_prn (Out_print_sph,
//     2_SPH_main_2018.f90:51-73, into <out_dir>/output.txt) when t_print_reset >= time_print.
// The fields OutputRes writes are downloaded from the device first; the smoothing length
// written is the problem's (sps_download has no h: with sle = 2 the written h is the
// initial one).  A block whose dt differs from the first block's is refused: the step
// context keeps dt_sph, and a new context would restart the pair list's reuse order.
// --fast selects the FP32 form.  --bc-nodes-only and --cspm-det-min set two constants that
// differ between the reference's source copies and that no input file holds: whether
// Normal_BCs loops over the nodes only (1: code/ and the strain-localisation copy) or over
// all particles (0: the Drucker-Prager and vertical-slope copies), and the CSPM determinant
// below which get_derivatives skips the correction (1e-7 in the Drucker-Prager copy, 1e-3
// elsewhere, both FP32 literals).
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sph_host.h"
#include "sps.h"

namespace {

struct Args {
  std::string dir, out = ".";
  bool fast = false;
  int bc_nodes_only = -1;
  double cspm_det_min = -1.0;
};

int usage() {
  std::fprintf(stderr,
               "usage: sps_run <problem_dir> [-o <out_dir>] [--fast] [--bc-nodes-only 0|1] "
               "[--cspm-det-min <x>]\n");
  return 2;
}

bool parse(int argc, char** argv, Args& a) {
  for (int i = 1; i < argc; i++) {
    std::string s = argv[i];
    auto value = [&](const char* name) -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "sps_run: %s needs a value\n", name);
        return nullptr;
      }
      return argv[++i];
    };
    if (s == "-o") {
      const char* v = value("-o");
      if (!v) return false;
      a.out = v;
    } else if (s == "--fast") {
      a.fast = true;
    } else if (s == "--bc-nodes-only") {
      const char* v = value("--bc-nodes-only");
      if (!v || (std::strcmp(v, "0") && std::strcmp(v, "1"))) return false;
      a.bc_nodes_only = v[0] - '0';
    } else if (s == "--cspm-det-min") {
      const char* v = value("--cspm-det-min");
      if (!v) return false;
      char* end = nullptr;
      errno = 0;
      a.cspm_det_min = std::strtod(v, &end);
      if (errno || !end || *end || !(a.cspm_det_min >= 0.0)) return false;
    } else if (!s.empty() && s[0] == '-') {
      std::fprintf(stderr, "sps_run: unknown option %s\n", s.c_str());
      return false;
    } else if (a.dir.empty()) {
      a.dir = s;
    } else {
      return false;
    }
  }
  return !a.dir.empty();
}

// the device state in the reference layout, as sps_download returns it
struct Fields {
  std::vector<double> x, vel, stress, rho, iv1, displ, fdp;
  std::vector<int32_t> bc;
  Fields(const sps_params& p, int32_t ntotal2) {
    const size_t nt = (size_t)p.nnode + p.nstress;
    x.resize(2 * (size_t)ntotal2);
    vel.resize(2 * (size_t)ntotal2);
    stress.resize(4 * (size_t)ntotal2);
    rho.resize(ntotal2);
    iv1.resize(nt);
    displ.resize(2 * (size_t)p.nnode);
    fdp.resize(nt);
    bc.resize(nt);
  }
};

class Run {
 public:
  Run(const Args& a, sph_problem* prob, const sps_params& p, const sph_problem_arrays& arr)
      : a_(a), prob_(prob), p_(p), arr_(arr), f_(p, arr.ntotal2) {}
  ~Run() {
    if (ctx_) sps_destroy(ctx_);
    if (prn_) std::fclose(prn_);
  }

  int main() {
    if (fail(sps_create(&p_, &ctx_), "sps_create")) return 1;
    if (fail(sps_upload(ctx_, arr_.x, arr_.vel, arr_.stress, arr_.mass, arr_.rho, arr_.hsml,
                        arr_.itype, arr_.intvars1, arr_.f_drucker, arr_.x00),
             "sps_upload"))
      return 1;
    // bc_or_not also carries the free-surface marks, so it is uploaded even without BCs
    if (fail(sps_upload_bcs(ctx_, arr_.bc_or_not, arr_.bc_info), "sps_upload_bcs")) return 1;
    const std::string prn = a_.out + "/output.txt";
    prn_ = std::fopen(prn.c_str(), "w");
    if (!prn_) {
      std::fprintf(stderr, "sps_run: cannot write %s\n", prn.c_str());
      return 1;
    }
    if (sph_write_mesh(prob_, a_.out.c_str())) {
      std::fprintf(stderr, "sps_run: OutputMesh into %s failed\n", a_.out.c_str());
      return 1;
    }
    total_mass_ = 0.0;
    for (int64_t i = 0; i < (int64_t)p_.nnode + p_.nstress; i++) total_mass_ += arr_.mass[i];

    const int32_t nb = sph_problem_nblocks(prob_);
    for (int32_t b = 0; b < nb; b++) {
      sph_run_block blk;
      if (sph_problem_block(prob_, b, &blk)) return 1;
      if (!(blk.dt > 0.0)) break;  // DTGT0 ends at a block with dt <= 0
      if (blk.dt != p_.dt_sph) {
        std::fprintf(stderr,
                     "sps_run: block %d has dt %.17g, the context was created with dt_sph "
                     "%.17g; a new dt needs a new step context, which restarts the pair "
                     "list's reuse order\n",
                     (int)b + 1, blk.dt, p_.dt_sph);
        return 1;
      }
      if (block(blk)) return 1;
    }
    return 0;
  }

 private:
  bool fail(int rc, const char* what) {
    if (rc == SPS_OK) return false;
    char buf[1024] = {0};
    sps_last_error(ctx_, buf, sizeof buf);
    std::fprintf(stderr, "sps_run: %s failed (%d): %s\n", what, rc, buf);
    return true;
  }

  int download() {
    return fail(sps_download(ctx_, f_.x.data(), f_.vel.data(), f_.stress.data(), f_.rho.data(),
                             f_.iv1.data(), f_.displ.data(), f_.bc.data(), f_.fdp.data()),
                "sps_download")
               ? 1
               : 0;
  }

  int output_res() {  // OutputRes
    if (download()) return 1;
    if (sph_write_output(prob_, a_.out.c_str(), itimestep_sph_, time_sph_, f_.x.data(),
                         f_.vel.data(), f_.stress.data(), f_.iv1.data(), f_.rho.data(),
                         arr_.hsml, f_.bc.data(), f_.displ.data())) {
      std::fprintf(stderr, "sps_run: OutputRes of step %d failed\n", (int)itimestep_sph_);
      return 1;
    }
    return 0;
  }

  int out_print() {  // Out_print_sph: the last node's position and velocity
    if (fail(sps_download(ctx_, f_.x.data(), f_.vel.data(), nullptr, nullptr, nullptr, nullptr,
                          nullptr, nullptr),
             "sps_download"))
      return 1;
    const size_t n = (size_t)p_.nnode - 1;
    std::fprintf(prn_, " .****  SPH ******........................................\n");
    std::fprintf(prn_, "  time step_sph is %d  time_sph = %.17g   dt_sph= %.17g  MASS =  %.17g\n",
                 (int)itimestep_sph_, time_sph_, p_.dt_sph, total_mass_);
    std::fprintf(prn_, " x velocity\n");
    std::fprintf(prn_, "  %.17g %.17g %.17g %.17g\n", f_.x[2 * n], f_.x[2 * n + 1],
                 f_.vel[2 * n], f_.vel[2 * n + 1]);
    std::fprintf(prn_, " .........................................\n");
    return std::fflush(prn_) == 0 ? 0 : 1;
  }

  int block(const sph_run_block& blk) {
    const double dt = blk.dt;
    if (output_res()) return 1;  // the results at the start of the block
    const float time_print = (float)(blk.print_step * dt);
    const float time_plot = (float)(blk.plot_step * dt);
    float t_print_reset = 0.0f, t_plot_reset = 0.0f;
    for (int32_t it = 1; it <= blk.maxtimestep; it++) {
      t_print_reset = (float)((double)t_print_reset + dt);
      t_plot_reset = (float)((double)t_plot_reset + dt);
      itimestep_sph_++;
      if (fail(sps_step(ctx_, 1, &time_sph_), "sps_step")) return 1;
      time_ = time_ + dt;
      if (time_ > blk.time_end) break;
      if (t_plot_reset >= time_plot) {
        if (output_res()) return 1;
        t_plot_reset = 0.0f;
      }
      if (t_print_reset >= time_print) {
        if (out_print()) return 1;
        t_print_reset = 0.0f;
      }
    }
    return 0;
  }

  const Args& a_;
  sph_problem* prob_;
  sps_params p_;
  const sph_problem_arrays& arr_;
  Fields f_;
  sps_ctx* ctx_ = nullptr;
  std::FILE* prn_ = nullptr;
  int32_t itimestep_sph_ = 0;
  double time_sph_ = 0.0, time_ = 0.0, total_mass_ = 0.0;
};

}  // namespace

int main(int argc, char** argv) {
  Args a;
  if (!parse(argc, argv, a)) return usage();
  sph_problem* prob = nullptr;
  char err[512] = {0};
  if (sph_problem_read(a.dir.c_str(), &prob, err, sizeof err)) {
    std::fprintf(stderr, "sps_run: %s: %s\n", a.dir.c_str(), err);
    return 1;
  }
  sps_params p = *sph_problem_params(prob);
  p.precision = a.fast ? SPS_PREC_FP32_FAST : SPS_PREC_FP64_PLAIN;
  if (a.bc_nodes_only >= 0) p.bc_nodes_only = a.bc_nodes_only;
  if (a.cspm_det_min >= 0.0) p.cspm_det_min = a.cspm_det_min;
  sph_problem_arrays arr;
  int rc = 1;
  if (sph_problem_get_arrays(prob, &arr) == 0) {
    Run run(a, prob, p, arr);
    rc = run.main();
  }
  sph_problem_free(prob);
  return rc;
}
