// ctx.cuh -- host-side context of one sps_ctx (device buffers, stream, graph).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "common.cuh"

namespace sps {

// kernels whose block size the autotuner chooses (sps_autotune)
enum TunedKernel { TK_HALF, TK_LISTS, TK_INTERP, TK_DERIVS, TK_ADAPT, TK_STAGE, TK_RKFINAL,
                   TK_XSPH, TK_N };
constexpr const char* kTunedNames[TK_N] = {"half", "lists", "interp", "derivs",
                                           "adapt_bc", "stage_begin", "rk_final", "xsph"};
// largest block each accepts (launch bounds)
constexpr int kTunedMax[TK_N] = {1024, 1024, 1024, 256, 1024, 1024, 1024, 1024};

// host copy of one realisation's problem description (the pointer fields of its params
// point into the vectors here)
struct HostReal {
  sps_params p{};
  std::vector<int32_t> nptstcurves;
  std::vector<double> ttcurves, bc_list;
  std::vector<float> ftcurves;
  // extent and smoothing lengths of the uploaded state (capacity sizing)
  double ncells_est = 0.0, hmax = 0.0, hmin_nd = 1e300;
  bool uploaded = false;
  // get_nodes_on_free_surface: every step when a later step reads its output (the
  // traction-free BC, or XSPH's marks next to BC particles, or standard SPH's position
  // copy after it); otherwise on demand when the state is downloaded, which gives the same
  // values because nothing else in the step reads them
  bool surf_every = false;
  bool surf_stale = false;
};

struct Ctx;
void drop_graphs(Ctx& c);

struct Ctx {
  sps_params p{};  // realisation 0 (the flags every realisation shares)
  std::vector<HostReal> hr;
  std::vector<Real> real;  // host copy of the per-realisation table
  Dev d{};                 // device pointers + constants, passed by value to kernels
  Dev* d_dev = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0;
  std::vector<void*> allocs;
  StepScalars* d_scal_table = nullptr;
  int scal_cap = 0;  // steps
  std::vector<StepScalars> h_scal;
  int* h_err = nullptr;  // pinned
  unsigned long long* h_chk = nullptr;  // pinned: upload checks and extents
  unsigned long long* d_chk = nullptr;
  double* stage = nullptr;  // device staging for interleaved host arrays (10 x ntotal2)
  bool uploaded = false;
  // get_nodes_on_free_surface: every step when a later step reads its output (the
  // traction-free BC, or XSPH's marks next to BC particles, or standard SPH's position
  // copy after it); otherwise on demand when the state is downloaded, which gives the same
  // values because nothing else in the step reads them
  bool surf_every = false;
  bool surf_stale = false;
  int64_t steps_done = 0;
  int precision = SPS_PREC_FP64_PLAIN;
  std::string last_error;
  // graphs of one step, one per step variant (bit 0: the outside approach's
  // re-interpolation at the start of the step, bit 1: its stress-point shift at the end,
  // bit 2: the lists written with their walk-order keys)
  cudaGraphExec_t graphs[8] = {nullptr, nullptr, nullptr, nullptr,
                               nullptr, nullptr, nullptr, nullptr};
  // keys in the step: when the state is downloaded (or snapshotted) with its free surface
  // after every step, the step writes the lists' keys (a few percent of the list build)
  // so that the detection need not rebuild the lists
  bool keys_in_step = false;   // steps write keys (the FP32 detection: the same-kind entries)
  bool keys_written = false;   // the last step wrote the keys
  bool same_written = false;   // the last step wrote the same-kind entries
  // the on-demand detection of the FP32 form runs in FP32 (launch_surface_f32) unless the
  // exact one is asked for (sps_set_surface_detection); the plain form's is always exact
  bool surface_exact = false;
  bool surface_f32() const { return precision == SPS_PREC_FP32_FAST && !surface_exact; }
  int64_t last_refresh = -1;   // steps_done at the last on-demand detection
  // FP32 form: the steps build their lists straight from the cell stencil (k_fgather) unless
  // every step runs the exact free-surface detection (its keyed lists come from the half
  // lists), the smoothing lengths evolve (sle 2: a rebuild after the step could not repeat
  // the build's band test) or the list capacity leaves no room for the gather's shared
  // memory (two lists of capC ints for each of 32 threads within 48 KB)
  bool lists_direct() const {
    return precision == SPS_PREC_FP32_FAST && !surf_every && d.sle != 2 &&
           2 * d.capC * 32 * 4 <= 49152;
  }
  // the last pair build left the half lists unwritten (k_fgather): sps_dump_pairs and the
  // keyed lists of the exact detection build them first (set by enqueue_step for every
  // step, since a replayed graph runs no host code)
  bool half_stale = false;
  int step_variant = 0;    // the variant launch_*_step enqueues
  int64_t itimestep = 0;   // itimestep_sph of the last step (0 after an upload)
  bool use_graph = true;
  // FP32 form: neighbours a pass of the interpolation (2, 4, 8) and of the node derivative
  // sums (1, 2, 4), whose entries and records are loaded before any is summed; chosen by
  // sps_autotune (results do not depend on them)
  int ahead[2] = {4, 2};
  // FP32 form: every realisation is Drucker-Prager (ncrit 12, ntype_eco > 1) in plane strain
  // without continuity density, so the stress-point tail takes its lean kernel
  bool lean_tail = false;
  // scratch for scans
  int scan_blocks = 0;
  // per-kernel event timing (sps_profile_step)
  bool profiling = false;
  std::vector<std::pair<const char*, cudaEvent_t>> prof_events;
  // training capture and learned surrogate (device buffers freed at destroy)
  float* cap_buf = nullptr;
  unsigned long long* cap_cnt = nullptr;
  uint2* mlp_frag = nullptr;
  float* mlp_bias = nullptr;
  unsigned long long* surr_cnt = nullptr;  // the 4 counters, then the gate (SurrGate)
  void* surr_rows = nullptr;                // cand_row, xcand, ycand, cand_count (one block)
  void* tc_img = nullptr;                   // tensor-core image of the network and biases
  int tc_grid = 0;                          // CTAs of the tensor-core forward pass
  double gate_min_frac = 0.5;               // sps_surrogate_gate
  int gate_max_period = 1024;
  // output snapshot (sps_snapshot): device copy of the output fields, pinned host copy,
  // the stream that moves one to the other, and the events that order them
  char* snap_dev = nullptr;
  char* snap_host = nullptr;
  size_t snap_bytes = 0;
  std::vector<int64_t> snap_roff;  // byte offset of each realisation's block
  cudaStream_t snap_stream = nullptr;
  // uploads: the host arrays are copied into the staging area on their own stream, which
  // may run while the previous step computes; the context stream waits for up_ready
  cudaStream_t up_stream = nullptr;
  cudaEvent_t up_ready = nullptr;
  cudaEvent_t snap_ready = nullptr, snap_done = nullptr;
  bool snap_pending = false;  // a snapshot was taken and not yet waited for
  bool snap_valid = false;    // snap_host holds a completed snapshot
  int64_t snap_step = 0;      // steps_done when it was taken
  int blk[TK_N] = {256, 256, 256, 256, 256, 256, 256, 256};  // block sizes (sps_autotune)
  int grid_of(int k, int n) const { return (n + blk[k] - 1) / blk[k]; }
  int64_t kernels_launched = 0;  // kernels enqueued by the launch functions
  int kernels_per_step = 0;
  // called before each kernel group: counts its kernels and, when profiling, records an
  // event that opens the group's timing interval
  void mark(const char* name, int nkernels = 1) {
    kernels_launched += nkernels;
    if (!profiling) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, stream);
    prof_events.push_back({name, e});
  }
};

// generic exclusive scans on the context stream
void scan_i32_to_i32(Ctx& c, const int32_t* in, int32_t* out, int n);
void scan_i32_to_i64(Ctx& c, const int32_t* in, int64_t* out, int n);

}  // namespace sps

#define SPS_CUDA_CHECK(expr)                                                         \
  do {                                                                               \
    cudaError_t e_ = (expr);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      throw std::runtime_error(std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    }                                                                                \
  } while (0)
