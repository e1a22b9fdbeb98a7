// sps_api.cu -- the C-ABI of include/sps.h on top of the CUDA step.
//
// sps_step(ctx, n, &time_sph) replaces n iterations of the reference driver's
//   call time_integration ; time_sph = time_sph + dt_sph      (code/1_SPH_2018.f90:82-83)
// The per-step scalars that depend only on time (gravity time-curve factor of
// gravity_force, 3_SPH_material_2018.f90:2830-2848, and the boundary-condition values of
// Normal_BCs, :1693-1724) are evaluated on the host with the reference's arithmetic and
// uploaded as a table; the device replays one captured CUDA graph per step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "ctx.cuh"
#include "mlp.cuh"
#include "sps_surrogate.h"

struct sps_ctx {
  sps::Ctx c;
};

namespace sps {
void drop_graphs(Ctx& c) {
  for (auto& g : c.graphs)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}
}  // namespace sps

namespace {

std::mutex g_err_mu;
std::string g_create_error;

constexpr int kBlock = 256;

template <typename T>
T* dalloc(sps::Ctx& c, size_t n) {
  void* p = nullptr;
  SPS_CUDA_CHECK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
  c.allocs.push_back(p);
  return static_cast<T*>(p);
}

double tcurve_value(const sps::HostReal& h, int it, double t) {
  int nc = h.p.ntcurves;
  if (it < 1 || it > nc) return 0.0;
  int npts = h.nptstcurves[it - 1];
  double tt0 = 0, tt1 = 0;
  int ip;
  for (ip = 1; ip <= npts - 1; ip++) {
    tt0 = h.ttcurves[(it - 1) + (size_t)(ip - 1) * nc];
    tt1 = h.ttcurves[(it - 1) + (size_t)ip * nc];
    if (t >= tt0 && t <= tt1) break;
    tt0 = -1000.0;
  }
  if (tt0 >= 0.0) {
    double xi = (t - tt0) / (tt1 - tt0);
    return (1.0 - xi) * (double)h.ftcurves[(it - 1) + (size_t)(ip - 1) * nc] +
           xi * (double)h.ftcurves[(it - 1) + (size_t)ip * nc];
  }
  return 0.0;
}

// time-only scalars of one realisation at time t: gravity time-curve factor and BC values
void fill_scalars(const sps::HostReal& h, double t, sps::StepScalars& s) {
  std::memset(&s, 0, sizeof(s));
  s.time_sph = t;
  if (h.p.ic_grav != 0) s.factg = tcurve_value(h, h.p.tcurve_grav, t) * h.p.ft_grav;
  for (int b = 0; b < h.p.no_bcs; b++) {
    const double* q = &h.bc_list[8 * (size_t)b];
    int itc = (int)q[2];
    double val = 0.0;
    if (itc == 0) {
      double a0 = q[4], a1 = q[3], w = q[5], phi = q[6], tt = q[7];
      double fact = 1.0 - std::exp(-t / tt);
      double argum = w * t - phi;
      val = (a0 + a1 * std::sin(argum)) * fact;
    } else if (itc > 0) {
      val = tcurve_value(h, itc, t) * q[3];
    }
    s.bcval[b] = val;
  }
}

// the per-step scalar table of nsteps steps from the times t[r] (advanced in place)
void fill_table(sps::Ctx& c, int nsteps, double* t) {
  const int R = c.d.R;
  c.h_scal.resize((size_t)nsteps * R);
  for (int k = 0; k < nsteps; k++)
    for (int r = 0; r < R; r++) {
      fill_scalars(c.hr[r], t[r], c.h_scal[(size_t)k * R + r]);
      t[r] = t[r] + c.hr[r].p.dt_sph;
    }
}

// the three id segments of realisation r: local start, count, global start
struct Seg {
  int64_t l, n, g;
};
void segments(const sps::Ctx& c, int r, Seg* s) {
  const sps::Real& M = c.real[r];
  s[0] = {0, M.nnode, M.node0};
  s[1] = {M.nnode, M.nsp, M.sp0};
  s[2] = {(int64_t)M.nnode + M.nsp, M.ndum, M.dum0};
}

__global__ void k_aos_to_soa2(const double* in, double* a, double* b, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    a[i] = in[2 * (size_t)i];
    b[i] = in[2 * (size_t)i + 1];
  }
}
__global__ void k_soa_to_aos2(double* out, const double* a, const double* b, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    out[2 * (size_t)i] = a[i];
    out[2 * (size_t)i + 1] = b[i];
  }
}

// ordered key of a double: unsigned order of the keys = numeric order of the values
__device__ __forceinline__ unsigned long long up_key(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
double up_unkey(unsigned long long k) {
  unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
}

__device__ __forceinline__ bool up_nonfinite(double v) {
  return ((unsigned long long)__double_as_longlong(v) & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
}

// the checks and extents of an upload, over the realisation's local ids l (nodes, then
// stress-points, then dummies, at global ids g0[k] + offset): out[0..5] = min x, min y,
// max x, max y, max h, min h over nodes and dummies (keys; the complement of the key for
// the maxima); out[6] = particles whose itype does not match their place (2 nodes,
// 1 stress-points, 25 dummies); out[7] = particles with a non-finite x, y or h
__global__ void k_upload_check(const int32_t* itype, const double* px, const double* py,
                               const double* hsml, int64_t g0n, int64_t nn, int64_t g0s,
                               int64_t ns, int64_t g0d, int64_t nd, unsigned long long* out) {
  unsigned long long v[6] = {~0ull, ~0ull, ~0ull, ~0ull, ~0ull, ~0ull};
  unsigned long long bad = 0, nonfin = 0;
  const int64_t n2 = nn + ns + nd;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n2;
       l += (int64_t)gridDim.x * blockDim.x) {
    int64_t g;
    int want;
    if (l < nn) {
      g = g0n + l;
      want = 2;
    } else if (l < nn + ns) {
      g = g0s + (l - nn);
      want = 1;
    } else {
      g = g0d + (l - nn - ns);
      want = 25;
    }
    bad += itype[g] != want;
    double x = px[g], y = py[g], h = hsml[g];
    if (up_nonfinite(x) || up_nonfinite(y) || up_nonfinite(h)) {
      nonfin++;
      continue;
    }
    unsigned long long k[5] = {up_key(x), up_key(y), ~up_key(x), ~up_key(y), ~up_key(h)};
    for (int q = 0; q < 5; q++) v[q] = k[q] < v[q] ? k[q] : v[q];
    if (want != 1) {
      unsigned long long kh = up_key(h);
      v[5] = kh < v[5] ? kh : v[5];
    }
  }
  __shared__ unsigned long long sh[32][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o; o >>= 1) {
    for (int q = 0; q < 6; q++) {
      unsigned long long u = __shfl_xor_sync(0xffffffffu, v[q], o);
      v[q] = u < v[q] ? u : v[q];
    }
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
    nonfin += __shfl_xor_sync(0xffffffffu, nonfin, o);
  }
  if (lane == 0) {
    for (int q = 0; q < 6; q++) sh[w][q] = v[q];
    sh[w][6] = bad;
    sh[w][7] = nonfin;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    for (int q = 0; q < 8; q++) {
      const bool sum = q >= 6;
      unsigned long long a = lane < nw ? sh[lane][q] : (sum ? 0ull : ~0ull);
      for (int o = 16; o; o >>= 1) {
        unsigned long long u = __shfl_xor_sync(0xffffffffu, a, o);
        a = sum ? a + u : (u < a ? u : a);
      }
      if (lane == 0) {
        if (sum) {
          if (a) atomicAdd(&out[q], a);
        } else {
          atomicMin(&out[q], a);
        }
      }
    }
  }
}

// Output snapshot: every realisation's fields in the layout sps_download returns them, one
// block per realisation at byte offset roff[r]: x(2,n2) vel(2,n2) stress(4,n2) rho(n2)
// intvars1(nt) f_drucker(nt) displ(2,nn) bc_or_not(nt) (dummy stress written as 0)
struct SnapBlock {
  size_t x, vel, stress, rho, iv1, fdp, displ, bc, bytes;
};
__host__ __device__ inline SnapBlock snap_block(int64_t nn, int64_t nt, int64_t n2) {
  SnapBlock b;
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  b.x = 0;
  b.vel = b.x + up(16 * n2);
  b.stress = b.vel + up(16 * n2);
  b.rho = b.stress + up(32 * n2);
  b.iv1 = b.rho + up(8 * n2);
  b.fdp = b.iv1 + up(8 * nt);
  b.displ = b.fdp + up(8 * nt);
  b.bc = b.displ + up(16 * nn);
  b.bytes = b.bc + up(4 * nt);
  return b;
}
__global__ void k_snap_pack(sps::Dev D, char* out, const int64_t* roff) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= D.N2) return;
  const int r = D.R == 1 ? 0 : D.rid[g];
  const sps::Real& M = sps::real_of(D, g);
  const int64_t nn = M.nnode, nt = nn + M.nsp, n2 = nt + M.ndum;
  int64_t l;
  if (g < D.NN) l = g - M.node0;
  else if (g < D.NT) l = nn + (g - M.sp0);
  else l = nt + (g - M.dum0);
  const SnapBlock b = snap_block(nn, nt, n2);
  char* base = out + roff[r];
  double2* x = reinterpret_cast<double2*>(base + b.x);
  double2* v = reinterpret_cast<double2*>(base + b.vel);
  double2* s = reinterpret_cast<double2*>(base + b.stress);  // 4 doubles per particle
  x[l] = make_double2(D.px[g], D.py[g]);
  v[l] = make_double2(D.vx[g], D.vy[g]);
  reinterpret_cast<double*>(base + b.rho)[l] = D.rho[g];
  if (g < D.NT) {
    s[2 * l] = make_double2(D.s0[g], D.s1[g]);
    s[2 * l + 1] = make_double2(D.s2[g], D.s3[g]);
    reinterpret_cast<double*>(base + b.iv1)[l] = D.iv1[g];
    reinterpret_cast<double*>(base + b.fdp)[l] = D.fdp[g];
    reinterpret_cast<int32_t*>(base + b.bc)[l] = D.bc_or_not[g];
    if (g < D.NN)
      reinterpret_cast<double2*>(base + b.displ)[l] = make_double2(D.dispx[g], D.dispy[g]);
  } else {
    s[2 * l] = make_double2(0.0, 0.0);
    s[2 * l + 1] = make_double2(0.0, 0.0);
  }
}
__global__ void k_aos_to_soa4(const double* in, double* a, double* b, double* c, double* d, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    a[i] = in[4 * (size_t)i];
    b[i] = in[4 * (size_t)i + 1];
    c[i] = in[4 * (size_t)i + 2];
    d[i] = in[4 * (size_t)i + 3];
  }
}
__global__ void k_soa_to_aos4(double* out, const double* a, const double* b, const double* c,
                              const double* d, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    out[4 * (size_t)i] = a[i];
    out[4 * (size_t)i + 1] = b[i];
    out[4 * (size_t)i + 2] = c[i];
    out[4 * (size_t)i + 3] = d[i];
  }
}
__global__ void k_check_finite(sps::Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  double v = D.px[i] + D.py[i] + D.vx[i] + D.vy[i] + D.s0[i] + D.s1[i] + D.s2[i] + D.s3[i];
  if (!isfinite(v)) atomicOr(D.err, 1 << 20);
}

int fail(sps::Ctx* c, int rc, const std::string& msg) {
  if (c) c->last_error = msg;
  else {
    std::lock_guard<std::mutex> g(g_err_mu);
    g_create_error = msg;
  }
  return rc;
}

void build_graph(sps::Ctx& c);

// the step variant of itimestep_sph `it` (time_integration, 2_SPH_main_2018.f90:99-108 and
// shift_stress_points :258): bit 0 re-interpolates at the start (SPH_shift, it > 1,
// mod(it - 1, shift_update) == 0), bit 1 repositions the stress-points at the end
// (mod(it, shift_update) == 0, with update_x)
int variant_of(const sps::Ctx& c, int64_t it) {
  const sps::Dev& D = c.d;
  if (!D.outside) return 0;
  int v = 0;
  if (c.p.sph_shift && it > 1 && (it - 1) % c.p.shift_update == 0) v |= 1;
  if (D.update_x && it % c.p.shift_update == 0) v |= 2;
  return v;
}

// enqueue one step (itimestep_sph advanced first) as its variant's graph, or directly
void enqueue_step(sps::Ctx& c) {
  c.itimestep += 1;
  c.step_variant = variant_of(c, c.itimestep) | (c.keys_in_step ? 4 : 0);
  c.keys_written = (c.keys_in_step && !c.surface_f32() && !c.lists_direct()) || c.surf_every;
  c.same_written = c.keys_in_step || c.surf_every || c.d.same_entries;
  // set here, on the host, for every step: a replayed graph runs no host code
  c.half_stale = c.lists_direct();
  if (c.use_graph && !c.profiling) {
    if (!c.graphs[c.step_variant]) build_graph(c);
    SPS_CUDA_CHECK(cudaGraphLaunch(c.graphs[c.step_variant], c.stream));
  } else if (c.precision == SPS_PREC_FP64_PLAIN) {
    sps::launch_plain_step(c);
  } else {
    sps::launch_fast_step(c);
  }
}

void build_graph(sps::Ctx& c) {
  cudaGraph_t g;
  SPS_CUDA_CHECK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
  int64_t k0 = c.kernels_launched;
  if (c.precision == SPS_PREC_FP64_PLAIN) sps::launch_plain_step(c);
  else sps::launch_fast_step(c);
  c.kernels_per_step = (int)(c.kernels_launched - k0);
  SPS_CUDA_CHECK(cudaStreamEndCapture(c.stream, &g));
  SPS_CUDA_CHECK(cudaGraphInstantiate(&c.graphs[c.step_variant], g, 0));
  cudaGraphDestroy(g);
}

void ensure_scal(sps::Ctx& c, int n) {
  if (n <= c.scal_cap) return;
  int cap = std::max(n, 256);
  void* p = nullptr;
  SPS_CUDA_CHECK(cudaMalloc(&p, sizeof(sps::StepScalars) * (size_t)cap * c.d.R));
  c.allocs.push_back(p);
  c.d_scal_table = static_cast<sps::StepScalars*>(p);
  c.scal_cap = cap;
  c.d.scal_table = c.d_scal_table;
  drop_graphs(c);
}

std::string err_text(int e) {
  std::string m;
  if (e & sps::ERR_HALF_CAP) m += "half-stencil pair capacity exceeded; ";
  if (e & sps::ERR_LIST_CAP) m += "neighbour list capacity exceeded (raise max_neighbours); ";
  if (e & sps::ERR_CELLS) m += "cell grid capacity exceeded; ";
  if (e & sps::ERR_NPAIRS) m += "more than 2^30 pairs; ";
  if (e & sps::ERR_BOUND) m += "more than 8 wall particles within 0.75 dx of a node; ";
  if (e & (1 << 20)) m += "non-finite value in the particle state; ";
  if (e & sps::kErrTensorCore) m += "the surrogate's tensor-core inference timed out; ";
  return m;
}

}  // namespace

extern "C" {

namespace {

// the per-material constants of the viscoplastic laws (invar09, yieldf09, Get_Dmatx in
// 3_SPH_material_2018.f90), with the expressions the reference evaluates per call
void viscoplastic_constants(const sps_params& q, sps::Real& M) {
  const double root3 = (double)std::sqrt(3.0f);
  const double young = q.props[2], poiss = q.props[3];
  M.vp_fdatm0 = q.props[6];
  M.vp_hards = q.props[7];
  M.vp_gamma = q.props[9];
  M.vp_delta = q.props[10];
  M.vp_nflow = q.props[11];
  M.vp_snphi = std::sin(q.props[8] * (double)0.017453292f);
  M.vp_den = root3 * (3.0 - M.vp_snphi);
  M.vp_cons1 = M.ncrit == 3 ? M.vp_snphi / 3.0 : (2.0 * M.vp_snphi) / M.vp_den;
  double* D = M.vp_D;
  for (int k = 0; k < 16; k++) D[k] = 0.0;
  if (q.ntype_solid == 1) {  // plane stress
    const double c = young / (1.0 - poiss * poiss);
    D[0] = c;
    D[5] = c;
    D[1] = c * poiss;
    D[4] = c * poiss;
    D[10] = ((1.0 - poiss) * c) / 2.0;
  } else {  // plane strain (2), axisymmetric (3)
    const double c = (young * (1.0 - poiss)) / ((1.0 + poiss) * (1.0 - 2.0 * poiss));
    const double cp = (c * poiss) / (1.0 - poiss);
    D[0] = c;
    D[5] = c;
    D[1] = cp;
    D[4] = cp;
    D[3] = cp;
    D[7] = cp;
    D[12] = cp;
    D[13] = cp;
    D[15] = c;
    D[10] = q.ntype_solid == 2 ? ((1.0 - 2.0 * poiss) * c) / (2.0 * (1.0 - poiss))
                               : (c * (1.0 - 2.0 * poiss)) / (2.0 * (1.0 - poiss));
  }
}

// the checks sps_create makes on one problem
int check_params(const sps_params* p) {
  if (p->ndimn != 2 || p->nstre != 4)
    return fail(nullptr, SPS_ERR_UNSUPPORTED, "only ndimn = 2, nstre = 4 are implemented");
  if (p->nnode <= 0 || p->nstress < 0 || p->ndummy < 0 || p->ndummy2 < 0 || p->ndummy2 > p->ndummy)
    return fail(nullptr, SPS_ERR_ARG, "inconsistent particle counts");
  int ntype_eco = (int)p->props[0], ncrit = (int)p->props[1];
  if (ntype_eco > 1 && ncrit == 5)
    return fail(nullptr, SPS_ERR_UNSUPPORTED,
                "Modified Cam Clay (ncrit = 5): the reference never integrates its yield-surface "
                "size Internal_Vars(3), which stays 0 and divides yieldf09's flow vector");
  if (ntype_eco > 1 && !((ncrit >= 1 && ncrit <= 4) || ncrit == 12))
    return fail(nullptr, SPS_ERR_UNSUPPORTED,
                "material law: ncrit must be 1-4 (viscoplastic) or 12 (Drucker-Prager)");
  if (ntype_eco > 1 && ncrit <= 4 && !(p->props[6] > (double)0.001f))
    return fail(nullptr, SPS_ERR_ARG,
                "viscoplastic law: initial yield stress must exceed 0.001 (invar09 stops)");
  if (ntype_eco > 1 && ncrit <= 4 && (p->ntype_solid < 1 || p->ntype_solid > 3))
    return fail(nullptr, SPS_ERR_UNSUPPORTED, "viscoplastic law: ntype_solid must be 1, 2 or 3");
  if (p->skf < 1 || p->skf > 3) return fail(nullptr, SPS_ERR_ARG, "skf must be 1, 2 or 3");
  if (p->no_bcs > sps::kMaxBC) return fail(nullptr, SPS_ERR_UNSUPPORTED, "more than 16 BCs");
  if (p->no_bcs > 0 && !p->bc_list) return fail(nullptr, SPS_ERR_ARG, "bc_list missing");
  if (!p->sp_sph && p->nstress != p->nnode)
    return fail(nullptr, SPS_ERR_ARG, "standard SPH needs nstress == nnode");
  if (p->sp_sph && !p->inside_approach &&
      (p->npoints < 1 || p->npoints > 4 || p->shift_update < 1 ||
       p->nstress != p->npoints * p->nnode || (p->vel_vector && p->npoints != 2)))
    return fail(nullptr, SPS_ERR_ARG,
                "outside approach: npoints 1-4 per node (2 with vel_vector), nstress = "
                "npoints * nnode, shift_update >= 1");
  if (!p->sp_sph && p->inside_approach)
    return fail(nullptr, SPS_ERR_ARG, "standard SPH has no inside approach");
  if (p->precision != SPS_PREC_FP64_PLAIN && p->precision != SPS_PREC_FP32_FAST)
    return fail(nullptr, SPS_ERR_ARG, "unknown precision");
  for (int b = 0; b < p->no_bcs; b++)
    if ((int)p->bc_list[8 * (size_t)b + 2] < 0)
      return fail(nullptr, SPS_ERR_UNSUPPORTED, "negative time-curve index in bc_list");
  if (p->ic_grav != 0 && (p->tcurve_grav < 1 || p->tcurve_grav > p->ntcurves))
    return fail(nullptr, SPS_ERR_ARG, "gravity time curve out of range");
  if (!(p->cspm_det_min >= 0.0 && p->cspm_det_min < 1e300))
    return fail(nullptr, SPS_ERR_ARG, "cspm_det_min must be finite and >= 0");
  if (p->bc_nodes_only != 0 && p->bc_nodes_only != 1)
    return fail(nullptr, SPS_ERR_ARG, "bc_nodes_only must be 0 or 1");
  return SPS_OK;
}

// the solver flags a batch must share
bool same_flags(const sps_params& a, const sps_params& b) {
  return a.sp_sph == b.sp_sph && a.inside_approach == b.inside_approach && a.cspm == b.cspm &&
         a.xsph == b.xsph && a.update_x == b.update_x && a.cont_density == b.cont_density &&
         a.sle == b.sle && a.skf == b.skf && a.precision == b.precision && a.pi == b.pi &&
         a.ntype_solid == b.ntype_solid && a.art_stress == b.art_stress &&
         a.cspm_det_min == b.cspm_det_min && a.bc_nodes_only == b.bc_nodes_only &&
         (a.inside_approach || !a.sp_sph ||
          (a.npoints == b.npoints && a.sph_shift == b.sph_shift &&
           a.vel_vector == b.vel_vector && a.shift_update == b.shift_update));
}

}  // namespace

int sps_create(const sps_params* p, sps_ctx** out) { return sps_create_batch(1, p, out); }

int sps_create_batch(int32_t nreal, const sps_params* ps, sps_ctx** out) {
  if (!ps || !out || nreal < 1) return fail(nullptr, SPS_ERR_ARG, "null argument or no realisation");
  *out = nullptr;
  if (nreal > 65535) return fail(nullptr, SPS_ERR_ARG, "at most 65535 realisations");
  int64_t NN = 0, NS = 0, ND = 0;
  for (int r = 0; r < nreal; r++) {
    int rc = check_params(&ps[r]);
    if (rc != SPS_OK) return rc;
    if (!same_flags(ps[0], ps[r]))
      return fail(nullptr, SPS_ERR_ARG, "the realisations of a batch must share the solver flags");
    if (nreal > 1 && ps[r].no_bcs > 0)
      return fail(nullptr, SPS_ERR_UNSUPPORTED, "boundary conditions in a batch of several realisations");
    NN += ps[r].nnode;
    NS += ps[r].nstress;
    ND += ps[r].ndummy;
  }
  if (NN + NS + ND >= (1LL << 28))  // half-list entries keep particle ids in 28 bits
    return fail(nullptr, SPS_ERR_ARG, "too many particles (at most 2^28 - 1 per context)");
  const sps_params* p = &ps[0];
  sps_ctx* h = nullptr;
  try {
    h = new sps_ctx();
    sps::Ctx& c = h->c;
    c.p = *p;
    c.precision = p->precision;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) throw std::runtime_error("no CUDA device");
    c.device = dev;
    SPS_CUDA_CHECK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    SPS_CUDA_CHECK(cudaStreamCreateWithFlags(&c.up_stream, cudaStreamNonBlocking));
    SPS_CUDA_CHECK(cudaEventCreateWithFlags(&c.up_ready, cudaEventDisableTiming));
    sps::Dev& D = c.d;
    D.R = nreal;
    D.NN = (int)NN;
    D.NT = (int)(NN + NS);
    D.N2 = (int)(NN + NS + ND);
    c.hr.resize(nreal);
    c.real.resize(nreal);
    int64_t on = 0, os = NN, od = NN + NS;
    for (int r = 0; r < nreal; r++) {
      const sps_params& q = ps[r];
      sps::HostReal& hr = c.hr[r];
      hr.p = q;
      if (q.ntcurves > 0) {
        size_t nt = (size_t)q.ntcurves * q.mptstcurves;
        hr.nptstcurves.assign(q.nptstcurves, q.nptstcurves + q.ntcurves);
        hr.ttcurves.assign(q.ttcurves, q.ttcurves + nt);
        hr.ftcurves.assign(q.ftcurves, q.ftcurves + nt);
      }
      if (q.no_bcs > 0) hr.bc_list.assign(q.bc_list, q.bc_list + 8 * (size_t)q.no_bcs);
      hr.p.nptstcurves = hr.nptstcurves.data();
      hr.p.ttcurves = hr.ttcurves.data();
      hr.p.ftcurves = hr.ftcurves.data();
      hr.p.bc_list = hr.bc_list.data();
      hr.p.wall_position = nullptr;
      hr.p.horizontal_or_not = nullptr;
      sps::Real& M = c.real[r];
      M.node0 = (int)on;
      M.nnode = q.nnode;
      M.sp0 = (int)os;
      M.nsp = q.nstress;
      M.dum0 = (int)od;
      M.ndum = q.ndummy;
      M.ndum2 = q.ndummy2;
      on += q.nnode;
      os += q.nstress;
      od += q.ndummy;
      M.ntype_eco = (int)q.props[0];
      M.ncrit = (int)q.props[1];
      M.ntype_solid = q.ntype_solid;
      M.ic_grav = q.ic_grav;
      M.dt = q.dt_sph;
      M.dt6 = q.dt_sph / 6.0;
      M.dx = q.dx;
      M.alpha = q.alpha;
      M.beta = q.beta;
      M.damping = q.damping;
      M.D11 = q.D11;
      M.D12 = q.D12;
      M.D22 = q.D22;
      M.D33 = q.D33;
      M.D41 = q.D41;
      M.D42 = q.D42;
      M.D11f = (float)q.D11;
      M.D12f = (float)q.D12;
      M.D22f = (float)q.D22;
      M.D33f = (float)q.D33;
      M.D41f = (float)q.D41;
      M.D42f = (float)q.D42;
      M.tanfi = q.props[12];
      M.coh = q.props[13];
      M.young = q.props[2];
      M.poiss = q.props[3];
      double den = std::sqrt(9.0 + 12.0 * (M.tanfi * M.tanfi));
      M.alpha2 = M.tanfi / den;
      M.kc = (3.0 * M.coh) / den;
      M.kc_shift = M.alpha2 > 0.0 ? M.kc / (3.0 * M.alpha2) : 0.0;
      M.alpha2f = (float)M.alpha2;
      M.kcf = (float)M.kc;
      {  // drucker_prager's FP32 constants (host FP32, no contraction: -ffp-contract=off)
        const float tf = (float)M.tanfi, cf = (float)M.coh, yf = (float)M.young,
                    pf = (float)M.poiss;
        const float denf = std::sqrt(9.0f + 12.0f * (tf * tf));
        M.dpf_alpha2 = tf / denf;
        M.dpf_kc = (3.0f * cf) / denf;
        M.dpf_G = yf / (2.0f * (1.0f + pf));
        M.dpf_K = yf / (3.0f * (1.0f - 2.0f * pf));
      }
      for (int d = 0; d < 2; d++) {
        M.xmin_dom[d] = q.xmin_domain[d];
        M.xmax_dom[d] = q.xmax_domain[d];
        M.cgrav[d] = q.cgrav[d];
      }
      viscoplastic_constants(q, M);
      M.r_x = q.r_x;
      M.r_y = q.r_y;
      M.disp_tol = q.disp_tol;
    }
    D.capC = D.capS = D.capH = 0;  // sized at upload from the kernel support
    D.skf = p->skf;
    D.scale_k = p->skf == 1 ? 2 : 3;
    D.cspm = p->cspm;
    D.xsph = p->xsph;
    D.update_x = p->update_x;
    D.cont_density = p->cont_density;
    D.sle = p->sle;
    D.sp_sph = p->sp_sph;
    D.inside = p->inside_approach;
    D.no_bcs = p->no_bcs;
    D.ifsigman = p->ifsigman;
    D.cspm_det = p->cspm_det_min;
    D.bc_nodes_only = p->bc_nodes_only;
    // (the outside approach shifts the stress-points right after the detection, so the
    // detection cannot wait for the download)
    c.surf_every = p->update_x && (p->ifsigman == 1 || (p->xsph && p->no_bcs > 0) ||
                                   !p->sp_sph || !p->inside_approach);
    D.pi = p->pi;
    for (int b = 0; b < p->no_bcs; b++) D.bcvar[b] = (int)p->bc_list[8 * (size_t)b + 1];
    const size_t N2 = D.N2, NT = D.NT, NN_ = D.NN;
    {
      sps::Real* rd = dalloc<sps::Real>(c, nreal);
      SPS_CUDA_CHECK(cudaMemcpyAsync(rd, c.real.data(), sizeof(sps::Real) * nreal,
                                     cudaMemcpyHostToDevice, c.stream));
      D.real = rd;
      D.real0 = c.real[0];
      c.lean_tail = p->precision == SPS_PREC_FP32_FAST && !p->cont_density;
      for (const sps::Real& M : c.real)
        c.lean_tail = c.lean_tail && M.ntype_eco > 1 && M.ncrit == 12 && M.ntype_solid != 1;
      std::vector<uint16_t> rid(N2);
      for (int r = 0; r < nreal; r++) {
        const sps::Real& M = c.real[r];
        std::fill(rid.begin() + M.node0, rid.begin() + M.node0 + M.nnode, (uint16_t)r);
        std::fill(rid.begin() + M.sp0, rid.begin() + M.sp0 + M.nsp, (uint16_t)r);
        std::fill(rid.begin() + M.dum0, rid.begin() + M.dum0 + M.ndum, (uint16_t)r);
      }
      uint16_t* ridd = dalloc<uint16_t>(c, N2);
      SPS_CUDA_CHECK(cudaMemcpyAsync(ridd, rid.data(), sizeof(uint16_t) * N2, cudaMemcpyHostToDevice,
                                     c.stream));
      SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
      D.rid = ridd;
    }
    D.px = dalloc<double>(c, N2);
    D.py = dalloc<double>(c, N2);
    D.vx = dalloc<double>(c, N2);
    D.vy = dalloc<double>(c, N2);
    D.s0 = dalloc<double>(c, N2);
    D.s1 = dalloc<double>(c, N2);
    D.s2 = dalloc<double>(c, N2);
    D.s3 = dalloc<double>(c, N2);
    D.mass = dalloc<double>(c, N2);
    D.rho = dalloc<double>(c, N2);
    D.hsml = dalloc<double>(c, N2);
    D.iv1 = dalloc<double>(c, NT);
    D.fdp = dalloc<double>(c, NT);
    D.x00x = dalloc<double>(c, N2);
    D.x00y = dalloc<double>(c, N2);
    D.dispx = dalloc<double>(c, NN_);
    D.dispy = dalloc<double>(c, NN_);
    D.itype = dalloc<int32_t>(c, N2);
    D.out = dalloc<uint8_t>(c, N2);
    D.bc_or_not = dalloc<int32_t>(c, NT);
    D.bc_info = dalloc<int32_t>(c, 8 * NT);
    D.bc_int = dalloc<int32_t>(c, NN_);
    D.wallpos = dalloc<float>(c, N2);
    D.horiz = dalloc<float>(c, N2);
    D.grad_u = dalloc<double>(c, 4 * NT);
    D.nrmx = dalloc<double>(c, NT);
    D.nrmy = dalloc<double>(c, NT);
    D.subset = dalloc<int8_t>(c, NT);
    D.fint = dalloc<float>(c, NT);
    D.vol32 = p->precision == SPS_PREC_FP32_FAST ? dalloc<float>(c, NT) : nullptr;
    D.x0x = dalloc<double>(c, N2);  // every particle: the positions of the step's pair build
    D.x0y = dalloc<double>(c, N2);
    D.vx0 = dalloc<double>(c, NT);
    D.vy0 = dalloc<double>(c, NT);
    for (int k = 0; k < 4; k++) {
      D.st0[k] = dalloc<double>(c, NT);
      D.RKs[k] = dalloc<double>(c, NT);
      D.RHS1[k] = dalloc<double>(c, NT);
    }
    for (int k = 0; k < 2; k++) {
      D.RKv[k] = dalloc<double>(c, NT);
      D.RHS2[k] = dalloc<double>(c, NT);
    }
    D.rho0 = dalloc<double>(c, NT);
    D.hsml0 = dalloc<double>(c, NT);
    D.RKr = dalloc<double>(c, NT);
    D.RKh = dalloc<double>(c, NT);
    D.RKd = dalloc<double>(c, NT);
    D.RHSr = dalloc<double>(c, NT);
    D.RHSh = dalloc<double>(c, NT);
    D.fbx = dalloc<double>(c, NN_);
    D.art_stress = p->art_stress ? 1 : 0;
    // the same-kind lists (node-node, stress-point-stress-point) are read within a step only
    // by XSPH, artificial viscosity and artificial stress; the free-surface detection
    // builds its own lists with walk-order keys, which always carry them
    D.same_entries = (p->xsph || D.art_stress) ? 1 : 0;
    for (int r = 0; r < nreal; r++)
      if (ps[r].alpha > 0 || ps[r].beta > 0) D.same_entries = 1;
    D.outside = p->sp_sph && !p->inside_approach;
    D.npoints = D.outside ? p->npoints : 1;
    D.vel_vector = D.outside && p->vel_vector;
    if (D.vel_vector) {
      D.x10x = dalloc<double>(c, NN_);
      D.x10y = dalloc<double>(c, NN_);
      D.disp10 = dalloc<double>(c, NN_);
      SPS_CUDA_CHECK(cudaMemsetAsync(D.disp10, 0, sizeof(double) * NN_, c.stream));
    }
    D.artR = D.art_stress ? dalloc<double>(c, 3 * (size_t)NN_) : nullptr;
    D.fby = dalloc<double>(c, NN_);
    D.Ddev = dalloc<double>(c, NT);
    D.vol = dalloc<double>(c, N2);
    D.rinv = dalloc<double>(c, N2);
    for (int k = 0; k < 3; k++) D.A[k] = dalloc<double>(c, NT);
    D.fast = (p->precision == SPS_PREC_FP32_FAST) ? 1 : 0;
    D.l2_prefetch = 0;  // off until the autotuner finds it faster
    // stress-point and node targets in sorted order (both forms)
    D.tgtS = dalloc<int32_t>(c, NT - NN_ + 1);
    D.tgtN = dalloc<int32_t>(c, NN_ + 1);
    D.tflag = dalloc<int32_t>(c, 2 * N2);
    D.toff = dalloc<int32_t>(c, 2 * N2 + 2);
    D.lcol = dalloc<int32_t>(c, N2);
    if (D.fast) {
      D.recV = dalloc<float4>(c, N2);
      D.recS = dalloc<float4>(c, NT);
      D.recI = dalloc<float4>(c, N2);
      D.recA = dalloc<float4>(c, NT);
      D.recAl = dalloc<float4>(c, NT);
    }
    D.cell_of = dalloc<int32_t>(c, N2);
    D.sorted = dalloc<int32_t>(c, N2);
    D.spos = dalloc<int32_t>(c, N2);
    D.xr = dalloc<float>(c, N2);
    D.yr = dalloc<float>(c, N2);
    D.hr = dalloc<float>(c, N2);
    D.xrl = dalloc<float>(c, N2);
    D.srec = dalloc<float4>(c, N2);
    D.srecl = dalloc<float2>(c, N2);
    D.yrl = dalloc<float>(c, N2);
    D.grid = dalloc<sps::Grid>(c, nreal);
    D.gtot = dalloc<sps::GridTotal>(c, 1);
    D.bbox = dalloc<unsigned long long>(c, 6 * (size_t)nreal);
    D.half_cnt = dalloc<int32_t>(c, N2);
    D.half_meta = dalloc<int4>(c, N2);
    D.half_off = dalloc<int64_t>(c, N2 + 1);
    D.degC = dalloc<int32_t>(c, N2);
    D.degS = dalloc<int32_t>(c, N2);
    D.meta = dalloc<sps::PairMeta>(c, nreal);
    D.step_idx = dalloc<int>(c, 1);
    D.cur = dalloc<sps::StepScalars>(c, nreal);
    D.err = dalloc<int>(c, 1);
    D.scan_tmp = dalloc<int64_t>(c, (N2 + 4096) / 4096 + 64);
    // upload staging: x, vel, x00 (2 each), stress (4), mass, rho, hsml, intvars1,
    // f_drucker (1 each) as doubles, itype as int32
    c.stage = dalloc<double>(c, 16 * (size_t)N2);
    c.d_chk = dalloc<unsigned long long>(c, 8);
    SPS_CUDA_CHECK(cudaMemsetAsync(D.meta, 0, sizeof(sps::PairMeta) * nreal, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.bbox, 0xff, sizeof(unsigned long long) * 6 * nreal, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.gtot, 0, sizeof(sps::GridTotal), c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.err, 0, sizeof(int), c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.grad_u, 0, sizeof(double) * 4 * NT, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.nrmx, 0, sizeof(double) * NT, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.nrmy, 0, sizeof(double) * NT, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.subset, 0, NT, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.fint, 0, sizeof(float) * NT, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.bc_or_not, 0, sizeof(int32_t) * NT, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.bc_info, 0, sizeof(int32_t) * 8 * NT, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.bc_int, 0, sizeof(int32_t) * NN_, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.fbx, 0, sizeof(double) * NN_, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.fby, 0, sizeof(double) * NN_, c.stream));
    {
      // dummy wall tables: realisation r's entries ntotal_r.. go to its dummy ids
      std::vector<float> wp(N2, 0.0f), ho(N2, 0.0f);
      for (int r = 0; r < nreal; r++) {
        const sps_params& q = ps[r];
        const sps::Real& M = c.real[r];
        size_t nt_r = (size_t)q.nnode + q.nstress;
        if (q.wall_position)
          std::copy(q.wall_position + nt_r, q.wall_position + nt_r + q.ndummy, wp.begin() + M.dum0);
        if (q.horizontal_or_not)
          std::copy(q.horizontal_or_not + nt_r, q.horizontal_or_not + nt_r + q.ndummy,
                    ho.begin() + M.dum0);
      }
      SPS_CUDA_CHECK(cudaMemcpyAsync(D.wallpos, wp.data(), sizeof(float) * N2, cudaMemcpyHostToDevice, c.stream));
      SPS_CUDA_CHECK(cudaMemcpyAsync(D.horiz, ho.data(), sizeof(float) * N2, cudaMemcpyHostToDevice, c.stream));
      SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    }
    SPS_CUDA_CHECK(cudaMallocHost(&c.h_err, sizeof(int)));
    SPS_CUDA_CHECK(cudaMallocHost(&c.h_chk, 8 * sizeof(unsigned long long)));
    ensure_scal(c, 256);
    D.cell_cap = 0;  // sized at upload
    c.d_dev = nullptr;
  } catch (const std::bad_alloc&) {
    sps_destroy(h);
    return fail(nullptr, SPS_ERR_CUDA, "host allocation failed");
  } catch (const std::exception& e) {
    sps_destroy(h);
    return fail(nullptr, SPS_ERR_CUDA, e.what());
  }
  *out = h;
  return SPS_OK;
}

namespace {
// the free-surface detection of the last step, when it was left for the download
void refresh_surface(sps::Ctx& c, bool sync = true) {
  if (!c.surf_stale) return;
  // detections one or two steps apart: let the following steps write the keys
  c.keys_in_step = c.last_refresh >= 0 && c.steps_done - c.last_refresh <= 2;
  c.last_refresh = c.steps_done;
  if (c.surface_f32()) {
    // the FP32 detection walks the same-kind lists: the steps wrote them (with or without
    // keys) or the lists are built again with them
    if (!c.same_written) sps::launch_lists_same(c);
    sps::launch_surface_f32(c);
  } else {
    if (!c.keys_written) sps::launch_lists_keys(c);
    sps::launch_surface(c);
  }
  SPS_CUDA_CHECK(cudaGetLastError());
  if (sync) SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
  c.surf_stale = false;
}
}  // namespace

int sps_upload(sps_ctx* h, const double* x, const double* vel, const double* stress,
               const double* mass, const double* rho, const double* hsml, const int32_t* itype,
               const double* intvars1, const double* f_drucker, const double* x00) {
  if (!h) return SPS_ERR_ARG;
  if (h->c.d.R != 1)
    return fail(&h->c, SPS_ERR_ARG, "sps_upload: a batch takes sps_upload_real per realisation");
  return sps_upload_real(h, 0, x, vel, stress, mass, rho, hsml, itype, intvars1, f_drucker, x00);
}

int sps_upload_real(sps_ctx* h, int32_t r, const double* x, const double* vel,
                    const double* stress, const double* mass, const double* rho,
                    const double* hsml, const int32_t* itype, const double* intvars1,
                    const double* f_drucker, const double* x00) {
  if (!h) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  sps::Dev& D = c.d;
  if (r < 0 || r >= D.R) return fail(&c, SPS_ERR_ARG, "sps_upload_real: no such realisation");
  if (!x || !vel || !stress || !mass || !rho || !hsml || !itype)
    return fail(&c, SPS_ERR_ARG, "sps_upload: null array");
  const sps::Real& M = c.real[r];
  const size_t nn = M.nnode, nt = (size_t)M.nnode + M.nsp, n2 = nt + M.ndum;
  Seg sg[3];
  segments(c, r, sg);
  try {
    // every host array is copied into the staging area on the upload stream, which may
    // run while the previous step still computes (the state it reads is untouched); the
    // context stream waits for the copies, transposes the interleaved arrays and moves
    // the others into the state, reduces the checks and extents, and synchronises once
    double* st_x = c.stage;
    double* st_v = st_x + 2 * n2;
    double* st_0 = st_v + 2 * n2;
    double* st_s = st_0 + 2 * n2;
    double* st_m = st_s + 4 * n2;
    double* st_r = st_m + n2;
    double* st_h = st_r + n2;
    double* st_i = st_h + n2;
    double* st_f = st_i + n2;
    int32_t* st_t = reinterpret_cast<int32_t*>(st_f + n2);
    auto nbk = [](int64_t n) { return (int)((n + kBlock - 1) / kBlock); };
    auto h2d = [&](void* dst, const void* src, size_t bytes) {
      if (bytes) SPS_CUDA_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c.up_stream));
    };
    h2d(st_x, x, sizeof(double) * 2 * n2);
    h2d(st_v, vel, sizeof(double) * 2 * n2);
    h2d(st_0, x00 ? x00 : x, sizeof(double) * 2 * n2);
    h2d(st_s, stress, sizeof(double) * 4 * n2);
    h2d(st_m, mass, sizeof(double) * n2);
    h2d(st_r, rho, sizeof(double) * n2);
    h2d(st_h, hsml, sizeof(double) * n2);
    h2d(st_t, itype, sizeof(int32_t) * n2);
    if (intvars1) h2d(st_i, intvars1, sizeof(double) * nt);
    if (f_drucker) h2d(st_f, f_drucker, sizeof(double) * nt);
    SPS_CUDA_CHECK(cudaEventRecord(c.up_ready, c.up_stream));
    SPS_CUDA_CHECK(cudaStreamWaitEvent(c.stream, c.up_ready, 0));
    auto soa2 = [&](double* st, double* a, double* b) {
      for (const Seg& q : sg)
        if (q.n > 0)
          k_aos_to_soa2<<<nbk(q.n), kBlock, 0, c.stream>>>(st + 2 * q.l, a + q.g, b + q.g, (int)q.n);
    };
    auto d2d = [&](void* dst, const void* src, size_t esz, int nseg) {
      for (int k = 0; k < nseg; k++)
        if (sg[k].n > 0)
          SPS_CUDA_CHECK(cudaMemcpyAsync((char*)dst + esz * sg[k].g, (const char*)src + esz * sg[k].l,
                                         esz * sg[k].n, cudaMemcpyDeviceToDevice, c.stream));
    };
    soa2(st_x, D.px, D.py);
    soa2(st_v, D.vx, D.vy);
    if (D.vel_vector && nn > 0) {  // Setup_Global_Arrays (3_SPH_material_2018.f90:1032)
      SPS_CUDA_CHECK(cudaMemcpyAsync(D.x10x + M.node0, D.px + M.node0, sizeof(double) * nn,
                                     cudaMemcpyDeviceToDevice, c.stream));
      SPS_CUDA_CHECK(cudaMemcpyAsync(D.x10y + M.node0, D.py + M.node0, sizeof(double) * nn,
                                     cudaMemcpyDeviceToDevice, c.stream));
      SPS_CUDA_CHECK(cudaMemsetAsync(D.disp10 + M.node0, 0, sizeof(double) * nn, c.stream));
    }
    soa2(st_0, D.x00x, D.x00y);
    for (const Seg& q : sg)
      if (q.n > 0)
        k_aos_to_soa4<<<nbk(q.n), kBlock, 0, c.stream>>>(st_s + 4 * q.l, D.s0 + q.g, D.s1 + q.g,
                                                          D.s2 + q.g, D.s3 + q.g, (int)q.n);
    d2d(D.mass, st_m, sizeof(double), 3);
    d2d(D.rho, st_r, sizeof(double), 3);
    d2d(D.hsml, st_h, sizeof(double), 3);
    d2d(D.itype, st_t, sizeof(int32_t), 3);
    for (int k = 0; k < 2; k++) {  // nodes and stress-points
      const Seg& q = sg[k];
      if (q.n == 0) continue;
      if (intvars1)
        SPS_CUDA_CHECK(cudaMemcpyAsync(D.iv1 + q.g, st_i + q.l, sizeof(double) * q.n, cudaMemcpyDeviceToDevice, c.stream));
      else
        SPS_CUDA_CHECK(cudaMemsetAsync(D.iv1 + q.g, 0, sizeof(double) * q.n, c.stream));
      if (f_drucker)
        SPS_CUDA_CHECK(cudaMemcpyAsync(D.fdp + q.g, st_f + q.l, sizeof(double) * q.n, cudaMemcpyDeviceToDevice, c.stream));
      else
        SPS_CUDA_CHECK(cudaMemsetAsync(D.fdp + q.g, 0, sizeof(double) * q.n, c.stream));
    }
    for (const Seg& q : sg)
      if (q.n > 0) SPS_CUDA_CHECK(cudaMemsetAsync(D.out + q.g, 0, q.n, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.dispx + M.node0, 0, sizeof(double) * nn, c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(D.dispy + M.node0, 0, sizeof(double) * nn, c.stream));
    for (const Seg& q : sg)
      if (q.n > 0) sps::launch_vol(c, (int)q.g, (int)(q.g + q.n));
    SPS_CUDA_CHECK(cudaMemsetAsync(c.d_chk, 0xff, 6 * sizeof(unsigned long long), c.stream));
    SPS_CUDA_CHECK(cudaMemsetAsync(c.d_chk + 6, 0, 2 * sizeof(unsigned long long), c.stream));
    if (n2 > 0)
      k_upload_check<<<std::min(nbk((int64_t)n2), 4 * 152), kBlock, 0, c.stream>>>(
          D.itype, D.px, D.py, D.hsml, sg[0].g, sg[0].n, sg[1].g, sg[1].n, sg[2].g, sg[2].n,
          c.d_chk);
    SPS_CUDA_CHECK(cudaGetLastError());
    SPS_CUDA_CHECK(cudaMemcpyAsync(c.h_chk, c.d_chk, 8 * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    sps::HostReal& hr = c.hr[r];
    if (c.h_chk[6]) {
      // the device state of r now holds the rejected arrays: r needs a valid upload
      hr.uploaded = false;
      c.uploaded = false;
      return fail(&c, SPS_ERR_ARG,
                  "sps_upload: itype must be 2 (nodes), then 1 (stress-points), then 25 (dummies)");
    }
    if (c.h_chk[7]) {
      hr.uploaded = false;
      c.uploaded = false;
      return fail(&c, SPS_ERR_ARG, "sps_upload: non-finite position or smoothing length");
    }
    double xmn[2] = {up_unkey(c.h_chk[0]), up_unkey(c.h_chk[1])};
    double xmx[2] = {up_unkey(~c.h_chk[2]), up_unkey(~c.h_chk[3])};
    double hmax = n2 ? up_unkey(~c.h_chk[4]) : 0.0;
    double hmin_nd = c.h_chk[5] == ~0ull ? 1e300 : up_unkey(c.h_chk[5]);
    if (n2 == 0) xmn[0] = xmn[1] = xmx[0] = xmx[1] = 0.0;
    // this realisation's extent, for the cell grid capacity (4x margin for spreading)
    double cell = 2.0 * hmax;
    double ncr = 1.0;
    for (int d = 0; d < 2; d++) ncr *= std::floor((xmx[d] - xmn[d]) / cell + 1.0) + 2.0;
    hr.ncells_est = ncr;
    hr.hmax = hmax;
    hr.hmin_nd = hmin_nd;
    hr.uploaded = true;
    double nc = 0.0;
    for (const sps::HostReal& q : c.hr) nc += q.ncells_est;
    int cap = (int)std::min(4.0 * nc + 1024.0, 2.0e9 / 4.0);
    if (cap > D.cell_cap) {
      D.cell_cnt = dalloc<int32_t>(c, (size_t)cap + 2);
      D.cell_start = dalloc<int32_t>(c, (size_t)cap + 2);
      D.cell_cursor = dalloc<int32_t>(c, (size_t)cap + 2);
      D.cell_cap = cap;
      size_t nscan = std::max<size_t>((size_t)D.N2, (size_t)cap + 2);
      D.scan_tmp = dalloc<int64_t>(c, nscan / 4096 + 64);
      drop_graphs(c);
    }
    // neighbour capacities: one species holds about pi (scale_k h / dx)^2 partners in the
    // support; 2x headroom plus the wall rows.  max_neighbours (total per particle) raises
    // or lowers the per-list capacity explicitly.
    {
      int est = 0;
      for (int q = 0; q < D.R; q++) {
        if (!c.hr[q].uploaded) continue;
        double rs = (double)D.scale_k * c.hr[q].hmax / c.hr[q].p.dx;
        // npoints stress-points per node spacing (both approaches)
        const double np = (double)std::max(1, c.hr[q].p.npoints);
        est = std::max(est, (int)std::ceil(2.0 * M_PI * rs * rs * np) + 8);
      }
      int capn = c.p.max_neighbours > 0 ? std::max(4, c.p.max_neighbours / 2) : std::max(48, est);
      capn = std::min(capn, 65535);  // half-list positions are kept in 16 bits
      if (capn > D.capH || (c.p.max_neighbours > 0 && capn != D.capH)) {
        D.half = dalloc<int4>(c, (size_t)D.N2 * (size_t)capn);
        // the lists hold their entries in pairs (ell()): an even number of rows
        const size_t rows = (size_t)capn + (capn & 1);
        D.cross = dalloc<int4>(c, (size_t)D.N2 * rows);
        D.same = dalloc<int4>(c, (size_t)D.N2 * rows);
        D.crossW = c.precision == SPS_PREC_FP32_FAST ? dalloc<int2>(c, (size_t)D.N2 * rows)
                                                     : nullptr;
        D.keyC = dalloc<int32_t>(c, (size_t)D.N2 * (size_t)capn);
        D.keyS = dalloc<int32_t>(c, (size_t)D.N2 * (size_t)capn);
        D.capH = D.capC = D.capS = capn;
        drop_graphs(c);
      }
    }
    // node-wall boundary force can use the pair lists when every node-dummy pair closer
    // than 0.75 dx is inside the kernel support (in every realisation)
    int bfl = 1;
    for (const sps::HostReal& q : c.hr)
      if (q.uploaded && !((double)D.scale_k * q.hmin_nd > 0.76 * q.p.dx)) bfl = 0;
    if (bfl != D.bound_from_lists) drop_graphs(c);
    D.bound_from_lists = bfl;
    // the FP32 form's interpolation reads the compact {id, W} entries that the gathered
    // lists also write
    const int uw = c.lists_direct() && D.crossW ? 1 : 0;
    if (uw != D.use_crossW) drop_graphs(c);
    D.use_crossW = uw;
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  bool all = true;
  for (const sps::HostReal& q : c.hr) all = all && q.uploaded;
  c.uploaded = all;
  c.surf_stale = false;  // an uploaded state carries its own bc_or_not
  c.itimestep = 0;       // the next step is the first of the run
  return SPS_OK;
}

int sps_upload_bcs(sps_ctx* h, const int32_t* bc_or_not, const int32_t* bc_info) {
  if (!h) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (c.d.R != 1) return fail(&c, SPS_ERR_UNSUPPORTED, "boundary conditions in a batch");
  try {
    const size_t NT = c.d.NT;
    if (bc_or_not)
      SPS_CUDA_CHECK(cudaMemcpyAsync(c.d.bc_or_not, bc_or_not, sizeof(int32_t) * NT, cudaMemcpyHostToDevice, c.stream));
    if (bc_info) {
      for (size_t i = 0; i < NT; i++)
        for (int r = 2; r < 7; r++) {
          int b = bc_info[8 * i + r];
          if (b < 0 || b > c.p.no_bcs)
            return fail(&c, SPS_ERR_ARG, "sps_upload_bcs: bc_info refers to a missing BC");
        }
      SPS_CUDA_CHECK(cudaMemcpyAsync(c.d.bc_info, bc_info, sizeof(int32_t) * 8 * NT, cudaMemcpyHostToDevice, c.stream));
    }
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_step(sps_ctx* h, int32_t nsteps, double* time_sph) {
  if (!h || !time_sph || nsteps < 0) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (!c.uploaded) return fail(&c, SPS_ERR_STATE, "sps_step before sps_upload");
  if (nsteps == 0) return SPS_OK;
  try {
    const int R = c.d.R;
    std::vector<double> t(time_sph, time_sph + R);
    const int chunk_max = std::max(16, std::min(4096, 65536 / R));
    int done = 0;
    while (done < nsteps) {
      int chunk = std::min(nsteps - done, chunk_max);
      ensure_scal(c, chunk);
      fill_table(c, chunk, t.data());
      SPS_CUDA_CHECK(cudaMemcpyAsync(c.d_scal_table, c.h_scal.data(),
                                     sizeof(sps::StepScalars) * c.h_scal.size(),
                                     cudaMemcpyHostToDevice, c.stream));
      SPS_CUDA_CHECK(cudaMemsetAsync(c.d.step_idx, 0, sizeof(int), c.stream));
      for (int k = 0; k < chunk; k++) enqueue_step(c);
      done += chunk;
    }
    int nb = (c.d.NT + kBlock - 1) / kBlock;
    k_check_finite<<<nb, kBlock, 0, c.stream>>>(c.d);
    SPS_CUDA_CHECK(cudaGetLastError());
    SPS_CUDA_CHECK(cudaMemcpyAsync(c.h_err, c.d.err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    c.steps_done += nsteps;
    if (c.d.update_x && !c.surf_every) c.surf_stale = true;
    for (int r = 0; r < R; r++) time_sph[r] = t[r];
    int e = *c.h_err;
    if (e) {
      SPS_CUDA_CHECK(cudaMemsetAsync(c.d.err, 0, sizeof(int), c.stream));
      SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
      if (e & (1 << 20)) return fail(&c, SPS_ERR_NONFINITE, err_text(e));
      if (e & sps::kErrTensorCore) return fail(&c, SPS_ERR_CUDA, err_text(e));
      return fail(&c, SPS_ERR_CAPACITY, err_text(e));
    }
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_download(sps_ctx* h, double* x, double* vel, double* stress, double* rho,
                 double* intvars1, double* displ, int32_t* bc_or_not, double* f_drucker) {
  if (!h) return SPS_ERR_ARG;
  if (h->c.d.R != 1)
    return fail(&h->c, SPS_ERR_ARG, "sps_download: a batch takes sps_download_real per realisation");
  return sps_download_real(h, 0, x, vel, stress, rho, intvars1, displ, bc_or_not, f_drucker);
}

int sps_download_real(sps_ctx* h, int32_t r, double* x, double* vel, double* stress, double* rho,
                      double* intvars1, double* displ, int32_t* bc_or_not, double* f_drucker) {
  if (!h) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  sps::Dev& D = c.d;
  if (r < 0 || r >= D.R) return fail(&c, SPS_ERR_ARG, "sps_download_real: no such realisation");
  const sps::Real& M = c.real[r];
  const size_t nn = M.nnode, nt = (size_t)M.nnode + M.nsp, n2 = nt + M.ndum;
  Seg sg[3];
  segments(c, r, sg);
  try {
    if (bc_or_not) refresh_surface(c, false);
    // the interleaved outputs are transposed into the staging buffer side by side, every
    // copy is enqueued, and the stream is synchronised once
    double* st_x = c.stage;
    double* st_v = st_x + 2 * n2;
    double* st_s = st_v + 2 * n2;
    double* st_d = st_s + 4 * n2;
    auto nbk = [](int64_t n) { return (int)((n + kBlock - 1) / kBlock); };
    auto down2 = [&](double* dst, double* st, const double* a, const double* b, int nseg, size_t n) {
      for (int k = 0; k < nseg; k++)
        if (sg[k].n > 0)
          k_soa_to_aos2<<<nbk(sg[k].n), kBlock, 0, c.stream>>>(st + 2 * sg[k].l, a + sg[k].g,
                                                                b + sg[k].g, (int)sg[k].n);
      SPS_CUDA_CHECK(cudaMemcpyAsync(dst, st, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, c.stream));
    };
    auto down1 = [&](void* dst, const void* src, size_t esz, int nseg) {
      for (int k = 0; k < nseg; k++)
        if (sg[k].n > 0)
          SPS_CUDA_CHECK(cudaMemcpyAsync((char*)dst + esz * sg[k].l, (const char*)src + esz * sg[k].g,
                                         esz * sg[k].n, cudaMemcpyDeviceToHost, c.stream));
    };
    if (x) down2(x, st_x, D.px, D.py, 3, n2);
    if (vel) down2(vel, st_v, D.vx, D.vy, 3, n2);
    if (displ) down2(displ, st_d, D.dispx, D.dispy, 1, nn);
    if (stress) {
      for (int k = 0; k < 2; k++) {
        const Seg& q = sg[k];
        if (q.n > 0)
          k_soa_to_aos4<<<nbk(q.n), kBlock, 0, c.stream>>>(st_s + 4 * q.l, D.s0 + q.g, D.s1 + q.g,
                                                            D.s2 + q.g, D.s3 + q.g, (int)q.n);
      }
      // dummy stress is pair-local in the reference; report zero like its RK4 clear (:690)
      if (n2 > nt)
        SPS_CUDA_CHECK(cudaMemsetAsync(st_s + 4 * nt, 0, sizeof(double) * 4 * (n2 - nt), c.stream));
      SPS_CUDA_CHECK(cudaMemcpyAsync(stress, st_s, sizeof(double) * 4 * n2, cudaMemcpyDeviceToHost, c.stream));
    }
    if (rho) down1(rho, D.rho, sizeof(double), 3);
    if (intvars1) down1(intvars1, D.iv1, sizeof(double), 2);
    if (bc_or_not) down1(bc_or_not, D.bc_or_not, sizeof(int32_t), 2);
    if (f_drucker) down1(f_drucker, D.fdp, sizeof(double), 2);
    SPS_CUDA_CHECK(cudaGetLastError());
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

// ---- output snapshot -------------------------------------------------------------------

int sps_snapshot(sps_ctx* h) {
  if (!h) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (!c.uploaded) return fail(&c, SPS_ERR_STATE, "sps_snapshot before sps_upload");
  sps::Dev& D = c.d;
  try {
    if (!c.snap_dev) {
      // one block per realisation in the layout sps_download returns
      std::vector<int64_t> roff(D.R + 1, 0);
      for (int r = 0; r < D.R; r++) {
        const sps::Real& M = c.real[r];
        const int64_t nt = (int64_t)M.nnode + M.nsp;
        roff[r + 1] = roff[r] + (int64_t)snap_block(M.nnode, nt, nt + M.ndum).bytes;
      }
      c.snap_roff = roff;
      c.snap_bytes = (size_t)roff[D.R];
      void* p = nullptr;
      SPS_CUDA_CHECK(cudaMalloc(&p, c.snap_bytes + sizeof(int64_t) * (D.R + 1)));
      c.snap_dev = static_cast<char*>(p);
      SPS_CUDA_CHECK(cudaMemcpy(c.snap_dev + c.snap_bytes, roff.data(), sizeof(int64_t) * (D.R + 1),
                                cudaMemcpyHostToDevice));
      SPS_CUDA_CHECK(cudaMallocHost(&p, c.snap_bytes));
      c.snap_host = static_cast<char*>(p);
      SPS_CUDA_CHECK(cudaStreamCreateWithFlags(&c.snap_stream, cudaStreamNonBlocking));
      SPS_CUDA_CHECK(cudaEventCreateWithFlags(&c.snap_ready, cudaEventDisableTiming));
      SPS_CUDA_CHECK(cudaEventCreateWithFlags(&c.snap_done, cudaEventDisableTiming));
    }
    // the host copy of an earlier snapshot must have left the device buffer
    if (c.snap_pending) SPS_CUDA_CHECK(cudaStreamWaitEvent(c.stream, c.snap_done, 0));
    refresh_surface(c, false);
    if (D.N2 > 0)
      k_snap_pack<<<(D.N2 + kBlock - 1) / kBlock, kBlock, 0, c.stream>>>(
          D, c.snap_dev, reinterpret_cast<const int64_t*>(c.snap_dev + c.snap_bytes));
    SPS_CUDA_CHECK(cudaGetLastError());
    SPS_CUDA_CHECK(cudaEventRecord(c.snap_ready, c.stream));
    SPS_CUDA_CHECK(cudaStreamWaitEvent(c.snap_stream, c.snap_ready, 0));
    SPS_CUDA_CHECK(cudaMemcpyAsync(c.snap_host, c.snap_dev, c.snap_bytes, cudaMemcpyDeviceToHost,
                                   c.snap_stream));
    SPS_CUDA_CHECK(cudaEventRecord(c.snap_done, c.snap_stream));
    c.snap_pending = true;
    c.snap_valid = false;
    c.snap_step = c.steps_done;
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

namespace {
// block until the snapshot has reached host memory
int snapshot_ready(sps::Ctx& c, int32_t r, const char* who) {
  if (r < 0 || r >= c.d.R) return fail(&c, SPS_ERR_ARG, std::string(who) + ": no such realisation");
  if (!c.snap_pending && !c.snap_valid)
    return fail(&c, SPS_ERR_STATE, std::string(who) + " without sps_snapshot");
  try {
    if (c.snap_pending) {
      SPS_CUDA_CHECK(cudaEventSynchronize(c.snap_done));
      c.snap_pending = false;
      c.snap_valid = true;
    }
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}
}  // namespace

int sps_snapshot_view(sps_ctx* h, int32_t r, const double** x, const double** vel,
                      const double** stress, const double** rho, const double** intvars1,
                      const double** displ, const int32_t** bc_or_not, const double** f_drucker,
                      int64_t* step) {
  if (!h) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  int rc = snapshot_ready(c, r, "sps_snapshot_view");
  if (rc != SPS_OK) return rc;
  const sps::Real& M = c.real[r];
  const int64_t nn = M.nnode, nt = nn + M.nsp, n2 = nt + M.ndum;
  const SnapBlock b = snap_block(nn, nt, n2);
  const char* base = c.snap_host + c.snap_roff[r];
  auto D = [&](size_t off) { return reinterpret_cast<const double*>(base + off); };
  if (x) *x = D(b.x);
  if (vel) *vel = D(b.vel);
  if (stress) *stress = D(b.stress);
  if (rho) *rho = D(b.rho);
  if (intvars1) *intvars1 = D(b.iv1);
  if (displ) *displ = D(b.displ);
  if (bc_or_not) *bc_or_not = reinterpret_cast<const int32_t*>(base + b.bc);
  if (f_drucker) *f_drucker = D(b.fdp);
  if (step) *step = c.snap_step;
  return SPS_OK;
}

int sps_snapshot_wait(sps_ctx* h, int32_t r, double* x, double* vel, double* stress, double* rho,
                      double* intvars1, double* displ, int32_t* bc_or_not, double* f_drucker,
                      int64_t* step) {
  if (!h) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  int rc = snapshot_ready(c, r, "sps_snapshot_wait");
  if (rc != SPS_OK) return rc;
  const sps::Real& M = c.real[r];
  const int64_t nn = M.nnode, nt = nn + M.nsp, n2 = nt + M.ndum;
  const SnapBlock b = snap_block(nn, nt, n2);
  const char* base = c.snap_host + c.snap_roff[r];
  auto put = [&](void* dst, size_t off, size_t bytes) {
    if (dst && bytes) std::memcpy(dst, base + off, bytes);
  };
  put(x, b.x, 16 * n2);
  put(vel, b.vel, 16 * n2);
  put(stress, b.stress, 32 * n2);
  put(rho, b.rho, 8 * n2);
  put(intvars1, b.iv1, 8 * nt);
  put(f_drucker, b.fdp, 8 * nt);
  put(displ, b.displ, 16 * nn);
  put(bc_or_not, b.bc, 4 * nt);
  if (step) *step = c.snap_step;
  return SPS_OK;
}

int sps_download_surface(sps_ctx* h, int32_t r, double* normal, int32_t* subset) {
  if (!h) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  sps::Dev& D = c.d;
  if (r < 0 || r >= D.R) return fail(&c, SPS_ERR_ARG, "sps_download_surface: no such realisation");
  Seg sg[3];
  segments(c, r, sg);
  try {
    refresh_surface(c);
    for (int k = 0; k < 2; k++) {  // nodes and stress-points
      const Seg& q = sg[k];
      if (q.n == 0) continue;
      if (normal) {
        std::vector<double> nx(q.n), ny(q.n);
        SPS_CUDA_CHECK(cudaMemcpy(nx.data(), D.nrmx + q.g, sizeof(double) * q.n, cudaMemcpyDeviceToHost));
        SPS_CUDA_CHECK(cudaMemcpy(ny.data(), D.nrmy + q.g, sizeof(double) * q.n, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < q.n; i++) {
          normal[2 * (q.l + i)] = nx[i];
          normal[2 * (q.l + i) + 1] = ny[i];
        }
      }
      if (subset) {
        std::vector<int8_t> sb(q.n);
        SPS_CUDA_CHECK(cudaMemcpy(sb.data(), D.subset + q.g, q.n, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < q.n; i++) subset[q.l + i] = sb[i];
      }
    }
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_dump_pairs(sps_ctx* h, int32_t* pair_i, int32_t* pair_j, int32_t* pint_type, float* w,
                   float* dwdx, float* dwdy, int64_t* npairs) {
  if (!h) return SPS_ERR_ARG;
  if (h->c.d.R != 1)
    return fail(&h->c, SPS_ERR_ARG, "sps_dump_pairs: a batch takes sps_dump_pairs_real");
  return sps_dump_pairs_real(h, 0, pair_i, pair_j, pint_type, w, dwdx, dwdy, npairs);
}

int sps_dump_pairs_real(sps_ctx* h, int32_t r, int32_t* pair_i, int32_t* pair_j,
                        int32_t* pint_type, float* w, float* dwdx, float* dwdy, int64_t* npairs) {
  if (!h || !npairs) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  sps::Dev& D = c.d;
  if (r < 0 || r >= D.R) return fail(&c, SPS_ERR_ARG, "sps_dump_pairs_real: no such realisation");
  try {
    sps::PairMeta meta;
    sps::Grid g;
    sps::GridTotal gt;
    SPS_CUDA_CHECK(cudaMemcpy(&meta, D.meta + r, sizeof(meta), cudaMemcpyDeviceToHost));
    if (!pair_i) {
      *npairs = meta.n;
      return SPS_OK;
    }
    if (*npairs < meta.n) return fail(&c, SPS_ERR_CAPACITY, "sps_dump_pairs: buffer too small");
    sps::ensure_half_lists(c);  // after a step that gathered its lists directly
    SPS_CUDA_CHECK(cudaGetLastError());
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    SPS_CUDA_CHECK(cudaMemcpy(&g, D.grid + r, sizeof(g), cudaMemcpyDeviceToHost));
    SPS_CUDA_CHECK(cudaMemcpy(&gt, D.gtot, sizeof(gt), cudaMemcpyDeviceToHost));
    int32_t lohi[2] = {0, 0};
    if (!gt.overflow) {
      SPS_CUDA_CHECK(cudaMemcpy(&lohi[0], D.cell_start + g.cell0, sizeof(int32_t), cudaMemcpyDeviceToHost));
      SPS_CUDA_CHECK(cudaMemcpy(&lohi[1], D.cell_start + g.cell0 + g.ncells, sizeof(int32_t),
                                cudaMemcpyDeviceToHost));
    }
    const size_t N2 = D.N2, lo = lohi[0], hi = lohi[1];
    std::vector<int32_t> cnt(N2), sorted(N2), itype(N2);
    std::vector<int4> half((hi - lo) * D.capH + 1);
    SPS_CUDA_CHECK(cudaMemcpy(cnt.data(), D.half_cnt, sizeof(int32_t) * N2, cudaMemcpyDeviceToHost));
    SPS_CUDA_CHECK(cudaMemcpy(sorted.data(), D.sorted, sizeof(int32_t) * N2, cudaMemcpyDeviceToHost));
    SPS_CUDA_CHECK(cudaMemcpy(itype.data(), D.itype, sizeof(int32_t) * N2, cudaMemcpyDeviceToHost));
    if (hi > lo)
      SPS_CUDA_CHECK(cudaMemcpy(half.data(), D.half + lo * D.capH, sizeof(int4) * (hi - lo) * D.capH,
                                cudaMemcpyDeviceToHost));
    const sps::Real& M = c.real[r];
    auto local = [&](int gid) -> int32_t {  // global id -> 1-based reference id of r
      if (gid < D.NN) return gid - M.node0 + 1;
      if (gid < D.NT) return M.nnode + (gid - M.sp0) + 1;
      return M.nnode + M.nsp + (gid - M.dum0) + 1;
    };
    // creation order
    std::vector<int32_t> ci, cj, ct;
    std::vector<float> cw, cx, cy;
    ci.reserve(meta.n);
    for (size_t s = lo; s < hi; s++)
      for (int k = 0; k < cnt[s]; k++) {
        const int4 e = half[(s - lo) * D.capH + k];
        int a = sorted[s], b = (int)((unsigned)e.x & ((1u << 28) - 1u));  // the partner's id
        float ww, gx, gy;
        std::memcpy(&ww, &e.y, 4);
        std::memcpy(&gx, &e.z, 4);
        std::memcpy(&gy, &e.w, 4);
        int ta = itype[a], tb = itype[b];
        int ia = std::abs(ta), ib = std::abs(tb);
        // Pint_Update orientation (3_SPH_material_2018.f90:1599-1614)
        if ((ia == 2 && ib == 1) || (ia == 2 && ib == 25) || (ia == 1 && ib == 25)) {
          std::swap(a, b);
          gx = -gx;
          gy = -gy;
        }
        int sum = ta + tb;
        int t = sum == 3 ? 1 : sum == 2 ? 2 : sum == 4 ? 3 : sum == 27 ? 6 : sum == 26 ? 9 : 0;
        ci.push_back(local(a));
        cj.push_back(local(b));
        ct.push_back(t);
        cw.push_back(ww);
        cx.push_back(gx);
        cy.push_back(gy);
      }
    int64_t n = (int64_t)ci.size(), m = meta.m_prev, k = 0;
    auto put = [&](int64_t q) {
      pair_i[k] = ci[q];
      pair_j[k] = cj[q];
      if (pint_type) pint_type[k] = ct[q];
      if (w) w[k] = cw[q];
      if (dwdx) dwdx[k] = cx[q];
      if (dwdy) dwdy[k] = cy[q];
      k++;
    };
    for (int64_t a = n - 1; a >= m; a--) put(a);
    for (int64_t a = 0; a < std::min(n, m); a++) put(a);
    *npairs = n;
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_kernels_per_step(sps_ctx* h, int32_t* n) {
  if (!h || !n) return SPS_ERR_ARG;
  try {
    if (!h->c.graphs[h->c.step_variant]) build_graph(h->c);
  } catch (const std::exception& e) {
    return fail(&h->c, SPS_ERR_CUDA, e.what());
  }
  *n = h->c.kernels_per_step;
  return SPS_OK;
}

int sps_selftest_division(sps_ctx* h, int64_t n, uint64_t seed, int64_t* mismatches) {
  if (!h || !mismatches || n < 0) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  try {
    unsigned long long* d = nullptr;
    SPS_CUDA_CHECK(cudaMalloc(&d, sizeof(unsigned long long)));
    SPS_CUDA_CHECK(cudaMemsetAsync(d, 0, sizeof(unsigned long long), c.stream));
    sps::launch_selftest_div(c, n, seed, d);
    unsigned long long v = 0;
    SPS_CUDA_CHECK(cudaMemcpyAsync(&v, d, sizeof(v), cudaMemcpyDeviceToHost, c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    cudaFree(d);
    *mismatches = (int64_t)v;
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_selftest_cone(sps_ctx* h, int64_t n, uint64_t seed, int64_t* mismatches,
                      int64_t* certified) {
  if (!h || !mismatches || !certified || n < 0) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  try {
    unsigned long long* d = nullptr;
    SPS_CUDA_CHECK(cudaMalloc(&d, 2 * sizeof(unsigned long long)));
    SPS_CUDA_CHECK(cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), c.stream));
    sps::launch_selftest_cone(c, n, seed, d);
    SPS_CUDA_CHECK(cudaGetLastError());
    unsigned long long v[2] = {0, 0};
    SPS_CUDA_CHECK(cudaMemcpyAsync(v, d, sizeof(v), cudaMemcpyDeviceToHost, c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    cudaFree(d);
    *mismatches = (int64_t)v[0];
    *certified = (int64_t)v[1];
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_selftest_convert(sps_ctx* h, int64_t n, uint64_t seed, int64_t* mismatches) {
  if (!h || !mismatches || n < 0) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  try {
    unsigned long long* d = nullptr;
    SPS_CUDA_CHECK(cudaMalloc(&d, sizeof(unsigned long long)));
    SPS_CUDA_CHECK(cudaMemsetAsync(d, 0, sizeof(unsigned long long), c.stream));
    sps::launch_selftest_conv(c, n, seed, d);
    unsigned long long v = 0;
    SPS_CUDA_CHECK(cudaMemcpyAsync(&v, d, sizeof(v), cudaMemcpyDeviceToHost, c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    cudaFree(d);
    *mismatches = (int64_t)v;
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_set_surface_detection(sps_ctx* h, int32_t exact) {
  if (!h || (exact != 0 && exact != 1)) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (c.surface_exact == (exact != 0)) return SPS_OK;
  try {
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    c.surface_exact = exact != 0;
    // the step graphs that write the lists for a download differ between the two
    c.keys_written = c.same_written = false;
    drop_graphs(c);
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_tuned_lookahead(sps_ctx* h, int32_t* ahead) {
  if (!h || !ahead) return SPS_ERR_ARG;
  ahead[0] = h->c.ahead[0];
  ahead[1] = h->c.ahead[1];
  return SPS_OK;
}

int sps_tuned_prefetch(sps_ctx* h, int32_t* flags) {
  if (!h || !flags) return SPS_ERR_ARG;
  *flags = h->c.d.l2_prefetch;
  return SPS_OK;
}

int sps_set_prefetch(sps_ctx* h, int32_t flags) {
  if (!h) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (flags < 0 || flags > 3) return fail(&c, SPS_ERR_ARG, "sps_set_prefetch: flags 0 .. 3");
  try {
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    c.d.l2_prefetch = flags;
    drop_graphs(c);
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_set_lookahead(sps_ctx* h, int32_t interp, int32_t derivs) {
  if (!h) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if ((interp != 2 && interp != 4 && interp != 8) || (derivs != 1 && derivs != 2 && derivs != 4))
    return fail(&c, SPS_ERR_ARG, "sps_set_lookahead: interp 2, 4 or 8; derivs 1, 2 or 4");
  try {
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    c.ahead[0] = interp;
    c.ahead[1] = derivs;
    drop_graphs(c);
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_get_stream(sps_ctx* h, void** stream) {
  if (!h || !stream) return SPS_ERR_ARG;
  *stream = (void*)h->c.stream;
  return SPS_OK;
}

namespace {
void profile_run(sps::Ctx& c, int nsteps, double* t, std::vector<std::string>& kn,
                 std::vector<double>& kms, std::vector<int>& kl);
}  // namespace

int sps_profile_step(sps_ctx* h, int32_t nsteps, double* time_sph, char* names, int32_t names_len,
                     double* ms, int32_t* launches, int32_t cap, int32_t* nkernels) {
  if (!h || !time_sph || nsteps <= 0 || !names || !ms || !launches || !nkernels)
    return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (!c.uploaded) return fail(&c, SPS_ERR_STATE, "sps_profile_step before sps_upload");
  std::vector<std::string> kn;
  std::vector<double> kms;
  std::vector<int> kl;
  try {
    std::vector<double> t(time_sph, time_sph + c.d.R);
    profile_run(c, nsteps, t.data(), kn, kms, kl);
    SPS_CUDA_CHECK(cudaMemcpy(c.h_err, c.d.err, sizeof(int), cudaMemcpyDeviceToHost));
    for (int r = 0; r < c.d.R; r++) time_sph[r] = t[r];
    c.steps_done += nsteps;
    if (c.d.update_x && !c.surf_every) c.surf_stale = true;
  } catch (const std::exception& e) {
    c.profiling = false;
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  int n = (int)std::min<size_t>(kn.size(), (size_t)cap);
  size_t off = 0;
  for (int k = 0; k < n; k++) {
    size_t L = kn[k].size() + 1;
    if (off + L <= (size_t)names_len) {
      std::memcpy(names + off, kn[k].c_str(), L);
      off += L;
    }
    ms[k] = kms[k];
    launches[k] = kl[k];
  }
  *nkernels = n;
  if (*c.h_err) {
    int e = *c.h_err;
    cudaMemset(c.d.err, 0, sizeof(int));
    return fail(&c, SPS_ERR_CAPACITY, err_text(e));
  }
  return SPS_OK;
}

namespace {

// nsteps steps with CUDA events around every kernel group (no graph): per-group totals
void profile_run(sps::Ctx& c, int nsteps, double* t, std::vector<std::string>& kn,
                 std::vector<double>& kms, std::vector<int>& kl) {
  ensure_scal(c, nsteps);
  fill_table(c, nsteps, t);
  SPS_CUDA_CHECK(cudaMemcpyAsync(c.d_scal_table, c.h_scal.data(),
                                 sizeof(sps::StepScalars) * c.h_scal.size(),
                                 cudaMemcpyHostToDevice, c.stream));
  SPS_CUDA_CHECK(cudaMemsetAsync(c.d.step_idx, 0, sizeof(int), c.stream));
  c.profiling = true;
  for (int k = 0; k < nsteps; k++) {
    enqueue_step(c);
    c.mark("end");
  }
  c.profiling = false;
  SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
  SPS_CUDA_CHECK(cudaGetLastError());
  for (size_t k = 0; k + 1 < c.prof_events.size(); k++) {
    const char* nm = c.prof_events[k].first;
    if (std::strcmp(nm, "end") == 0) continue;
    float e = 0.0f;
    cudaEventElapsedTime(&e, c.prof_events[k].second, c.prof_events[k + 1].second);
    size_t q = 0;
    while (q < kn.size() && kn[q] != nm) q++;
    if (q == kn.size()) {
      kn.push_back(nm);
      kms.push_back(0.0);
      kl.push_back(0);
    }
    kms[q] += e;
    kl[q] += 1;
  }
  for (auto& pe : c.prof_events) cudaEventDestroy(pe.second);
  c.prof_events.clear();
}

// the surrogate's counters and its gate, one allocation
constexpr size_t kSurrBytes = 4 * sizeof(unsigned long long) + sizeof(sps::SurrGate);

// the gate's starting state: on, probing every step, with the context's policy
void reset_gate(sps::Ctx& c) {
  sps::SurrGate g = {};
  g.on = 1;
  g.wait = 0;
  g.period = 1;
  g.max_period = c.gate_max_period;
  g.min_frac = c.gate_min_frac;
  SPS_CUDA_CHECK(cudaMemcpyAsync(c.d.surr_gate, &g, sizeof(g), cudaMemcpyHostToDevice, c.stream));
  SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
}

// the device arrays a step carries over from the previous step (or the upload)
std::vector<std::pair<void*, size_t>> carried_state(sps::Ctx& c) {
  sps::Dev& D = c.d;
  const size_t N2 = D.N2, NT = D.NT, NN = D.NN, d8 = sizeof(double);
  std::vector<std::pair<void*, size_t>> v = {
      {D.px, d8 * N2},   {D.py, d8 * N2},    {D.vx, d8 * N2},      {D.vy, d8 * N2},
      {D.s0, d8 * N2},   {D.s1, d8 * N2},    {D.s2, d8 * N2},      {D.s3, d8 * N2},
      {D.rho, d8 * N2},  {D.hsml, d8 * N2},  {D.vol, d8 * N2},     {D.rinv, d8 * N2},
      {D.iv1, d8 * NT},  {D.fdp, d8 * NT},   {D.grad_u, 4 * d8 * NT},
      {D.dispx, d8 * NN}, {D.dispy, d8 * NN}, {D.bc_or_not, sizeof(int32_t) * NT},
      {D.out, N2},       {D.meta, sizeof(sps::PairMeta) * D.R},
      {D.nrmx, d8 * NT}, {D.nrmy, d8 * NT}, {D.subset, NT}, {D.fint, sizeof(float) * NT},
      {D.bc_int, sizeof(int32_t) * NN}};
  if (D.vel_vector) {
    v.push_back({D.x10x, d8 * NN});
    v.push_back({D.x10y, d8 * NN});
    v.push_back({D.disp10, d8 * NN});
  }
  if (D.fast) {
    v.push_back({D.recV, sizeof(float4) * N2});
    v.push_back({D.recS, sizeof(float4) * NT});
    v.push_back({D.recI, sizeof(float4) * N2});
    v.push_back({D.recA, sizeof(float4) * NT});
    v.push_back({D.recAl, sizeof(float4) * NT});
  }
  if (c.surr_cnt) v.push_back({c.surr_cnt, kSurrBytes});
  if (c.cap_cnt) v.push_back({c.cap_cnt, sizeof(unsigned long long)});
  return v;
}

}  // namespace

int sps_autotune(sps_ctx* h, int32_t nsteps, int32_t* blocks) {
  if (!h || nsteps <= 0) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (!c.uploaded) return fail(&c, SPS_ERR_STATE, "sps_autotune before sps_upload");
  void* snap = nullptr;
  try {
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    auto st = carried_state(c);
    size_t total = 0;
    for (auto& a : st) total += (a.second + 255) & ~size_t(255);
    SPS_CUDA_CHECK(cudaMalloc(&snap, total));
    auto copy = [&](bool save) {
      size_t off = 0;
      for (auto& a : st) {
        char* sp = static_cast<char*>(snap) + off;
        if (save) SPS_CUDA_CHECK(cudaMemcpyAsync(sp, a.first, a.second, cudaMemcpyDeviceToDevice, c.stream));
        else SPS_CUDA_CHECK(cudaMemcpyAsync(a.first, sp, a.second, cudaMemcpyDeviceToDevice, c.stream));
        off += (a.second + 255) & ~size_t(255);
      }
      SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    };
    copy(true);
    // the profiled steps overwrite the pair tables: detect a pending free surface first
    refresh_surface(c);
    const bool stale = c.surf_stale;
    const int64_t it0 = c.itimestep;
    const bool kin = c.keys_in_step, kw = c.keys_written, sw = c.same_written;
    const int cand[] = {64, 128, 256, 512};
    int best[sps::TK_N];
    double best_ms[sps::TK_N];
    for (int k = 0; k < sps::TK_N; k++) {
      best[k] = c.blk[k];
      best_ms[k] = 1e300;
    }
    std::vector<double> t(c.d.R, 0.0);
    for (int b : cand) {
      for (int k = 0; k < sps::TK_N; k++) c.blk[k] = std::min(b, sps::kTunedMax[k]);
      std::vector<std::string> kn;
      std::vector<double> kms;
      std::vector<int> kl;
      std::fill(t.begin(), t.end(), 0.0);
      c.itimestep = it0;
      profile_run(c, nsteps, t.data(), kn, kms, kl);
      copy(false);
      for (int k = 0; k < sps::TK_N; k++)
        for (size_t q = 0; q < kn.size(); q++)
          // the FP32 form's direct list gather takes the pair search's block size
          if ((kn[q] == sps::kTunedNames[k] || (k == sps::TK_HALF && kn[q] == "gather")) &&
              kms[q] < best_ms[k]) {
            best_ms[k] = kms[q];
            best[k] = c.blk[k];
          }
    }
    for (int k = 0; k < sps::TK_N; k++) {
      c.blk[k] = best[k];
      if (blocks) blocks[k] = best[k];
    }
    // FP32 form: the neighbour sums' look-ahead (neighbours loaded before any is summed),
    // at the chosen block sizes; the two groups are timed in the same profiled steps
    if (c.precision == SPS_PREC_FP32_FAST && c.d.sp_sph) {
      const int la[4][2] = {{2, 1}, {2, 2}, {4, 2}, {8, 4}};
      int best_la[2] = {c.ahead[0], c.ahead[1]};
      double best_la_ms[2] = {1e300, 1e300};
      const char* names[2] = {"interp", "derivs"};
      for (const auto& v : la) {
        c.ahead[0] = v[0];
        c.ahead[1] = v[1];
        std::vector<std::string> kn;
        std::vector<double> kms;
        std::vector<int> kl;
        std::fill(t.begin(), t.end(), 0.0);
        c.itimestep = it0;
        profile_run(c, nsteps, t.data(), kn, kms, kl);
        copy(false);
        for (int g = 0; g < 2; g++)
          for (size_t q = 0; q < kn.size(); q++)
            if (kn[q] == names[g] && kms[q] < best_la_ms[g]) {
              best_la_ms[g] = kms[q];
              best_la[g] = v[g];
            }
      }
      c.ahead[0] = best_la[0];
      c.ahead[1] = best_la[1];
      // then the bulk L2 prefetch of the list entries, off and on for both groups
      double best_pf_ms[2] = {1e300, 1e300};
      int best_pf = 0;
      for (int pf : {0, 3}) {
        c.d.l2_prefetch = pf;
        std::vector<std::string> kn;
        std::vector<double> kms;
        std::vector<int> kl;
        std::fill(t.begin(), t.end(), 0.0);
        c.itimestep = it0;
        profile_run(c, nsteps, t.data(), kn, kms, kl);
        copy(false);
        for (int g = 0; g < 2; g++)
          for (size_t q = 0; q < kn.size(); q++)
            if (kn[q] == names[g] && kms[q] < best_pf_ms[g]) {
              best_pf_ms[g] = kms[q];
              best_pf = (best_pf & ~(1 << g)) | (pf & (1 << g));
            }
      }
      c.d.l2_prefetch = best_pf;
    }
    c.surf_stale = stale;
    c.itimestep = it0;
    c.keys_in_step = kin;
    c.keys_written = kw;
    c.same_written = sw;
    SPS_CUDA_CHECK(cudaMemsetAsync(c.d.err, 0, sizeof(int), c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    cudaFree(snap);
    snap = nullptr;
    drop_graphs(c);
  } catch (const std::exception& e) {
    c.profiling = false;
    if (snap) cudaFree(snap);
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_last_error(sps_ctx* h, char* buf, int32_t len) {
  std::string m;
  if (h) m = h->c.last_error;
  else {
    std::lock_guard<std::mutex> g(g_err_mu);
    m = g_create_error;
  }
  if (buf && len > 0) std::snprintf(buf, (size_t)len, "%s", m.c_str());
  return (int)m.size();
}

void sps_destroy(sps_ctx* h) {
  if (!h) return;
  sps::Ctx& c = h->c;
  sps::drop_graphs(c);
  if (c.stream) cudaStreamSynchronize(c.stream);
  for (void* p : {(void*)c.cap_buf, (void*)c.cap_cnt, (void*)c.mlp_frag, (void*)c.mlp_bias,
                  (void*)c.surr_cnt, c.surr_rows, c.tc_img})
    if (p) cudaFree(p);
  for (void* p : c.allocs) cudaFree(p);
  if (c.h_err) cudaFreeHost(c.h_err);
  if (c.h_chk) cudaFreeHost(c.h_chk);
  if (c.snap_stream) {
    cudaStreamSynchronize(c.snap_stream);
    cudaStreamDestroy(c.snap_stream);
  }
  if (c.snap_ready) cudaEventDestroy(c.snap_ready);
  if (c.snap_done) cudaEventDestroy(c.snap_done);
  if (c.snap_dev) cudaFree(c.snap_dev);
  if (c.snap_host) cudaFreeHost(c.snap_host);
  if (c.up_stream) cudaStreamDestroy(c.up_stream);
  if (c.up_ready) cudaEventDestroy(c.up_ready);
  if (c.stream) cudaStreamDestroy(c.stream);
  delete h;
}

// ---- learned surrogate: capture and installation (include/sps_surrogate.h) ----------------

int sps_capture(sps_ctx* h, int64_t cap) {
  if (!h || cap < 0) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  try {
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    if (c.cap_buf) cudaFree(c.cap_buf);
    c.cap_buf = nullptr;
    c.d.cap_buf = nullptr;
    c.d.cap_max = 0;
    if (cap > 0) {
      if (!c.cap_cnt) {
        void* p = nullptr;
        SPS_CUDA_CHECK(cudaMalloc(&p, sizeof(unsigned long long)));
        c.cap_cnt = static_cast<unsigned long long*>(p);
      }
      void* p = nullptr;
      SPS_CUDA_CHECK(cudaMalloc(&p, sizeof(float) * SPS_MLP_TUPLE * (size_t)cap));
      c.cap_buf = static_cast<float*>(p);
      SPS_CUDA_CHECK(cudaMemsetAsync(c.cap_cnt, 0, sizeof(unsigned long long), c.stream));
      c.d.cap_buf = c.cap_buf;
      c.d.cap_cnt = c.cap_cnt;
      c.d.cap_max = cap;
    }
    drop_graphs(c);
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_capture_read(sps_ctx* h, float* tuples, int64_t* n, int64_t* seen) {
  if (!h || !n || *n < 0 || (*n > 0 && !tuples)) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (!c.cap_buf) return fail(&c, SPS_ERR_STATE, "sps_capture_read without sps_capture");
  try {
    unsigned long long cnt = 0;
    SPS_CUDA_CHECK(cudaMemcpyAsync(&cnt, c.cap_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    int64_t held = std::min<int64_t>((int64_t)cnt, c.d.cap_max);
    int64_t k = std::min<int64_t>(held, *n);
    if (k > 0)
      SPS_CUDA_CHECK(cudaMemcpyAsync(tuples, c.cap_buf, sizeof(float) * SPS_MLP_TUPLE * (size_t)k,
                                     cudaMemcpyDeviceToHost, c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    *n = k;
    if (seen) *seen = (int64_t)cnt;
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_surrogate_install(sps_ctx* h, sps_mlp* m, const sps_surrogate_opts* o) {
  if (!h || (m && !o)) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (m && c.precision != SPS_PREC_FP32_FAST)
    return fail(&c, SPS_ERR_UNSUPPORTED, "the surrogate runs in the FP32 form only");
  try {
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    if (m) {
      if (!c.mlp_frag) {
        void* p = nullptr;
        SPS_CUDA_CHECK(cudaMalloc(&p, sizeof(uint2) * sps::MLP_FRAG_U2));
        c.mlp_frag = static_cast<uint2*>(p);
        SPS_CUDA_CHECK(cudaMalloc(&p, sizeof(float) * sps::MLP_BIAS));
        c.mlp_bias = static_cast<float*>(p);
        SPS_CUDA_CHECK(cudaMalloc(&p, kSurrBytes));
        c.surr_cnt = static_cast<unsigned long long*>(p);
      }
      const size_t ns = (size_t)(c.d.NT - c.d.NN);
      if (!c.surr_rows) {
        // xcand (16 ns floats; its rows are written as float4, so it comes first, at the
        // allocation's alignment), ycand (4 ns floats), cand_row (ns ints), cand_count (4 ints)
        void* p = nullptr;
        SPS_CUDA_CHECK(cudaMalloc(&p, sizeof(float) * 20 * ns + sizeof(int) * ns + 64));
        c.surr_rows = p;
        SPS_CUDA_CHECK(cudaMalloc(&p, sps::mlp_tc_image_bytes() +
                                          sizeof(float) * sps::mlp_tc_bias_count()));
        c.tc_img = p;
        SPS_CUDA_CHECK(sps::mlp_tc_prepare());
        int nsm = 0;
        SPS_CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));
        c.tc_grid = sps::mlp_tc_grid((int)ns, nsm);
      }
      {
        char* b = static_cast<char*>(c.surr_rows);
        c.d.xcand = reinterpret_cast<float*>(b);
        c.d.ycand = c.d.xcand + 16 * ns;
        c.d.cand_row = reinterpret_cast<int*>(c.d.ycand + 4 * ns);
        c.d.cand_count = c.d.cand_row + ns;
        c.d.tc_img = c.tc_img;
        c.d.tc_bias = reinterpret_cast<const float*>(static_cast<char*>(c.tc_img) +
                                                     sps::mlp_tc_image_bytes());
      }
      cudaStream_t ms = sps::mlp_stream(m);
      SPS_CUDA_CHECK(cudaStreamSynchronize(ms));
      sps::mlp_pack(m, c.mlp_frag, c.mlp_bias, ms);
      sps::mlp_tc_pack(sps::mlp_params(m), c.tc_img, const_cast<float*>(c.d.tc_bias), ms);
      SPS_CUDA_CHECK(cudaGetLastError());
      SPS_CUDA_CHECK(cudaStreamSynchronize(ms));
      SPS_CUDA_CHECK(cudaMemsetAsync(c.surr_cnt, 0, sizeof(unsigned long long) * 4, c.stream));
      c.d.surr = 1;
      c.d.mlp_frag = c.mlp_frag;
      c.d.mlp_bias = c.mlp_bias;
      c.d.surr_cnt = c.surr_cnt;
      c.d.surr_gate = reinterpret_cast<sps::SurrGate*>(c.surr_cnt + 4);
      reset_gate(c);
      c.d.surr_tol = o->tol;
      for (int k = 0; k < SPS_MLP_NIN; k++) {
        c.d.env_lo[k] = o->env_lo[k];
        c.d.env_hi[k] = o->env_hi[k];
      }
      c.d.out_max = o->out_max;
    } else {
      c.d.surr = 0;
    }
    drop_graphs(c);
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_surrogate_gate(sps_ctx* h, double min_answered, int32_t max_period) {
  if (!h || !(min_answered <= 1.0) || max_period < 1) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  c.gate_min_frac = min_answered;
  c.gate_max_period = max_period;
  if (!c.surr_cnt) return SPS_OK;  // applied at install
  try {
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    reset_gate(c);
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_surrogate_gate_stats(sps_ctx* h, int64_t* steps) {
  if (!h || !steps) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  steps[0] = steps[1] = 0;
  if (!c.surr_cnt) return SPS_OK;
  try {
    sps::SurrGate g;
    SPS_CUDA_CHECK(cudaMemcpyAsync(&g, c.d.surr_gate, sizeof(g), cudaMemcpyDeviceToHost, c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    steps[0] = (int64_t)g.steps_on;
    steps[1] = (int64_t)g.steps_off;
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

int sps_surrogate_stats(sps_ctx* h, int64_t* counts, int32_t reset) {
  if (!h || !counts) return SPS_ERR_ARG;
  sps::Ctx& c = h->c;
  if (!c.surr_cnt) {
    for (int k = 0; k < 4; k++) counts[k] = 0;
    return SPS_OK;
  }
  try {
    unsigned long long v[4];
    SPS_CUDA_CHECK(cudaMemcpyAsync(v, c.surr_cnt, sizeof(v), cudaMemcpyDeviceToHost, c.stream));
    if (reset) SPS_CUDA_CHECK(cudaMemsetAsync(c.surr_cnt, 0, sizeof(v), c.stream));
    SPS_CUDA_CHECK(cudaStreamSynchronize(c.stream));
    for (int k = 0; k < 4; k++) counts[k] = (int64_t)v[k];
  } catch (const std::exception& e) {
    return fail(&c, SPS_ERR_CUDA, e.what());
  }
  return SPS_OK;
}

}  // extern "C"
