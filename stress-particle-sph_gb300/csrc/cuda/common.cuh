// common.cuh -- device-side layout and shared device functions of the SPS step.
//
// Data layout in HBM (one context = a batch of R realisations; a single problem is R = 1):
//   particle ids: the nodes of every realisation, then their stress-points, then their
//     dummies; realisation r owns the contiguous ranges [node0, +nnode), [sp0, +nsp),
//     [dum0, +ndum) of its Real entry, and rid[id] = r.  For R = 1 this is the reference's
//     own order (nodes, stress-points, dummies).
//   particle state, structure of arrays:
//     px,py  vx,vy  s0..s3 (sxx,syy,sxy,szz)  mass rho hsml itype  iv1 fdp  x00x,x00y ...
//   per-step cell sort: cell_of[id], cell_start[c], sorted[s] (id at sorted position s),
//     spos[id]; every realisation has its own grid (the reference's grid of that problem
//     alone) whose cells are numbered from its cell0, so the sorted order is realisation by
//     realisation, cells ascending, particle id ascending within a cell, out-of-domain
//     particles of all realisations last.
//   pair tables per step:
//     half[s*capH + k]  pairs created by the particle at sorted position s (the reference's
//                       grid_find_NEW creation order), 16 B {partner id | pair type << 28,
//                       w, dwdx, dwdy}
//     cross/same lists  entry k of list column lcol[s] at ell(k, col, N2): per target, the
//                       neighbours it meets in the reference's linked-list walk order, 16 B
//                       {u id, w, Gx, Gy} with G the kernel gradient with respect to the
//                       target, entries 2j and 2j+1 side by side in one 32-byte sector;
//                       columns are grouped by target kind (Dev::lcol).
// The FP64 plain kernels reproduce the reference's arithmetic operation by operation
// (compiled with -fmad=false: no multiply-add contraction).
#pragma once
#include <cstdint>

#include "sps.h"

namespace sps {

constexpr int kMaxBC = 16;

struct StepScalars {
  double time_sph;
  double factg;
  double bcval[kMaxBC];
};

// unevaluated sum hi + lo of two FP32 numbers (double-float)
struct dfl {
  float hi, lo;
};

// the grid of one realisation for one step (grid_find_NEW)
struct Grid {
  double xmin[2];
  double deltx[2];
  double rdeltx[2];  // RN(1 / deltx): the cell index divides by the cell size with div_rcp
  int ndiv[2];
  int ncells;    // cells of this realisation
  int cell0;     // global number of its first cell
  int overflow;  // no active particle (no cell size) or the cells exceed the capacity
  float tau;     // width of the FP32 prefilter's guard band (relative to the support^2)
  // every active particle has the same smoothing length h this step: the kernel's
  // h-only subexpressions are formed once (same operations, same values)
  int uniform_h;
  double h, yh, hh, yhh, factor, factor6, c3;
  // the same constants, and the cell size, as double-float pairs (FP32 form)
  dfl df_h, df_yh, df_yhh, df_factor, df_factor6, df_c3, df_cell[2];
};

// totals over the realisations of a step
struct GridTotal {
  int ncells;    // cells of all realisations; the out-of-domain bucket is cell ncells
  int nactive;   // particles in cells (sorted positions below nactive)
  int overflow;  // cells exceeded the capacity
};

// pair bookkeeping of grid_find_NEW's linked list, per realisation
struct PairMeta {
  int64_t n;       // pairs found this step
  int64_t m_prev;  // list nodes before this step (m_pairs)
  int64_t m;       // list nodes after this step
  int64_t base;    // global creation index of the realisation's first pair this step
};

// constants of one realisation (a batch packs problems that share the solver flags but
// not their sizes, material, time step, gravity or domain)
struct Real {
  int node0, nnode, sp0, nsp, dum0, ndum, ndum2;  // id ranges (ndum2: innermost layer)
  int ntype_eco, ncrit, ntype_solid, ic_grav;
  double dt, dx, alpha, beta, damping;
  double D11, D12, D22, D33, D41, D42;
  float D11f, D12f, D22f, D33f, D41f, D42f;  // the same rounded to FP32 (FP32 form's rates)
  double tanfi, coh, young, poiss;
  double alpha2, kc;  // adapt_stress2 constants (FP64)
  float alpha2f, kcf; // the same rounded to FP32 (the FP32 form's inside-the-cone test)
  // drucker_prager's FP32 material constants (tan phi, alpha, k_c, G, K), evaluated once on
  // the host in IEEE FP32 with the routine's expressions (the FP32 form's body reads them)
  float dpf_alpha2, dpf_kc, dpf_G, dpf_K;
  double dt6;  // dt / 6 (RK4's final weight), formed on the host
  double kc_shift;    // kc / (3 alpha2): the apex mean stress of the tension cut
  double xmin_dom[2], xmax_dom[2];
  double cgrav[2];
  // viscoplastic laws (ncrit 1-4): props 7, 8, 10-12, and the material constants that the
  // reference recomputes per call, evaluated once on the host with the same expressions
  double vp_fdatm0, vp_hards, vp_gamma, vp_delta, vp_nflow;
  double vp_snphi;  // sin(phi 0.017453292)
  double vp_den;    // root3 (3 - sin phi): the Drucker-Prager yield denominator
  double vp_cons1;  // yieldf09's cons1 (Mohr-Coulomb sin phi / 3, Drucker-Prager)
  double vp_D[16];  // Get_Dmatx, row-major
  // outside approach: stress-point shift distances and the velocity-vector tolerance
  double r_x, r_y, disp_tol;
};

// device error bit of a tensor-core inference whose wait ran out
constexpr int kErrTensorCore = 1 << 21;

enum ErrBits : int {
  ERR_HALF_CAP = 1,
  ERR_LIST_CAP = 2,
  ERR_CELLS = 4,
  ERR_NPAIRS = 8,
  ERR_BOUND = 16,
};

// The surrogate's gate (sps_surrogate_gate): the network runs in a step only while it
// answers at least min_frac of the step's loading evaluations (a step without any counts as
// below).  After a step below that it
// is off for `period` steps and then runs one step again (a probe); the period doubles, up
// to max_period, while probes keep failing, and returns to 1 after a step that passes.
// Updated on the device at the end of every step, so no host synchronisation is needed.
struct SurrGate {
  int on, wait, period, max_period;
  double min_frac;                          // <= 0: always on
  unsigned long long load0, ans0;           // the counters at the start of the step
  unsigned long long steps_on, steps_off;   // steps with and without the network
};

struct Dev {
  // sizes (all realisations)
  int NN, NT, N2;  // nodes, nodes + stress-points, all particles
  int R;           // realisations
  int capH, capC, capS;
  int cell_cap;
  // solver flags shared by the realisations
  int skf, scale_k, cspm, xsph, update_x, cont_density, sle, sp_sph, inside, no_bcs;
  double cspm_det;    // CSPM determinant threshold of the replaced source copy
  int bc_nodes_only;  // Normal_BCs over the nodes only (code/, strain-localisation copy)
  int bound_from_lists;
  double pi;
  int bcvar[kMaxBC];
  // per-realisation constants and the realisation of every particle; a single problem
  // (R = 1) also carries its entry here, in the kernel parameters (constant bank)
  const Real* real;
  const uint16_t* rid;
  Real real0;
  // particle state (id order)
  double *px, *py, *vx, *vy, *s0, *s1, *s2, *s3;
  double *mass, *rho, *hsml, *iv1, *fdp, *x00x, *x00y, *dispx, *dispy;
  int32_t* itype;
  uint8_t* out;
  int32_t *bc_or_not, *bc_info;
  int32_t* bc_int;
  float *wallpos, *horiz;
  double* grad_u;  // (4, NT): grad_u(a,b) at a + 2b
  // step temporaries
  double *x0x, *x0y, *vx0, *vy0;  // positions and velocities at the start of the step
  double *st0[4], *rho0, *hsml0;  // RK4 initial stress / rho / hsml (stress-points)
  double *RKv[2], *RKs[4], *RKr, *RKh, *RKd;
  double *RHS1[4], *RHS2[2], *RHSr, *RHSh;
  double *fbx, *fby;  // boundary force (nodes), once per step
  // outside approach (stress-points attached to nodes, npoints each, shifted with them)
  int outside, npoints, vel_vector;
  double *x10x, *x10y, *disp10;  // velocity-vector variant: x_10(2,nnode), disp_10(nnode)
  int art_stress;      // artificial_force on (input.txt art_stress)
  int same_entries;    // k_lists writes the same-kind lists' entries only when a step kernel
                      // reads them (XSPH, artificial viscosity or stress) or with keys;
                      // their lengths (degS) always
  double* artR;        // its per-node rotated tensile stresses R(3) of the stage, (3, NN)
  double *vol, *rinv;  // m / rho and 1 / rho per particle (refreshed when rho changes)
  double* A[3];        // sigma_k / (rho * rho) of the stage, per particle
  // FP32 form: packed neighbour records (written by the per-particle kernels)
  int fast;
  // velocities and sigma/rho^2 are double-float pairs (hi = RN32(x), lo = RN32(x - hi)) so
  // that neighbour differences keep FP64-level accuracy
  float4* recV;   // {vx_hi, vy_hi, vx_lo, vy_lo}               all particles
  float4* recS;   // {sxx, syy, sxy, szz}                        nodes + stress-points
  float4* recI;   // {intvar1, m/rho, rho, m}                    all particles
  float4* recA;   // {sxx, syy, sxy}/rho^2 (hi), m               nodes + stress-points
  float4* recAl;  // {sxx, syy, sxy}/rho^2 (lo), 0               nodes + stress-points
  double* Ddev;
  // training capture (sps_capture): one tuple per loading stress-point evaluation
  float* cap_buf;               // (cap_max, 18) floats, or null when not capturing
  unsigned long long* cap_cnt;  // tuples offered since the capture started
  long long cap_max;
  // learned surrogate (sps_surrogate_install), FP32 form only
  int surr;
  const uint2* mlp_frag;  // packed BF16 B fragments of the four layers
  const float* mlp_bias;  // FP32 biases of the four layers
  float env_lo[14], env_hi[14], out_max;
  double surr_tol;
  unsigned long long* surr_cnt;  // loading, answered, outside envelope, drift-rejected
  struct SurrGate* surr_gate;    // whether this step runs the network (sps_surrogate_gate)
  // the network's rows of a stage (tensor-core inference): per stress-point its row or -1,
  // the rows' inputs (16 floats) and outputs (4 floats), and the row count of each stage
  int* cand_row;
  float *xcand, *ycand;
  int* cand_count;
  const void* tc_img;   // the network as the tensor-core kernel's shared-memory image
  const float* tc_bias;
  // cells
  int32_t *cell_of, *cell_cnt, *cell_start, *cell_cursor, *sorted, *spos;
  float *xr, *yr, *hr;
  float *xrl, *yrl;  // FP32 form: low parts of the cell-relative offsets
  float4* srec;       // by sorted position: (xr, yr, hr, 0) of the particle there
  float2* srecl;      // by sorted position, FP32 form: (xrl, yrl)
  Grid* grid;                // per realisation
  GridTotal* gtot;
  unsigned long long* bbox;  // per realisation: ordered keys of minx, miny, -maxx, -maxy, -maxh, minh
  // pairs
  int4* half;
  int32_t* half_cnt;
  int4* half_meta;    // per creator (sorted position): group starts 1-4 (16 bits each),
                      // pair count, id
  int64_t* half_off;  // exclusive scan of half_cnt over sorted positions (size N2+1)
  int4 *cross, *same;
  // FP32 form with gathered lists: the cross lists' {neighbour id, W} again, 8 bytes an
  // entry at k * N2 + col (a warp reads entry k of its columns as one contiguous run): the
  // interpolation reads only these, half the bytes of the full entries
  int2* crossW;
  int use_crossW;
  // per-target lists, entries in pairs: entries 2j and 2j+1 of list column c side by side
  // at (j * N2 + c) * 2 (ell()), one 32-byte sector; keys flat at k * N2 + c
  int32_t *keyC, *keyS;  // per entry: 2 x (position in the reference's walk order) + (target is pair_i)
  int32_t *degC, *degS;  // by list column
  int l2_prefetch;  // FP32 form: bulk L2 prefetch of list entries (bit 0 interp, bit 1 derivs)
  // sorted positions of the stress-point and of the node targets (each in sorted order), so
  // that the gathers run one kind per warp
  int32_t *tgtS, *tgtN, *tflag, *toff;
  // list column of every sorted position: the stress-points first, then the nodes (each in
  // sorted order, as tgtS and tgtN), then the rest.  The k-th target of a one-kind launch
  // has column k (stress-points) or NT - NN + k (nodes), so a warp reads its targets' list
  // entries as one contiguous run per slot.
  int32_t* lcol;
  // get_nodes_on_free_surface: normal (module FP64), subset (1 surface, 2 inside), f_int
  double *nrmx, *nrmy;
  int8_t* subset;
  float* fint;
  float* vol32;  // FP32 form: m / rho per particle for the FP32 free-surface detection
  int ifsigman;
  PairMeta* meta;  // per realisation
  // scalars of the current step, per realisation (table: [step][realisation])
  const StepScalars* scal_table;
  int* step_idx;
  StepScalars* cur;
  int* err;
  // scan scratch
  int64_t* scan_tmp;
};

// Index of entry k of list column col in the per-target lists (cross, same).  Entries 2j and
// 2j+1 of a column share one 32-byte sector, so that the list build, which appends a
// target's entries one by one, writes whole sectors; the columns of consecutive targets
// stay adjacent, so a warp reading entry k of its targets still reads one contiguous run.
__device__ __forceinline__ size_t ell(int k, int col, int N2) {
  return (((size_t)(k >> 1) * (size_t)N2 + (size_t)col) << 1) | (size_t)(k & 1);
}

// Bulk L2 prefetch of the list entries of a warp's targets (one-kind launches, whose active
// lanes hold consecutive list columns).  For each entry pair j from 1 to the warp's largest
// degree, the 32-byte sectors of the warp's columns are one contiguous run (ell()), which
// the warp's first active lane requests with one cp.async.bulk.prefetch.L2: the entries
// stream from DRAM ahead of the dependent record gathers.  A hint: no result depends on it.
__device__ __forceinline__ void prefetch_list_l2(const int4* list, int col, int deg, int N2) {
  const unsigned act = __activemask();
  const int maxdeg = (int)__reduce_max_sync(act, (unsigned)deg);
  const int col0 = (int)__reduce_min_sync(act, (unsigned)col);
  const int col1 = (int)__reduce_max_sync(act, (unsigned)col);
  if ((int)(threadIdx.x & 31) == __ffs(act) - 1) {
    const uint32_t bytes = (uint32_t)(col1 - col0 + 1) * 32u;
    for (int j = 1; 2 * j < maxdeg; j++) {
      const int4* p = list + ell(2 * j, col0, N2);
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
    }
  }
}

// an ordered key of a non-NaN double on the integer pipe: the bit pattern with the
// magnitude bits of a negative value flipped, -0 taken as +0 (a < b exactly when
// f64_key(a) < f64_key(b))
__device__ __forceinline__ long long f64_key(double a) {
  long long ia = __double_as_longlong(a);
  if ((ia << 1) == 0) ia = 0;
  return ia ^ ((ia >> 63) & 0x7FFFFFFFFFFFFFFFll);
}
__device__ __forceinline__ bool f64_isnan(double a) {
  return (__double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFll) > 0x7FF0000000000000ll;
}
// a >= b for non-NaN doubles, on the integer pipe
__device__ __forceinline__ bool f64_ge(double a, double b) { return f64_key(a) >= f64_key(b); }

// Correctly rounded a / b given y = RN(1/b), by Markstein's theorem (P. Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990; see also Muller et al., Handbook of Floating-Point Arithmetic, the theorem on
// FMA-based division): when y is within 1/2 ulp of 1/b and q within 1 ulp of a/b, the
// corrected q' = RN(q + y * (a - b q)) equals RN(a/b).  q = RN(a y) can be up to 1.5 ulp
// off, so one correction step brings it within 1 ulp and a second one rounds correctly.
// Valid for normal operands without overflow or underflow (masses, densities and kernel
// values here); a zero numerator returns a signed zero.  Bit-for-bit agreement with the
// IEEE division is checked on the GPU by sps_selftest.
__device__ __forceinline__ double div_rcp(double a, double b, double y) {
  if ((__double_as_longlong(a) << 1) == 0) return a * y;  // a zero, tested on the integer pipe
  double q = a * y;
  double r = fma(-b, q, a);
  q = fma(r, y, q);
  r = fma(-b, q, a);
  return fma(r, y, q);
}

// ---- FP64 <-> FP32 conversions on the integer pipe --------------------------------------
// GB300 issues double/float conversions on its FP64 pipe (2 per SM per clock); the FP32
// form converts every record it writes, so these do the same roundings with 32-bit integer
// operations on the bit patterns.  Values outside the range handled (zero, float
// subnormals, overflow, Inf/NaN) take the hardware conversion.

// The rare cases take the hardware conversions out of line: inlined, the compiler may
// evaluate both sides of the branch and keep the FP64 pipe busy with a conversion whose
// result is then discarded.  Zeros, which are common, are handled on the integer pipe.
static __device__ __noinline__ float f32_rn_hw(double x) { return (float)x; }
static __device__ __noinline__ double f64_of_hw(float f) { return (double)f; }
static __device__ __noinline__ float2 f32_split_hw(double x) {
  const float hi = (float)x;
  return make_float2(hi, (float)(x - (double)hi));
}

// RN-even double -> float, identical to (float)x
__device__ __forceinline__ float f32_rn(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned h32 = (unsigned)(u >> 32), l32 = (unsigned)u;
  const int E = (int)((h32 >> 20) & 0x7FFu);
  if (E < 897 || E > 1150) {
    if ((u << 1) == 0ull) return __uint_as_float(h32 & 0x80000000u);  // +-0
    return f32_rn_hw(x);
  }
  const unsigned f23 = ((h32 & 0xFFFFFu) << 3) | (l32 >> 29);
  const unsigned rem = l32 & 0x1FFFFFFFu;
  const unsigned up = (rem > 0x10000000u) || (rem == 0x10000000u && (f23 & 1u));
  return __uint_as_float(((h32 & 0x80000000u) | ((unsigned)(E - 896) << 23) | f23) + up);
}

// (float)r for |r| < 2^30, round to nearest even, on the integer pipe (GB300 issues the
// hardware int -> float conversion on its FP64 pipe): the leading bit found with clz, the
// bits below the 24 kept rounded by their remainder
__device__ __forceinline__ float i2f_rn(int r) {
  if (r == 0) return 0.0f;
  const unsigned sgn = r < 0 ? 0x80000000u : 0u;
  const unsigned a = r < 0 ? 0u - (unsigned)r : (unsigned)r;
  const int e = 31 - __clz((int)a);  // the leading bit, 0 .. 29
  unsigned m;
  if (e <= 23) {
    m = a << (23 - e);
  } else {
    const int sh = e - 23;
    m = a >> sh;
    const unsigned rem = a & ((1u << sh) - 1u), half = 1u << (sh - 1);
    m += (rem > half || (rem == half && (m & 1u))) ? 1u : 0u;  // may carry into bit 24
  }
  // a carry to 2^24 moves into the exponent field by the addition
  return __uint_as_float(sgn | ((unsigned)(e + 127) << 23) + (m - 0x800000u));
}

// hi = (float)x, lo = (float)(x - (double)hi): the exact remainder x - hi is the dropped
// significand bits (minus one float ulp when hi was rounded up), scaled by 2^(E-1075)
__device__ __forceinline__ void f32_split(double x, float& hi, float& lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned h32 = (unsigned)(u >> 32), l32 = (unsigned)u;
  const int E = (int)((h32 >> 20) & 0x7FFu);
  if (E < 949 || E > 1150) {
    if ((u << 1) == 0ull) {  // +-0: hi keeps the sign, x - hi = +0
      hi = __uint_as_float(h32 & 0x80000000u);
      lo = 0.0f;
      return;
    }
    const float2 v = f32_split_hw(x);  // returned by value: no local escapes to memory
    hi = v.x;
    lo = v.y;
    return;
  }
  const unsigned f23 = ((h32 & 0xFFFFFu) << 3) | (l32 >> 29);
  const unsigned rem = l32 & 0x1FFFFFFFu;
  const unsigned up = (rem > 0x10000000u) || (rem == 0x10000000u && (f23 & 1u));
  hi = __uint_as_float(((h32 & 0x80000000u) | ((unsigned)(E - 896) << 23) | f23) + up);
  int r = (int)rem - (up ? 0x20000000 : 0);
  if (h32 & 0x80000000u) r = -r;
  lo = i2f_rn(r) * __uint_as_float((unsigned)(E - 948) << 23);
}

// exact float -> double, identical to (double)f
__device__ __forceinline__ double f64_of(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu;
  if (e == 0u || e == 255u) {
    if ((b << 1) == 0u)  // +-0
      return __longlong_as_double((long long)((unsigned long long)(b & 0x80000000u) << 32));
    return f64_of_hw(f);
  }
  const unsigned h32 = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
  const unsigned l32 = b << 29;
  return __longlong_as_double((long long)(((unsigned long long)h32 << 32) | l32));
}

// (float)(a / b) of the IEEE double quotient, given y = RN(1/b), with one FP64 multiply in
// almost every case.  q = RN(a y) is within 3 double ulps of RN(a / b) (y and the product
// each add at most half an ulp of relative error).  When the 29 significand bits that the
// float rounding drops are at least 8 away from the float rounding boundaries (0, the
// half-way point, 2^29: the low 28 of them in [8, 2^28 - 8]), every double within 3 ulps of q
// has the same exponent and rounds to the same float, so f32_rn(q) is the answer.
// Otherwise (about one case in 2^24), and outside f32_rn's exponent range (zero included),
// the correctly rounded quotient div_rcp(a, b, y) is rounded instead.  Checked against the
// IEEE division bit for bit by sps_selftest_division.
static __device__ __noinline__ float div_rcp_f32_slow(double a, double b, double y) {
  return f32_rn(div_rcp(a, b, y));
}
__device__ __forceinline__ float div_rcp_f32(double a, double b, double y) {
  const double q = a * y;
  const unsigned long long u = (unsigned long long)__double_as_longlong(q);
  const int E = (int)((u >> 52) & 0x7FFu);
  const unsigned m28 = (unsigned)u & 0x0FFFFFFFu;
  if (E >= 897 && E <= 1150 && (m28 - 8u) <= 0x0FFFFFF0u) return f32_rn(q);
  return div_rcp_f32_slow(a, b, y);
}

// ----------------------------------------------------------------------------------------
// kernel (example_problems/soil_failure_bui_et_al_2008/2_SPH_main_2018.f90:1440-1538).
// FP64 with the FP32 literal 2./3. (:1480); x**n expanded into multiplications.
__device__ __forceinline__ void sph_kernel(int skf, double pi, double r, double dx0, double dx1,
                                           double hsml, double* w, double* dw0, double* dw1) {
  double q = r / hsml;
  *w = 0.0;
  *dw0 = 0.0;
  *dw1 = 0.0;
  if (skf == 1) {
    double factor = 15.0 / (7.0 * pi * hsml * hsml);
    if (q >= 0 && q <= 1.0) {
      const double two_thirds = (double)(2.0f / 3.0f);
      *w = factor * ((two_thirds - q * q) + (q * q * q) / 2.0);
      double a = (factor * (-2.0 + 1.5 * q)) / (hsml * hsml);
      *dw0 = a * dx0;
      *dw1 = a * dx1;
    } else if (q > 1.0 && q <= 2.0) {
      double t = 2.0 - q;
      *w = (factor / 6.0) * ((t * t) * t);
      double a = (((factor / 6.0) * 3.0) * (t * t)) / hsml;
      *dw0 = -(a * (dx0 / r));
      *dw1 = -(a * (dx1 / r));
    }
  } else if (skf == 2) {
    double factor = 1.0 / ((hsml * hsml) * pi);
    if (q >= 0 && q <= 3.0) {
      *w = factor * exp(-(q * q));
      *dw0 = *w * (((-2.0 * dx0) / hsml) / hsml);
      *dw1 = *w * (((-2.0 * dx1) / hsml) / hsml);
    }
  } else if (skf == 3) {
    double factor = 7.0 / (478.0 * pi * hsml * hsml);
    double a = 3.0 - q, b = 2.0 - q, c1 = 1.0 - q;
    double a2 = a * a, b2 = b * b, c2 = c1 * c1;
    double a4 = a2 * a2, b4 = b2 * b2;
    double a5 = (a2 * a) * a2, b5 = (b2 * b) * b2, c5 = (c2 * c1) * c2;
    if (q >= 0 && q <= 1.0) {
      *w = factor * ((a5 - 6.0 * b5) + 15.0 * c5);
      double g = ((-120.0 + 120.0 * q) - 50.0 * (q * q)) / (hsml * hsml);
      *dw0 = factor * (g * dx0);
      *dw1 = factor * (g * dx1);
    } else if (q > 1.0 && q <= 2.0) {
      *w = factor * (a5 - 6.0 * b5);
      double g = (factor * (-5.0 * a4 + 30.0 * b4)) / hsml;
      *dw0 = g * (dx0 / r);
      *dw1 = g * (dx1 / r);
    } else if (q > 2.0 && q <= 3.0) {
      *w = factor * a5;
      double g = (factor * (-5.0 * a4)) / hsml;
      *dw0 = g * (dx0 / r);
      *dw1 = g * (dx1 / r);
    }
  }
}

// cubic kernel for a uniform smoothing length: identical results to sph_kernel(1, ...)
// with the h-only subexpressions taken from g and the divisions by h, h*h and r done by
// div_rcp with their exact reciprocals
__device__ __forceinline__ void cubic_uniform(const Grid& g, double r, double dx0, double dx1,
                                              double* w, double* dw0, double* dw1) {
  double q = div_rcp(r, g.h, g.yh);
  *w = 0.0;
  *dw0 = 0.0;
  *dw1 = 0.0;
  // the branch tests on the integer pipe (ordered keys; q is a non-negative quotient or NaN,
  // which takes neither branch)
  const long long kq = f64_key(q);
  const bool qnan = f64_isnan(q);
  if (!qnan && kq >= 0 && kq <= f64_key(1.0)) {
    const double two_thirds = (double)(2.0f / 3.0f);
    *w = g.factor * ((two_thirds - q * q) + (q * q * q) * 0.5);  // / 2.0, exactly
    double a = div_rcp(g.factor * (-2.0 + 1.5 * q), g.hh, g.yhh);
    *dw0 = a * dx0;
    *dw1 = a * dx1;
  } else if (!qnan && kq > f64_key(1.0) && kq <= f64_key(2.0)) {
    double t = 2.0 - q;
    *w = g.factor6 * ((t * t) * t);
    double a = div_rcp(g.c3 * (t * t), g.h, g.yh);
    double yr = __drcp_rn(r);  // RN(1 / r), the correctly rounded reciprocal
    *dw0 = -(a * div_rcp(dx0, r, yr));
    *dw1 = -(a * div_rcp(dx1, r, yr));
  }
}

// adapt_stress2 body (3_SPH_material_2018.f90:2087-2161), FP64
static __device__ __noinline__ void adapt_stress_full(double alpha2, double kc, double& a,
                                                      double& b, double& c, double& d);
// Inside the cone, clearly: yield >= 0 and yield^2 >= varj2 (1 + 2^-49) imply
// yield >= RN(sqrt(varj2)) whatever the roundings of the two products (each within 2^-53),
// so adapt_stress2 leaves the stress as it is and neither its square root nor its tension
// cut (both out of line, below) need to run.  Bit-identical to the full routine.
__device__ __forceinline__ void adapt_stress(double alpha2, double kc, double& a, double& b,
                                             double& c, double& d) {
  const double smean = ((a + b) + d) / 3.0;
  const double d0 = a - smean, d1 = b - smean, d2 = c, d3 = d - smean;
  const double varj2 = d2 * d2 + 0.5 * ((d0 * d0 + d1 * d1) + d3 * d3);
  const double yield = -((alpha2 * 3.0) * smean) + kc;
  if (yield > 1e-100 && yield < 1e100 && yield * yield >= varj2 * (1.0 + 0x1.0p-49)) return;
  adapt_stress_full(alpha2, kc, a, b, c, d);
}
// adapt_stress2 (3_SPH_material_2018.f90:2087-2161) in the reference's FP64 arithmetic
static __device__ __noinline__ void adapt_stress_full(double alpha2, double kc, double& a,
                                                      double& b, double& c, double& d) {
  double smean = ((a + b) + d) / 3.0;
  double d0 = a - smean, d1 = b - smean, d2 = c, d3 = d - smean;
  double varj2 = d2 * d2 + 0.5 * ((d0 * d0 + d1 * d1) + d3 * d3);
  double yield = -((alpha2 * 3.0) * smean) + kc;
  if (yield < 0) {
    double shift = kc / (3.0 * alpha2);
    a = (a - smean) + shift;
    b = (b - smean) + shift;
    d = (d - smean) + shift;
    smean = ((a + b) + d) / 3.0;
    d0 = a - smean;
    d1 = b - smean;
    d2 = c;
    d3 = d - smean;
    varj2 = d2 * d2 + 0.5 * ((d0 * d0 + d1 * d1) + d3 * d3);
    yield = -((alpha2 * 3.0) * smean) + kc;
  }
  double sj = sqrt(varj2);
  if (yield < sj) {
    double rn = (-((3.0 * alpha2) * smean) + kc) / sj;
    if (sj <= (double)1e-5f) rn = 0.0;
    a = rn * d0 + smean;
    b = rn * d1 + smean;
    d = rn * d3 + smean;
    c = rn * d2;
  }
}

// FP32 value of x with the significand truncated (relative error below 2^-23), on the
// integer pipe; NaN outside the normal FP32 range (zero excepted), which fails every test
// that uses it
__device__ __forceinline__ float f32_trunc(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned h32 = (unsigned)(u >> 32), l32 = (unsigned)u;
  const int E = (int)((h32 >> 20) & 0x7FFu);
  if (E < 897 || E > 1150) return (u << 1) == 0ull ? 0.0f : __uint_as_float(0x7FC00000u);
  return __uint_as_float((h32 & 0x80000000u) | ((unsigned)(E - 896) << 23) |
                         ((h32 & 0xFFFFFu) << 3) | (l32 >> 29));
}

// True when the stress (a, b, c, d) lies inside the Drucker-Prager cone with a margin that
// covers every rounding of this FP32 evaluation: then yield >= 0 and yield^2 >= J2 hold in
// exact arithmetic with a relative margin far above the FP64 test's roundings, so the FP64
// return below leaves the stress unchanged and may be skipped (the result is bit-identical).
// Error bounds, u = 2^-24, M = max |component|: the truncated inputs carry 2u M; the mean
// 16u M; each deviator component 24u M (|d| <= 2.1 M); J2 = d2^2 + (d0^2 + d1^2 + d3^2)/2
// therefore 256u M^2; yield = kc - 3 alpha smean 4u kc + 64u alpha M.  These bounds are
// relative to M and hold while no FP32 square underflows or overflows, so the test also
// requires 1e-15 <= M <= 1e15 (then 256u M^2 stays far above the FP32 subnormal range and
// every absolute error that an underflowing term carries is far below it).  Anything
// outside these ranges fails the test and takes the FP64 path.
__device__ __forceinline__ bool inside_cone_f32(float alpha2, float kc, double a, double b,
                                                double c, double d) {
  const float af = f32_trunc(a), bf = f32_trunc(b), cf = f32_trunc(c), df = f32_trunc(d);
  const float m = fmaxf(fmaxf(fabsf(af), fabsf(bf)), fmaxf(fabsf(cf), fabsf(df)));
  const float u = 5.9604645e-08f;  // 2^-24
  const float smean = ((af + bf) + df) * (1.0f / 3.0f);
  const float d0 = af - smean, d1 = bf - smean, d3 = df - smean;
  const float j2 = fmaf(cf, cf, 0.5f * fmaf(d0, d0, fmaf(d1, d1, d3 * d3)));
  const float yl = (kc - (3.0f * alpha2) * smean) - (4.0f * u * kc + 64.0f * u * alpha2 * m);
  const float ej = 256.0f * u * (m * m);
  return m >= 1e-15f && m <= 1e15f && yl > 0.0f && yl * yl > (j2 + ej) * (1.0f + 16.0f * u);
}

// The same return for the FP32 form, without FP64 divisions or square roots in the common
// path (GB300 issues FP64 at a small fraction of its FP32 rate): the mean by a product with
// 1/3, the test yield < sqrt(J2) as yield^2 < J2 (yield >= 0), and for the stress-points
// actually returned 1/sqrt(J2) from an FP32 seed refined by two Newton steps in FP64
// (relative error ~1e-16).  Explicit fma() keeps the FMA where the unit disables it.
static __device__ __noinline__ void adapt_stress_fast_return(double alpha2, double kc,
                                                             double shift, double& a,
                                                             double& b, double& c, double& d);
__device__ __forceinline__ void adapt_stress_fast(double alpha2, double kc, double shift,
                                                  double& a, double& b, double& c, double& d) {
  const double third = 1.0 / 3.0;
  const double smean = ((a + b) + d) * third;
  const double d0 = a - smean, d1 = b - smean, d2 = c, d3 = d - smean;
  const double varj2 = fma(d2, d2, 0.5 * fma(d0, d0, fma(d1, d1, d3 * d3)));
  const double yield = fma(-3.0 * alpha2, smean, kc);
  // the returned points (few: the loading ones) take the return out of line
  if (yield < 0 || yield * yield < varj2) adapt_stress_fast_return(alpha2, kc, shift, a, b, c, d);
}
static __device__ __noinline__ void adapt_stress_fast_return(double alpha2, double kc,
                                                             double shift, double& a,
                                                             double& b, double& c, double& d) {
  const double third = 1.0 / 3.0;
  double smean = ((a + b) + d) * third;
  double d0 = a - smean, d1 = b - smean, d2 = c, d3 = d - smean;
  double varj2 = fma(d2, d2, 0.5 * fma(d0, d0, fma(d1, d1, d3 * d3)));
  double yield = fma(-3.0 * alpha2, smean, kc);
  if (yield < 0) {
    a = (a - smean) + shift;
    b = (b - smean) + shift;
    d = (d - smean) + shift;
    smean = ((a + b) + d) * third;
    d0 = a - smean;
    d1 = b - smean;
    d2 = c;
    d3 = d - smean;
    varj2 = fma(d2, d2, 0.5 * fma(d0, d0, fma(d1, d1, d3 * d3)));
    yield = fma(-3.0 * alpha2, smean, kc);
  }
  if (yield < 0 || yield * yield < varj2) {
    double rn = 0.0;
    if (varj2 > (double)1e-5f * (double)1e-5f) {
      double rs = (double)rsqrtf((float)varj2);
      rs = rs * fma(-0.5 * varj2 * rs, rs, 1.5);
      rs = rs * fma(-0.5 * varj2 * rs, rs, 1.5);
      rn = yield * rs;
    }
    a = fma(rn, d0, smean);
    b = fma(rn, d1, smean);
    d = fma(rn, d3, smean);
    c = rn * d2;
  }
}

// The viscoplastic laws of plastic_terms for ncrit <= 4 (3_SPH_material_2018.f90): Get_Vivel
// :2165, invar09 :2233, yieldf09 :2381, flowvp09 :2560, then Gs = -Dmatx vivel (:1930-1934).
// 2D branches, FP64 with the reference's FP32 constants (root3 = sqrt(3.00) in FP32,
// 0.01 and 0.1 as FP32 values).  Lode-angle functions are evaluated only for the laws that
// read them (Tresca, Mohr-Coulomb); von Mises and Drucker-Prager never use them.  Perzyna
// exponent n = 1 with delta = 1 takes fnorm itself (the reference's fnorm**1.0).
// s: stress (plane-stress szz substituted), iv1: accumulated deviatoric plastic strain.
__device__ __forceinline__ void viscoplastic(const Real& M, const double* s, double iv1,
                                             double* vivel, double* Gs) {
  const double root3 = (double)sqrtf(3.0f);
  for (int i = 0; i < 4; i++) vivel[i] = 0.0;
  // invar09
  const double smean = ((s[0] + s[1]) + s[3]) / 3.0;
  double dv[4] = {s[0] - smean, s[1] - smean, s[2], s[3] - smean};
  const double varj2 = dv[2] * dv[2] + 0.5 * ((dv[0] * dv[0] + dv[1] * dv[1]) + dv[3] * dv[3]);
  const double steff = sqrt(varj2);
  const bool lode = M.ncrit == 1 || M.ncrit == 3;
  double theta = 0.0;
  if (lode) {
    const double varj3 = dv[3] * (dv[3] * dv[3] - varj2);
    double sint3;
    if (steff != 0.0) {
      sint3 = -(((3.0 * root3) * varj3) / ((2.0 * varj2) * steff));
      if (sint3 > 1.0) sint3 = 1.0;
    } else {
      sint3 = 0.0;
    }
    if (sint3 < -1.0) sint3 = -1.0;
    if (sint3 > 1.0) sint3 = 1.0;
    theta = asin(sint3) / 3.0;
  }
  double yield;
  if (M.ncrit == 1) yield = (2.0 * cos(theta)) * steff;
  else if (M.ncrit == 2) yield = root3 * steff;
  else if (M.ncrit == 3)
    yield = smean * M.vp_snphi + steff * (cos(theta) - (sin(theta) * M.vp_snphi) / root3);
  else yield = ((6.0 * smean) * M.vp_snphi) / M.vp_den + steff;
  double fdatm = M.vp_fdatm0 + M.vp_hards * iv1;
  double fact = fabs(fdatm) / fabs(M.vp_fdatm0);
  if (fact < (double)0.1f) fact = (double)0.1f;
  fdatm = M.vp_fdatm0 * fact;
  if (yield > fdatm) {
    // flowvp09
    const double fnorm = (yield - fdatm) / fdatm;
    if (fnorm >= (double)0.01f) {
      double cmult;
      if (M.vp_nflow != 1.0) cmult = M.vp_gamma * (exp(M.vp_delta * fnorm) - 1.0);
      else cmult = M.vp_gamma * (M.vp_delta == 1.0 ? fnorm : pow(fnorm, M.vp_delta));
      // yieldf09
      double va2[4] = {0.0, 0.0, 0.0, 0.0};
      if (steff > 0) {
        for (int i = 0; i < 4; i++) va2[i] = dv[i] / (2.0 * steff);
        va2[2] = dv[2] / steff;
      }
      double cons1 = 0.0, cons2, cons3 = 0.0;
      const double va3[4] = {dv[1] * dv[3] + varj2 / 3.0, dv[0] * dv[3] + varj2 / 3.0,
                             -((2.0 * dv[2]) * dv[3]), (dv[0] * dv[1] - dv[2] * dv[2]) + varj2 / 3.0};
      if (lode) {
        const double tanth = tan(theta), tant3 = tan(3.0 * theta), sinth = sin(theta),
                     costh = cos(theta), cost3 = cos(3.0 * theta);
        const double abthe = fabs(theta * (double)57.29577951308f);
        if (M.ncrit == 1) {
          if (abthe >= 29.0) {
            cons2 = root3;
          } else {
            cons2 = 2.0 * (costh + sinth * tant3);
            cons3 = (root3 * sinth) / (varj2 * cost3);
          }
        } else {
          cons1 = M.vp_cons1;
          if (abthe >= 29.0) {
            const double plumi = theta > 0.0 ? -1.0 : 1.0;
            cons2 = 0.5 * (root3 + (plumi * cons1) * root3);
          } else {
            cons2 = costh * ((1.0 + tanth * tant3) + (cons1 * (tant3 - tanth)) * root3);
            cons3 = (root3 * sinth + (3.0 * cons1) * costh) / ((2.0 * varj2) * cost3);
          }
        }
      } else if (M.ncrit == 2) {
        cons2 = root3;
      } else {
        cons1 = M.vp_cons1;
        cons2 = 1.0;
      }
      const double va1[4] = {1.0, 1.0, 0.0, 1.0};
      for (int i = 0; i < 4; i++)
        vivel[i] = cmult * ((cons1 * va1[i] + cons2 * va2[i]) + cons3 * va3[i]);
    }
  }
  for (int i = 0; i < 4; i++) {
    double g = 0.0;
    for (int j = 0; j < 4; j++) g = g - M.vp_D[4 * i + j] * vivel[j];
    Gs[i] = g;
  }
}

// drucker_prager (3_SPH_material_2018.f90:1958-2083): FP32 body.  s: stress (plane-stress
// szz already substituted), gu: grad_u(2,2).  Updates *fdp, returns G and vivel.  (The FP32
// form uses drucker_prager_f32.)
__device__ __forceinline__ void drucker_prager(const Real& M, double time_sph, const double* s,
                                               const double* gu, double* fdp, double* G,
                                               double* vivel) {
  double f0 = *fdp;
  auto tof = [](double v) { return (float)v; };
  auto tod = [](float v) { return (double)v; };
  float tanfi = tof(M.tanfi), coh = tof(M.coh), young = tof(M.young), poiss = tof(M.poiss);
  float smean = (float)(((s[0] + s[1]) + s[3]) / 3.0);
  const double smd = tod(smean);
  float dv0 = tof(s[0] - smd);
  float dv1 = tof(s[1] - smd);
  float dv2 = tof(s[2]);
  float dv3 = tof(s[3] - smd);
  float varj2 = dv2 * dv2 + 0.5f * ((dv0 * dv0 + dv1 * dv1) + dv3 * dv3);
  float vari1 = 3.0f * smean;
  float eps11 = tof(gu[0]);
  float eps12 = tof(0.5 * (gu[2] + gu[1]));
  float eps22 = tof(gu[3]);
  float emean = eps11 + eps22;
  float den = sqrtf(9.0f + 12.0f * (tanfi * tanfi));
  float alpha2 = tanfi / den;
  float kc = (3.0f * coh) / den;
  float yield = -(alpha2 * vari1) + kc;
  float sj = sqrtf(varj2);
  *fdp = tod(sj - yield);
  float f1 = sj - yield;  // (float)(double)x == x
  double df = tod(f1) - f0;
  float G_mod = young / (2.0f * (1.0f + poiss));
  float K_mod = young / (3.0f * (1.0f - 2.0f * poiss));
  float s_eps = (dv0 * eps11 + (2.0f * dv2) * eps12) + dv1 * eps22;
  if (time_sph > 0 && f1 >= 0 && df >= 0 && sj >= 1e-5f) {
    float gs = G_mod / sj;
    float lambda_1 = ((3.0f * alpha2) * K_mod) * emean;
    float lambda_2 = gs * s_eps;
    float G2 = (lambda_1 + lambda_2) / G_mod;
    G[0] = tod((gs * dv0) * G2);
    G[1] = tod((gs * dv1) * G2);
    G[2] = tod((gs * dv2) * G2);
    G[3] = tod((gs * dv3) * G2);
    const float sixth = 1.0f / 6.0f;
    float rs = 1.0f / sj;
    double g2 = tod(G2);
    vivel[0] = tod((sixth * rs) * ((2.0f * dv0 - dv1) - dv3)) * g2;
    vivel[1] = tod((sixth * rs) * ((2.0f * dv1 - dv0) - dv3)) * g2;
    vivel[2] = tod(rs * dv2) * g2;
    vivel[3] = tod((sixth * rs) * ((2.0f * dv3 - dv0) - dv1)) * g2;
  } else {
    G[0] = G[1] = G[2] = G[3] = 0.0;
    vivel[0] = vivel[1] = vivel[2] = vivel[3] = 0.0;
  }
}

// exact a + b = s + e (Knuth's TwoSum: additions only, so nothing is contracted)
__device__ __forceinline__ float two_sum_f(float a, float b, float& e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}


// drucker_prager for the FP32 form, without FP64 arithmetic (GB300 issues FP64 at 1/64 of
// its FP32 rate): the stresses enter as hi + lo splits, the mean is formed in double-float
// and the deviator from it, so each deviatoric component keeps FP32 accuracy relative to
// itself; the loading test df >= 0 compares the FP64 values exactly on the integer pipe; the
// material constants are the host's FP32 evaluation (dpf_*).  Same outputs as
// drucker_prager: the updated f, the plastic source G and vivel.
// the body, with its outputs as the FP32 values they are (G, vivel); returns whether the
// point is loading (G non-zero)
__device__ __forceinline__ bool drucker_prager_f32v(const Real& M, double time_sph,
                                                    const double* s, const double* gu,
                                                    double* fdp, float* G, float* vivel) {
  const double f0 = *fdp;
  float s0h, s0l, s1h, s1l, s3h, s3l;
  f32_split(s[0], s0h, s0l);
  f32_split(s[1], s1h, s1l);
  f32_split(s[3], s3h, s3l);
  float e1, e2;
  const float t1 = two_sum_f(s0h, s1h, e1);
  const float th = two_sum_f(t1, s3h, e2);
  const float tl = ((e1 + e2) + (s0l + s1l)) + s3l;
  const float mh = __fdiv_rn(th, 3.0f);
  const float ml = __fmul_rn(__fadd_rn(fmaf(-3.0f, mh, th), tl), 1.0f / 3.0f);
  const float smean = mh + ml;
  const float dv0 = (s0h - mh) + (s0l - ml);
  const float dv1 = (s1h - mh) + (s1l - ml);
  const float dv3 = (s3h - mh) + (s3l - ml);
  const float dv2 = f32_rn(s[2]);
  const float varj2 = fmaf(dv2, dv2, 0.5f * fmaf(dv0, dv0, fmaf(dv1, dv1, dv3 * dv3)));
  const float vari1 = 3.0f * smean;
  const float eps11 = f32_rn(gu[0]);
  const float eps12 = 0.5f * (f32_rn(gu[2]) + f32_rn(gu[1]));
  const float eps22 = f32_rn(gu[3]);
  const float emean = eps11 + eps22;
  const float alpha2 = M.dpf_alpha2, kc = M.dpf_kc;
  const float yield = kc - alpha2 * vari1;
  const float sj = sqrtf(varj2);
  const float f1 = sj - yield;
  *fdp = f64_of(f1);
  const float s_eps = fmaf(dv0, eps11, fmaf(2.0f * dv2, eps12, dv1 * eps22));
  if (__double_as_longlong(time_sph) > 0 && f1 >= 0.0f && f64_ge(f64_of(f1), f0) &&
      sj >= 1e-5f) {
    const float G_mod = M.dpf_G, K_mod = M.dpf_K;
    const float gs = __fdiv_rn(G_mod, sj);
    const float lambda_1 = ((3.0f * alpha2) * K_mod) * emean;
    const float G2 = __fdiv_rn(fmaf(gs, s_eps, lambda_1), G_mod);
    G[0] = (gs * dv0) * G2;
    G[1] = (gs * dv1) * G2;
    G[2] = (gs * dv2) * G2;
    G[3] = (gs * dv3) * G2;
    const float rs = __frcp_rn(sj), r6 = rs * (1.0f / 6.0f);
    vivel[0] = (r6 * ((2.0f * dv0 - dv1) - dv3)) * G2;
    vivel[1] = (r6 * ((2.0f * dv1 - dv0) - dv3)) * G2;
    vivel[2] = (rs * dv2) * G2;
    vivel[3] = (r6 * ((2.0f * dv3 - dv0) - dv1)) * G2;
    return G[0] != 0.0f || G[1] != 0.0f || G[2] != 0.0f || G[3] != 0.0f;
  }
  G[0] = G[1] = G[2] = G[3] = 0.0f;
  vivel[0] = vivel[1] = vivel[2] = vivel[3] = 0.0f;
  return false;
}

// the same with FP64 outputs (exact conversions of the FP32 values)
__device__ __forceinline__ void drucker_prager_f32(const Real& M, double time_sph,
                                                   const double* s, const double* gu,
                                                   double* fdp, double* G, double* vivel) {
  float Gf[4], vf[4];
  drucker_prager_f32v(M, time_sph, s, gu, fdp, Gf, vf);
  for (int k = 0; k < 4; k++) {
    G[k] = f64_of(Gf[k]);
    vivel[k] = f64_of(vf[k]);
  }
}

__device__ __forceinline__ const Real& real_of(const Dev& D, int i) {
  return D.R == 1 ? D.real0 : D.real[D.rid[i]];
}
// the node at the same place as a stress-point (and back), when every node has one
__device__ __forceinline__ int node_of_sp(const Real& M, int t) { return M.node0 + (t - M.sp0); }
__device__ __forceinline__ int sp_of_node(const Real& M, int n) { return M.sp0 + (n - M.node0); }

// list column (Dev::lcol) of the k-th target of a launch: KIND 1 over tgtS, 2 over tgtN,
// 0 over every sorted position s
template <int KIND>
__device__ __forceinline__ int list_col(const Dev& D, int k, int s) {
  return KIND == 1 ? k : KIND == 2 ? (D.NT - D.NN) + k : D.lcol[s];
}

__device__ __forceinline__ bool is_sp(int t) { return t == 1; }
__device__ __forceinline__ bool is_node(int t) { return t == 2; }
__device__ __forceinline__ bool is_dummy(int t) { return t == 25; }

// pair type of Pint_Update (3_SPH_material_2018.f90:1617-1627) from the itype sum
__device__ __forceinline__ int pint_type(int ti, int tj) {
  int s = ti + tj;
  return s == 3 ? 1 : s == 2 ? 2 : s == 4 ? 3 : s == 27 ? 6 : s == 26 ? 9 : 0;
}

}  // namespace sps

// launchers implemented in the .cu units
namespace sps {
struct Ctx;
int launch_pair_build(Ctx& c);
int launch_plain_step(Ctx& c);
int launch_fast_step(Ctx& c);
void launch_vol(Ctx& c, int lo, int hi);
void launch_finterp(Ctx& c);
void launch_fderivs(Ctx& c, int stage);
void launch_fsp_tail(Ctx& c, int stage);
void launch_surface(Ctx& c);
void launch_surface_f32(Ctx& c);
void launch_lists_keys(Ctx& c);
void launch_lists_same(Ctx& c);
void ensure_half_lists(Ctx& c);
void launch_fxsph(Ctx& c);
void launch_selftest_div(Ctx& c, int64_t n, uint64_t seed, unsigned long long* d_bad);
void launch_selftest_conv(Ctx& c, int64_t n, uint64_t seed, unsigned long long* d_bad);
void launch_selftest_cone(Ctx& c, int64_t n, uint64_t seed, unsigned long long* d_out);
}  // namespace sps
