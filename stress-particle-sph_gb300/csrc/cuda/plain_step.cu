// plain_step.cu -- FP64 "plain" step of the SPS hot path (compiled with -fmad=false).
//
// One launch sequence per step restates time_integration
// (example_problems/soil_failure_bui_et_al_2008/2_SPH_main_2018.f90:78-184) and RK4
// (:653-802).  The reference scatters every pair into both of its particles while it walks
// the pair linked list; here every target gathers its own terms from its neighbour list,
// which is stored in that same walk order, so each sum is formed in the same order and the
// result is bit-identical to the CPU oracle.
//
//   k_step_init   save x0 / vx0 / stress0 / rho0, clear RK accumulators (RK4 :681-690)
//   k_bound       boundary_forces (:1039), once per step: positions are frozen in a step
//   per stage i = 1..4:
//     k_stage_begin  stage state, density, adapt_stress2, BCs            (:700-716)
//     k_interp       stress_point_update                                 (:403-482)
//     k_adapt_bc     adapt_stress2 + BCs after the interpolation         (:720-723)
//     k_derivs       get_derivatives, plastic_terms, gravity, artificial viscosity,
//                    spin, RHS, RK accumulation                           (:725-777)
//   k_rk_final     final RK4 update, adapt, BCs, Ddev, update_strain      (:784-799, :125)
//   k_interp + k_adapt_bc                                                 (:130-135)
//   k_trapezoid | k_xsph, displacement                                    (:140-171)
#include <cuda_runtime.h>

#include "ctx.cuh"
#include "stage_tail.cuh"

namespace sps {

namespace {

constexpr int kBlock = 256;

// adapt_stress2: the reference's FP64 arithmetic in the plain form, the division-free
// variant in the FP32 form.  Both first certify in FP32 the stresses clearly inside the cone
// (most of them), which either routine would leave unchanged, and skip every FP64
// operation for those: the results are bit-identical.
__device__ __forceinline__ void stress_return(const Dev& D, const Real& M, double& a,
                                              double& b, double& c, double& d) {
  if (inside_cone_f32(M.alpha2f, M.kcf, a, b, c, d)) return;
  if (D.fast) adapt_stress_fast(M.alpha2, M.kc, M.kc_shift, a, b, c, d);
  else adapt_stress(M.alpha2, M.kc, a, b, c, d);
}

// FP32-form neighbour records of particle i (velocity, volume, stress, internal variable)
__device__ __forceinline__ float4 split2(double x, double y) {
  float xh, xl, yh, yl;
  f32_split(x, xh, xl);
  f32_split(y, yh, yl);
  return make_float4(xh, yh, xl, yl);
}

// Only the records a later kernel reads are written (every FP64 -> FP32 conversion costs
// an FP64-pipe issue): node velocities always, stress-point velocities for XSPH, stress of
// stress-points, and {iv1, m/rho, rho, m} where those change (rec_i).
__device__ __forceinline__ void write_records(const Dev& D, int i, bool rec_i, double vx,
                                              double vy, double a, double b, double c, double d) {
  const bool sp = i >= D.NN;
  if (!sp || D.xsph) D.recV[i] = split2(vx, vy);
  if (sp) D.recS[i] = make_float4(f32_rn(a), f32_rn(b), f32_rn(c), f32_rn(d));
  if (rec_i)
    D.recI[i] = make_float4(f32_rn(D.iv1[i]), f32_rn(D.vol[i]), f32_rn(D.rho[i]), f32_rn(D.mass[i]));
}

__global__ void k_load_scalars(Dev D) {
  int k = *D.step_idx;
  if (D.surr && threadIdx.x < 4) D.cand_count[threadIdx.x] = 0;  // the network's rows
  for (int r = threadIdx.x; r < D.R; r += blockDim.x) D.cur[r] = D.scal_table[(size_t)k * D.R + r];
}

// end of a step: the step counter, and the surrogate's gate for the next step
__global__ void k_next_step(Dev D) {
  *D.step_idx += 1;
  if (!D.surr) return;
  SurrGate& g = *D.surr_gate;
  const unsigned long long l = D.surr_cnt[0], a = D.surr_cnt[1];
  if (g.on) {
    g.steps_on += 1;
    // deltas of this step (the counters restart from 0 when the host resets them)
    const unsigned long long dl = l >= g.load0 ? l - g.load0 : l;
    const unsigned long long da = a >= g.ans0 ? a - g.ans0 : a;
    // a step without loading evaluations gave the network nothing to answer: it counts as
    // a step that did not pay
    if (g.min_frac > 0.0 && (dl == 0 || (double)da < g.min_frac * (double)dl)) {
      g.on = 0;
      g.wait = g.period;
      g.period = g.period * 2 < g.max_period ? g.period * 2 : g.max_period;
    } else {
      g.period = 1;
    }
  } else {
    g.steps_off += 1;
    if (--g.wait <= 0) g.on = 1;
  }
  g.load0 = l;
  g.ans0 = a;
}

// over every particle (N2): the dummies' positions are kept too, so that x0x, x0y hold the
// positions of the step's pair build for every particle (a rebuild of the lists after the
// step decides its band pairs from them)
__global__ void k_step_init(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N2) return;
  D.x0x[i] = D.px[i];
  D.x0y[i] = D.py[i];
  if (i >= D.NT) return;
  D.vx0[i] = D.vx[i];
  D.vy0[i] = D.vy[i];
  if (i >= D.NN) {
    D.st0[0][i] = D.s0[i];
    D.st0[1][i] = D.s1[i];
    D.st0[2][i] = D.s2[i];
    D.st0[3][i] = D.s3[i];
    D.rho0[i] = D.rho[i];
    D.hsml0[i] = D.hsml[i];
    for (int k = 0; k < 4; k++) {
      D.RKs[k][i] = 0.0;
      D.RHS1[k][i] = 0.0;
    }
    D.RKr[i] = 0.0;
    D.RKh[i] = 0.0;
    D.RKd[i] = 0.0;
    D.RHSr[i] = 0.0;
    D.RHSh[i] = 0.0;
    D.vx[i] = 0.0;  // RK4 clears vel and stress (:690)
    D.vy[i] = 0.0;
  } else {
    D.RKv[0][i] = 0.0;
    D.RKv[1][i] = 0.0;
    D.RHS2[0][i] = 0.0;
    D.RHS2[1][i] = 0.0;
    D.s0[i] = 0.0;
    D.s1[i] = 0.0;
    D.s2[i] = 0.0;
    D.s3[i] = 0.0;
    D.fbx[i] = 0.0;
    D.fby[i] = 0.0;
  }
}

// boundary_forces, test == 2 (2_SPH_main_2018.f90:1117-1161): FP32 locals.  Only innermost
// dummies closer than 0.75 dx give a non-zero term; they are summed in ascending id.
__device__ __forceinline__ bool bound_term(const Dev& D, const Real& M, int i, int j, float& fx,
                                           float& fy) {
  const float cc = 20.0f;
  const float d0 = (float)(M.dx / 2.0);
  float r0 = (float)(D.px[i] - D.px[j]);
  float r1 = (float)(D.py[i] - D.py[j]);
  float r2 = sqrtf(r0 * r0 + r1 * r1);
  float h = (float)(0.5 * (D.hsml[i] + D.hsml[j]));
  float r_bound = r2 / (0.75f * h);
  float f2;
  if (r2 > 0 && r2 < 1.5f * d0) f2 = 1.0f - (r2 / (1.5f * d0));
  else f2 = 0.0f;
  float f;
  if (0 < r_bound && r_bound <= 2.0f / 3.0f) f = 2.0f / 3.0f;
  else if (2.0f / 3.0f < r_bound && r_bound <= 1) f = 2.0f * r_bound - 1.5f * (r_bound * r_bound);
  else if (1 < r_bound && r_bound < 2) f = 0.5f * ((2.0f - r_bound) * (2.0f - r_bound));
  else f = 0.0f;
  if (f2 == 0.0f || f == 0.0f) return false;
  float k = ((0.01f * (cc * cc)) * f2) * f;
  fx = k * (r0 / (r2 * r2));
  fy = k * (r1 / (r2 * r2));
  return true;
}

// boundary_forces (2_SPH_main_2018.f90:1039-1165), test 2: the wall force on every node
// from the innermost dummy row, once per step (positions are frozen within a step)
__global__ void k_bound(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NN) return;
  constexpr int K = 8;
  int ids[K];
  float tx[K], ty[K];
  int n = 0;
  const Real& M = real_of(D, i);
  const int j0 = M.dum0, j1 = M.dum0 + M.ndum2;
  if (D.bound_from_lists) {
    const int col = D.lcol[D.spos[i]];
    int deg = D.degC[col];
    // the partner ids four at a time (independent loads in flight together; the compact
    // entries when the lists were gathered), then the innermost dummies among them
    for (int k0 = 0; k0 < deg; k0 += 4) {
      int uu[4];
#pragma unroll
      for (int q = 0; q < 4; q++)
        uu[q] = k0 + q >= deg ? -1
                : D.use_crossW ? D.crossW[(size_t)(k0 + q) * D.N2 + col].x
                               : D.cross[ell(k0 + q, col, D.N2)].x;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int u = uu[q];
        if (u < j0 || u >= j1) continue;
        float fx, fy;
        if (!bound_term(D, M, i, u, fx, fy)) continue;
        if (n < K) {
          int p = n++;
          while (p > 0 && ids[p - 1] > u) {
            ids[p] = ids[p - 1];
            tx[p] = tx[p - 1];
            ty[p] = ty[p - 1];
            p--;
          }
          ids[p] = u;
          tx[p] = fx;
          ty[p] = fy;
        } else {
          atomicOr(D.err, ERR_BOUND);
        }
      }
    }
    double bx = 0.0, by = 0.0;
    for (int k = 0; k < n; k++) {
      bx = bx + f64_of(tx[k]);
      by = by + f64_of(ty[k]);
    }
    D.fbx[i] = bx;
    D.fby[i] = by;
  } else {
    double bx = 0.0, by = 0.0;
    for (int j = j0; j < j1; j++) {
      float fx, fy;
      if (!bound_term(D, M, i, j, fx, fy)) continue;
      bx = bx + (double)fx;
      by = by + (double)fy;
    }
    D.fbx[i] = bx;
    D.fby[i] = by;
  }
}

// start of RK4 stage i (2_SPH_main_2018.f90:700-716): stage velocity and stress,
// density_update (:807-821) and h with sle 2, adapt_stress2 and the fixed BCs
__global__ void k_stage_begin(Dev D, int stage) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  const double f1 = stage == 0 ? 0.0 : stage == 3 ? 1.0 : 0.5;  // RK4 nodes 0, 1/2, 1/2, 1
  const int r = D.R == 1 ? 0 : D.rid[i];
  const Real& M = real_of(D, i);
  const double f1dt = f1 * M.dt;
  const StepScalars& sc = D.cur[r];
  double vx = D.vx[i], vy = D.vy[i];
  double a = D.s0[i], b = D.s1[i], c = D.s2[i], d = D.s3[i];
  if (i < D.NN) {
    vx = D.vx0[i] + f1dt * D.RHS2[0][i];
    vy = D.vy0[i] + f1dt * D.RHS2[1][i];
  } else {
    a = D.st0[0][i] + f1dt * D.RHS1[0][i];
    b = D.st0[1][i] + f1dt * D.RHS1[1][i];
    c = D.st0[2][i] + f1dt * D.RHS1[2][i];
    d = D.st0[3][i] + f1dt * D.RHS1[3][i];
    if (D.cont_density) {
      const double* g = D.grad_u + 4 * (size_t)i;
      double rr = -D.rho[i] * (g[0] + g[3]);
      D.RHSr[i] = rr;
      double rho = D.rho0[i] + f1dt * rr;
      D.rho[i] = rho;
      D.vol[i] = D.mass[i] / rho;
      D.rinv[i] = 1.0 / rho;
      if (D.sle == 2) {
        double rh = -(D.hsml0[i] / (rho * 2.0)) * rr;
        D.RHSh[i] = rh;
        D.hsml[i] = D.hsml0[i] + f1dt * rh;
      }
    }
  }
  // the FP32 form returns only stress that changed since the last return: a node's
  // stress is unchanged since the previous k_adapt_bc (or zero after k_step_init), and
  // returning it again would change it by rounding only
  if (M.ncrit == 12 && (!D.fast || i >= D.NN)) stress_return(D, M, a, b, c, d);
  apply_bcs(D, sc, i, vx, vy, a, b, c, d);
  D.vx[i] = vx;
  D.vy[i] = vy;
  D.s0[i] = a;
  D.s1[i] = b;
  D.s2[i] = c;
  D.s3[i] = d;
  if (D.fast) write_records(D, i, D.cont_density, vx, vy, a, b, c, d);
}

// stress_point_update (2_SPH_main_2018.f90:403-482) as a gather per target
// KIND 0: every sorted position; 1: the stress-point targets tgt[0..ntgt); 2: the node
// targets (a warp then runs one branch only: the FP64 pipe is not shared by both)
template <int KIND>
__global__ void k_interp(Dev D, const int32_t* __restrict__ tgt, int ntgt) {
  const int k0 = blockIdx.x * blockDim.x + threadIdx.x;
  int s;
  if (KIND == 0) {
    s = k0;
    if (s >= D.N2) return;
  } else {
    if (k0 >= ntgt) return;
    s = tgt[k0];
  }
  int t = D.sorted[s];
  int tt = D.itype[t];
  if (t >= D.NT) return;
  if (!D.sp_sph) {
    const Real& M = real_of(D, t);
    if (t >= D.NN) {
      int n = node_of_sp(M, t);
      D.vx[t] = D.vx[n];
      D.vy[t] = D.vy[n];
    } else {
      int sp = sp_of_node(M, t);
      D.s0[t] = D.s0[sp];
      D.s1[t] = D.s1[sp];
      D.s2[t] = D.s2[sp];
      D.s3[t] = D.s3[sp];
      D.iv1[t] = D.iv1[sp];
      if (D.cont_density) D.rho0[t] = D.rho[sp];
    }
    return;
  }
  const int col = list_col<KIND>(D, k0, s);
  int deg = D.degC[col];
  if (KIND == 1 || (KIND == 0 && is_sp(tt))) {
    double v0 = 0.0, v1 = 0.0, norm = 0.0;
    for (int k = 0; k < deg; k++) {
      int4 e = D.cross[ell(k, col, D.N2)];
      int u = e.x;
      if (e.y < 0) continue;  // a dummy partner (sign bit of W)
      double w = f64_of(__int_as_float(e.y));  // exact, on the integer pipe
      double h2 = D.vol[u] * w;  // (mass/rho)*w with mass/rho formed once per particle
      v0 = v0 + D.vx[u] * h2;
      v1 = v1 + D.vy[u] * h2;
      norm = norm + div_rcp(w * D.mass[u], D.rho[u], D.rinv[u]);
    }
    if (norm != 0) {
      D.vx[t] = v0 / norm;
      D.vy[t] = v1 / norm;
    }
  } else {
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0, iv = 0.0, rt = 0.0, norm = 0.0;
    for (int k = 0; k < deg; k++) {
      int4 e = D.cross[ell(k, col, D.N2)];
      int u = e.x;
      if (e.y < 0) continue;  // a dummy partner (sign bit of W)
      double w = f64_of(__int_as_float(e.y));  // exact, on the integer pipe
      double ru = D.rho[u];
      double h1 = D.vol[u] * w;
      a = a + D.s0[u] * h1;
      b = b + D.s1[u] * h1;
      c = c + D.s2[u] * h1;
      d = d + D.s3[u] * h1;
      iv = iv + D.iv1[u] * h1;
      if (D.cont_density) rt = rt + ru * h1;
      norm = norm + div_rcp(w * D.mass[u], ru, D.rinv[u]);
    }
    if (norm != 0) {
      D.s0[t] = a / norm;
      D.s1[t] = b / norm;
      D.s2[t] = c / norm;
      D.s3[t] = d / norm;
      D.iv1[t] = iv / norm;
    } else {
      D.vx[t] = 0.0;
      D.vy[t] = 0.0;
    }
    if (D.cont_density) D.rho0[t] = rt / norm;  // staged: stress-points still read node rho
  }
}

// node density of stress_point_update with cont_density (2_SPH_main_2018.f90:403-482),
// applied after every node has read the stress-points
__global__ void k_node_rho(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < D.NN) {
    double r = D.rho0[i];
    D.rho[i] = r;
    D.vol[i] = D.mass[i] / r;
    D.rinv[i] = 1.0 / r;
  }
}

// adapt_stress2 + BCs after the interpolation (SP-SPH only), then sigma / rho^2 of the
// stage for get_derivatives (the same quotient the reference forms per pair)
__global__ void k_adapt_bc(Dev D, int with_A, int bcs = 1) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  const int r = D.R == 1 ? 0 : D.rid[i];
  const Real& M = real_of(D, i);
  const StepScalars& sc = D.cur[r];
  double vx = D.vx[i], vy = D.vy[i];
  double a = D.s0[i], b = D.s1[i], c = D.s2[i], d = D.s3[i];
  if (D.sp_sph) {
    // FP32 form: a stress-point's stress is unchanged since k_stage_begin / k_rk_final
    // returned it; only the interpolated node stress needs the return here
    if (M.ncrit == 12 && (!D.fast || i < D.NN)) stress_return(D, M, a, b, c, d);
    if (bcs) apply_bcs(D, sc, i, vx, vy, a, b, c, d);
    D.vx[i] = vx;
    D.vy[i] = vy;
    D.s0[i] = a;
    D.s1[i] = b;
    D.s2[i] = c;
    D.s3[i] = d;
  }
  if (with_A) {
    if (D.fast) {
      // sigma / rho^2 as sigma (1/rho)^2: no FP64 division (the records carry ~48 bits);
      // only the records are stored (k_fderivs forms the FP64 value again where it needs it)
      double ri = D.rinv[i];
      double ri2 = ri * ri;
      double A0 = a * ri2, A1 = b * ri2, A2 = c * ri2;
      float h0, h1, h2, l0, l1, l2;
      f32_split(A0, h0, l0);
      f32_split(A1, h1, l1);
      f32_split(A2, h2, l2);
      D.recA[i] = make_float4(h0, h1, h2, f32_rn(D.mass[i]));
      D.recAl[i] = make_float4(l0, l1, l2, 0.0f);
    } else {
      double r = D.rho[i];
      double r2 = r * r;
      D.A[0][i] = a / r2;
      D.A[1][i] = b / r2;
      D.A[2][i] = c / r2;
    }
  }
  if (D.fast) {
    if (i < D.NN || D.xsph) D.recV[i] = split2(vx, vy);
    if (D.cont_density)
      D.recI[i] = make_float4(f32_rn(D.iv1[i]), f32_rn(D.vol[i]), f32_rn(D.rho[i]), f32_rn(D.mass[i]));
  }
}

// m / rho and 1 / rho of particles [lo, hi)
__global__ void k_vol(Dev D, int lo, int hi) {
  int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi) return;
  double r = D.rho[i];
  D.vol[i] = D.mass[i] / r;
  D.rinv[i] = 1.0 / r;
  if (D.fast) {
    D.recV[i] = split2(D.vx[i], D.vy[i]);
    D.recI[i] = make_float4(i < D.NT ? (float)D.iv1[i] : 0.0f, (float)D.vol[i], (float)r,
                            (float)D.mass[i]);
  }
}

// artificial_force's per-particle part (2_SPH_main_2018.f90:930-981) for every node, from
// the stage's node stresses: the principal stresses at angle 0.5 atan(2 s12 / (s11 - s22))
// (0 unless s11 - s22 >= 1e-8), their tensile parts times -eps / rho^2 (eps = 0.1), rotated
// back as the reference does (its second component is R2(1) (cos^2 + sin^2))
__global__ void k_art_R(Dev D) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NN) return;
  const double eps = (double)0.1f;
  const double s0 = D.s0[i], s1 = D.s1[i], s2 = D.s2[i], rho = D.rho[i];
  const double s12 = s0 - s1;
  double th = 0.0;
  if (s12 >= (double)1e-08f) th = 0.5 * atan((2.0 * s2) / s12);
  const double co = cos(th), si = sin(th), cc = co * co, ss = si * si;
  const double cs2 = (2.0 * co) * si;
  const double sig0 = (cc * s0 + cs2 * s2) + ss * s1;
  const double sig1 = (ss * s0 - cs2 * s2) + cc * s1;
  const double R20 = sig0 > 0 ? -(eps * (sig0 / (rho * rho))) : 0.0;
  const double R21 = sig1 > 0 ? -(eps * (sig1 / (rho * rho))) : 0.0;
  D.artR[i] = R20 * cc + R21 * ss;
  D.artR[D.NN + i] = R20 * (cc + ss);
  D.artR[2 * (size_t)D.NN + i] = (R20 - R21) * (co * si);
}

// shift_stress_points (2_SPH_main_2018.f90:244-368) for node i and its stress-points
// (ids sp0 + npoints (i - node0) + q): with `reposition`, the points are placed again at the
// fixed offsets (npoints 1-3; the second point of two takes r_x as its y offset, as in the
// reference) or, with the velocity-vector variant, along the node velocity when the node
// moved more than disp_tol dx since the last shift; then, every step, they are put on the
// node when it is next to a wall and moves faster than 0.4, or has fewer than two node
// neighbours (isolated_nodes: its node-node pairs, the node's same-type list).  cos_theta,
// sin_theta, r_x2 and abs_vel are FP32 in the reference.
__global__ void k_shift(Dev D, int reposition) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NN) return;
  const Real& M = real_of(D, i);
  const int np = D.npoints;
  const int k = M.sp0 + np * (i - M.node0);
  const double xi = D.px[i], yi = D.py[i], v0 = D.vx[i], v1 = D.vy[i];
  if (reposition) {
    if (D.vel_vector) {
      const double ex = xi - D.x10x[i], ey = yi - D.x10y[i];
      const double d10 = sqrt(ex * ex + ey * ey) / M.dx;
      D.disp10[i] = d10;
      D.x10x[i] = xi;
      D.x10y[i] = yi;
      const double dx = M.dx;
      const float ct = (float)(v0 / sqrt(v0 * v0 + v1 * v1));
      const float st = (float)(v1 / sqrt(v0 * v0 + v1 * v1));
      float r0 = (float)((dx / 2) * (double)ct), r1 = (float)((dx / 2) * (double)st);
      if (r0 > 0 && r0 < dx / 5) r0 = (float)((double)r0 + dx / 3.0);
      if (r1 > 0 && r1 < dx / 5) r1 = (float)((double)r1 + dx / 3.0);
      if (r0 < 0 && r0 > -(dx / 5)) r0 = (float)((double)r0 - dx / 3.0);
      if (r1 < 0 && r1 > -(dx / 5)) r1 = (float)((double)r1 - dx / 3.0);
      if (d10 > M.disp_tol) {
        D.px[k] = xi + (double)r0;
        D.py[k] = yi + (double)r1;
        D.px[k + 1] = xi - (double)r0;
        D.py[k + 1] = yi - (double)r1;
      }
    } else if (np == 1) {
      D.px[k] = xi + M.r_x;
      D.py[k] = yi + M.r_y;
    } else if (np == 2) {
      D.px[k] = xi + M.r_x;
      D.py[k] = yi + M.r_y;
      D.px[k + 1] = xi - M.r_x;
      D.py[k + 1] = yi - M.r_x;
    } else if (np == 3) {
      D.px[k] = xi;
      D.py[k] = yi + M.r_y;
      D.px[k + 1] = xi - M.r_x;
      D.py[k + 1] = yi - M.r_y;
      D.px[k + 2] = xi + M.r_x;
      D.py[k + 2] = yi - M.r_y;
    }
  }
  const float abs_vel = (float)sqrt(v0 * v0 + v1 * v1);
  const int n_int = D.degS[D.lcol[D.spos[i]]];
  if ((D.bc_int[i] == 1 && abs_vel > 0.4f) || n_int < 2)
    for (int q = 0; q < np && q < 3; q++) {
      D.px[k + q] = xi;
      D.py[k + q] = yi;
    }
}

// get_derivatives (2_SPH_main_2018.f90:487-648) + the per-particle stage work of RK4.
// KIND as k_interp.
template <int KIND>
__global__ void k_derivs(Dev D, int stage, const int32_t* __restrict__ tgt, int ntgt) {
  const int k0 = blockIdx.x * blockDim.x + threadIdx.x;
  int s;
  if (KIND == 0) {
    s = k0;
    if (s >= D.N2) return;
  } else {
    if (k0 >= ntgt) return;
    s = tgt[k0];
  }
  int t = D.sorted[s];
  if (t >= D.NT) return;
  const double f2 = (stage == 1 || stage == 2) ? 2.0 : 1.0;  // RK4 weights 1, 2, 2, 1
  const Real& Mt = real_of(D, t);
  const StepScalars& sc = D.cur[D.R == 1 ? 0 : D.rid[t]];
  int tt = D.itype[t];
  const int col = list_col<KIND>(D, k0, s);
  int deg = D.degC[col];
  double AE[4] = {0.0, 0.0, 0.0, 0.0};
  const double xt = D.px[t], yt = D.py[t];
  if (KIND == 1 || (KIND == 0 && is_sp(tt))) {
    double g[4] = {0.0, 0.0, 0.0, 0.0};  // grad1(a,b) at a + 2b
    const double vt[2] = {D.vx[t], D.vy[t]};
    for (int k = 0; k < deg; k++) {
      int4 e = D.cross[ell(k, col, D.N2)];
      int u = e.x;
      const bool wall = e.y < 0;  // a dummy partner (sign bit of W)
      double Gx = f64_of(__int_as_float(e.z)), Gy = f64_of(__int_as_float(e.w));
      double mu = D.mass[u], ru = D.rho[u], iu = D.rinv[u];
      if (!wall) {  // node -- stress-point (target is pair_i)
        double h1 = div_rcp(Gx * mu, ru, iu);
        double h2 = div_rcp(Gy * mu, ru, iu);
        double du0 = D.vx[u] - vt[0], du1 = D.vy[u] - vt[1];
        g[0] = g[0] + du0 * h1;
        g[2] = g[2] + du0 * h2;
        g[1] = g[1] + du1 * h1;
        g[3] = g[3] + du1 * h2;
        if (D.cspm) {
          double xu = D.px[u] - xt, yu = D.py[u] - yt;
          AE[0] = AE[0] + xu * h1;
          AE[1] = AE[1] + yu * h1;
          AE[2] = AE[2] + xu * h2;
          AE[3] = AE[3] + yu * h2;
        }
      } else {  // stress-point -- dummy (dummy is pair_i)
        double wall = (double)D.wallpos[u];
        double da, db;
        if (D.horiz[u] == 1.0f) {
          da = fabs(yt - wall);
          db = fabs(D.py[u] - wall);
        } else {
          da = fabs(xt - wall);
          db = fabs(D.px[u] - wall);
        }
        double bq = 1.0 + db / da;
        double beta = 1.5 < bq ? 1.5 : bq;
        double dv0 = vt[0] * (1.0 - beta) + beta * 0.0;
        double dv1 = vt[1] * (1.0 - beta) + beta * 0.0;
        double hh1 = div_rcp(-Gx * mu, ru, iu);
        double hh2 = div_rcp(-Gy * mu, ru, iu);
        g[0] = g[0] + (vt[0] - dv0) * hh1;
        g[2] = g[2] + (vt[0] - dv0) * hh2;
        g[1] = g[1] + (vt[1] - dv1) * hh1;
        g[3] = g[3] + (vt[1] - dv1) * hh2;
      }
    }
    tail_sp(D, sc, t, g, AE, f2);
  } else if (is_node(tt)) {
    double g2[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};  // grad2(s,b) at s + 3b
    const double rt = D.rho[t];
    const double at[3] = {D.A[0][t], D.A[1][t], D.A[2][t]};  // sigma / rho^2 of the target
    const double stt[3] = {D.s0[t], D.s1[t], D.s2[t]};
    int bc_int = 0;
    for (int k = 0; k < deg; k++) {
      int4 e = D.cross[ell(k, col, D.N2)];
      int u = e.x;
      const bool wall = e.y < 0;  // a dummy partner (sign bit of W)
      double dwx = -f64_of(__int_as_float(e.z)), dwy = -f64_of(__int_as_float(e.w));
      double mu = D.mass[u];
      if (!wall) {  // node -- stress-point (stress-point is pair_i)
        const double au[3] = {D.A[0][u], D.A[1][u], D.A[2][u]};
        for (int q = 0; q < 3; q++) {
          double sum = at[q] + au[q];
          g2[q] = g2[q] - mu * (dwx * sum);
          g2[q + 3] = g2[q + 3] - mu * (dwy * sum);
        }
        if (D.cspm) {
          double ru = D.rho[u], iu = D.rinv[u];
          double h1b = -div_rcp(dwx * mu, ru, iu);
          double h2b = -div_rcp(dwy * mu, ru, iu);
          double xu = D.px[u] - xt, yu = D.py[u] - yt;
          AE[0] = AE[0] + xu * h1b;
          AE[1] = AE[1] + yu * h1b;
          AE[2] = AE[2] + xu * h2b;
          AE[3] = AE[3] + yu * h2b;
        }
      } else {  // node -- dummy: the dummy carries the node's stress
        bc_int = 1;
        double ru = D.rho[u];
        double ru2 = ru * ru;
        for (int q = 0; q < 3; q++) {
          double sum = at[q] + stt[q] / ru2;
          g2[q] = g2[q] - mu * (dwx * sum);
          g2[q + 3] = g2[q + 3] - mu * (dwy * sum);
        }
      }
    }
    const double vtx = D.vx[t], vty = D.vy[t];
    double avx = 0.0, avy = 0.0;
    if (Mt.alpha > 0 || Mt.beta > 0) {
      // artificial_viscosity (2_SPH_main_2018.f90:826-904): FP32 accumulators
      float ax = 0.0f, ay = 0.0f;
      int degs = D.degS[col];
      for (int k = 0; k < degs; k++) {
        int4 e = D.same[ell(k, col, D.N2)];
        int u = e.x;
        float xij = (float)(xt - D.px[u]);
        float yij = (float)(yt - D.py[u]);
        float h = (float)(0.5 * (D.hsml[t] + D.hsml[u]));
        float rho2 = (float)(0.5 * (rt + D.rho[u]));
        float div_u = (float)((double)xij * (vtx - D.vx[u]));
        div_u = (float)((double)div_u + (double)yij * (vty - D.vy[u]));
        float sq = sqrtf(xij * xij + yij * yij);
        float theta = (h * div_u) / (sq * sq + 0.01f * (h * h));
        float visc = 0.0f;
        if (div_u < 0)
          visc = (float)((-((Mt.alpha * 600.0) * (double)theta) + Mt.beta * (double)(theta * theta)) /
                         (double)rho2);
        float px = visc * __int_as_float(e.z), py = visc * __int_as_float(e.w);
        double mu = D.mass[u];
        ax = (float)((double)ax + (double)px * mu);
        ay = (float)((double)ay + (double)py * mu);
      }
      avx = -(double)ax;
      avy = -(double)ay;
    }
    double afx = 0.0, afy = 0.0;
    if (D.art_stress) art_force_node(D, col, t, &afx, &afy);
    tail_node(D, sc, t, g2, AE, bc_int, avx, avy, f2, afx, afy);
  }
}

// end of RK4 (2_SPH_main_2018.f90:784-799): velocity and stress from the accumulated
// rates, adapt_stress2, BCs, density and h, Ddev_strn; update_strain
// (3_SPH_material_2018.f90:1864-1880)
__global__ void k_rk_final(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  const int r = D.R == 1 ? 0 : D.rid[i];
  const Real& M = real_of(D, i);
  const StepScalars& sc = D.cur[r];
  const double dt6 = M.dt6;  // dt / 6, the host's IEEE quotient
  double vx = D.vx[i], vy = D.vy[i];
  double a = D.s0[i], b = D.s1[i], c = D.s2[i], d = D.s3[i];
  if (i < D.NN) {
    vx = D.vx0[i] + dt6 * D.RKv[0][i];
    vy = D.vy0[i] + dt6 * D.RKv[1][i];
  } else {
    a = D.st0[0][i] + dt6 * D.RKs[0][i];
    b = D.st0[1][i] + dt6 * D.RKs[1][i];
    c = D.st0[2][i] + dt6 * D.RKs[2][i];
    d = D.st0[3][i] + dt6 * D.RKs[3][i];
  }
  // FP32 form: node stress is unchanged since the last k_adapt_bc
  if (M.ncrit == 12 && (!D.fast || i >= D.NN)) stress_return(D, M, a, b, c, d);
  apply_bcs(D, sc, i, vx, vy, a, b, c, d);
  D.vx[i] = vx;
  D.vy[i] = vy;
  D.s0[i] = a;
  D.s1[i] = b;
  D.s2[i] = c;
  D.s3[i] = d;
  if (i >= D.NN) {
    if (D.cont_density) {
      double r = D.rho0[i] + dt6 * D.RKr[i];
      D.rho[i] = r;
      D.vol[i] = D.mass[i] / r;
      D.rinv[i] = 1.0 / r;
      if (D.sle == 2) D.hsml[i] = D.hsml0[i] + dt6 * D.RKh[i];
    }
    // RKd / 6 correctly rounded: the Markstein-corrected product with RN(1/6) for normal
    // operands (div_rcp), the IEEE division for zero and extreme exponents
    const double rkd = D.RKd[i];
    const int ex = (int)((__double_as_longlong(rkd) >> 52) & 0x7FF);
    double dd = (ex > 64 && ex < 1980) ? div_rcp(rkd, 6.0, 1.0 / 6.0) : rkd / 6.0;
    D.Ddev[i] = dd;
    D.iv1[i] = D.iv1[i] + M.dt * dd;  // update_strain (3_SPH_material_2018.f90:1864)
  }
  if (D.fast) write_records(D, i, i >= D.NN || D.cont_density, vx, vy, a, b, c, d);
}

// position update of time_integration without XSPH (2_SPH_main_2018.f90:145-146):
// x = x0 + vel_half dt with vel_half = 0.5 (v0 + v) rounded to FP32
__global__ void k_trapezoid(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  if (D.update_x) {
    // the conversions on the integer pipe (the same bits as the hardware's)
    float hx = f32_rn(0.5 * (D.vx0[i] + D.vx[i]));
    float hy = f32_rn(0.5 * (D.vy0[i] + D.vy[i]));
    const double dt = real_of(D, i).dt;
    double x = D.x0x[i] + f64_of(hx) * dt;
    double y = D.x0y[i] + f64_of(hy) * dt;
    D.px[i] = x;
    D.py[i] = y;
  }
}

// XSPH_update (2_SPH_main_2018.f90:189-239)
__global__ void k_xsph(Dev D) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  int t = D.sorted[s];
  if (t >= D.NT) return;
  const int col = D.lcol[s];
  int deg = D.degS[col];
  const double vt0 = D.vx[t], vt1 = D.vy[t];
  double s0 = 0.0, s1 = 0.0;
  int flag = D.bc_or_not[t];
  bool mark = false;
  for (int k = 0; k < deg; k++) {
    int4 e = D.same[ell(k, col, D.N2)];
    int u = e.x;
    double w = f64_of(__int_as_float(e.y));  // exact, on the integer pipe
    double vol = D.vol[u];
    s0 = s0 + (vol * (D.vx[u] - vt0)) * w;
    s1 = s1 + (vol * (D.vy[u] - vt1)) * w;
    if (t < D.NN && D.bc_or_not[u] == 2 && flag != 2) mark = true;
  }
  const double eps = 0.5;
  const double dt = real_of(D, t).dt;
  D.px[t] = D.x0x[t] + dt * (vt0 + eps * s0);
  D.py[t] = D.x0y[t] + dt * (vt1 + eps * s1);
  if (mark) D.bc_or_not[t] = 3;
}

// displ = x - x00 (2_SPH_main_2018.f90:166-171; stress-points follow the nodes in
// standard SPH), or accumulated from the velocities when positions are frozen (:180)
__global__ void k_displ(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NN) return;
  const Real& M = real_of(D, i);
  if (D.update_x) {
    if (!D.sp_sph) {
      D.px[sp_of_node(M, i)] = D.px[i];
      D.py[sp_of_node(M, i)] = D.py[i];
    }
    D.dispx[i] = D.px[i] - D.x00x[i];
    D.dispy[i] = D.py[i] - D.x00y[i];
  } else {
    D.dispx[i] = D.dispx[i] + (0.5 * (D.vx0[i] + D.vx[i])) * M.dt;
    D.dispy[i] = D.dispy[i] + (0.5 * (D.vy0[i] + D.vy[i])) * M.dt;
  }
}

}  // namespace

// self-test of div_rcp against the IEEE division on n pseudo-random operands
// (log-uniform magnitudes over the ranges the step meets, random signs)
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__global__ void k_selftest_div(int64_t n, uint64_t seed, unsigned long long* bad) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  unsigned long long nb = 0;
  for (; i < n; i += stride) {
    uint64_t r1 = mix64(seed ^ (uint64_t)i), r2 = mix64(r1), r3 = mix64(r2);
    double ea = -40.0 + 52.0 * ((r1 >> 11) * 0x1.0p-53);  // |a| in [1e-40, 1e12]
    double eb = -6.0 + 14.0 * ((r2 >> 11) * 0x1.0p-53);   // |b| in [1e-6, 1e8]
    double a = exp2(ea * 3.3219280948873622) * ((r3 & 1) ? -1.0 : 1.0);
    double b = exp2(eb * 3.3219280948873622) * ((r3 & 2) ? -1.0 : 1.0);
    double y = 1.0 / b;
    double q1 = div_rcp(a, b, y), q2 = a / b;
    if (__double_as_longlong(q1) != __double_as_longlong(q2)) nb++;
    // the float rounding of the quotient, also where the float boundary is near: a scaled
    // so that a / b sits within a few double ulps of a float or of a float half-way point
    if (__float_as_uint(div_rcp_f32(a, b, y)) != __float_as_uint((float)q2)) nb++;
    const float f2 = (float)q2;
    const double near = (r3 & 4) ? 0.5 * ((double)f2 + (double)nextafterf(f2, 2.0f * f2)) : (double)f2;
    const double a2 = near * b + (double)((int)((r3 >> 8) & 7) - 3) * ldexp(near * b, -52);
    const double q3 = a2 / b;
    if (__float_as_uint(div_rcp_f32(a2, b, y)) != __float_as_uint((float)q3)) nb++;
  }
  if (nb) atomicAdd(bad, nb);
}

// the integer-pipe conversions against the hardware ones on n pseudo-random doubles
// (log-uniform magnitudes 1e-45..1e45, both signs) and their float roundings
__global__ void k_selftest_conv(int64_t n, uint64_t seed, unsigned long long* bad) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  unsigned long long nb = 0;
  for (; i < n; i += stride) {
    uint64_t r1 = mix64(seed ^ (uint64_t)i), r2 = mix64(r1);
    double e = -45.0 + 90.0 * ((r1 >> 11) * 0x1.0p-53);
    double x = exp2(e * 3.3219280948873622) * ((r2 & 1) ? -1.0 : 1.0);
    if ((r2 & 0xF0) == 0) x = (double)(float)x;  // exact floats and halfway cases nearby
    if ((r2 & 0xF00) == 0) x = x + x * 0x1.0p-24;
    if ((r2 & 0xF000) == 0) x = (r2 & 1) ? -0.0 : 0.0;  // signed zeros (an integer-pipe case)
    float h = f32_rn(x), hs, ls;
    f32_split(x, hs, ls);
    float hr = (float)x, lr = (float)(x - (double)hr);
    double b = f64_of(hr);
    // the integer-pipe int -> float conversion over |r| < 2^29 (f32_split's remainders),
    // ties included (low bits cleared to land on halfway cases)
    int ri = (int)(r2 >> 34) - (1 << 29);
    if ((r2 & 0x30000) == 0) ri &= ~0x3F;
    if (__float_as_uint(i2f_rn(ri)) != __float_as_uint(__int2float_rn(ri))) nb++;
    if (__float_as_uint(h) != __float_as_uint(hr) || __float_as_uint(hs) != __float_as_uint(hr) ||
        __float_as_uint(ls) != __float_as_uint(lr) ||
        __double_as_longlong(b) != __double_as_longlong((double)hr))
      nb++;
  }
  if (nb) atomicAdd(bad, nb);
}

// the FP32 inside-the-cone certification of the stress return against the FP64 returns it
// lets the step skip, on n pseudo-random Drucker-Prager materials and stresses, a quarter
// of them placed within a relative 1e-3 .. 1e-9 of the cone and a quarter nearly
// hydrostatic: bad counts certified stresses that the plain form's adapt_stress (the
// reference's arithmetic) or the FP32 form's adapt_stress_fast would change in any bit;
// certified counts the certified ones
__global__ void k_selftest_cone(int64_t n, uint64_t seed, unsigned long long* bad,
                                unsigned long long* certified) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  unsigned long long nb = 0, nc = 0;
  for (; i < n; i += stride) {
    uint64_t r1 = mix64(seed ^ (uint64_t)i), r2 = mix64(r1), r3 = mix64(r2), r4 = mix64(r3);
    auto uni = [](uint64_t r) { return (double)(r >> 11) * 0x1.0p-53; };
    const double tanfi = 0.05 + 1.2 * uni(r1);
    const double coh = (r1 & 3) == 0 ? 0.0 : 1e5 * uni(mix64(r1 ^ 7));
    const double den = sqrt(9.0 + 12.0 * (tanfi * tanfi));
    const double alpha2 = tanfi / den, kc = (3.0 * coh) / den;
    // stress magnitudes 1e-30 .. 1e30 (the test's range guard), mostly 1e-3 .. 1e9
    const double scale = (r2 & 7) == 0 ? exp2(-100.0 + 200.0 * uni(r2)) : exp2(-10.0 + 40.0 * uni(r2));
    const double p = -scale * (uni(r3) - 0.1);         // mostly compressive mean stress
    double s0 = scale * (2.0 * uni(mix64(r3 ^ 1)) - 1.0), s1 = scale * (2.0 * uni(mix64(r3 ^ 2)) - 1.0);
    double s2 = scale * (2.0 * uni(mix64(r3 ^ 3)) - 1.0);
    const int mode = (int)(r4 & 3);
    if (mode == 3) {  // nearly hydrostatic
      const double f = exp2(-30.0 * uni(mix64(r4 ^ 5)));
      s0 *= f;
      s1 *= f;
      s2 *= f;
    }
    // deviator (s0, s1, -(s0 + s1), s2): sxx, syy, szz around the mean p, and sxy
    double a = p + s0, b = p + s1, d = p - (s0 + s1), c = s2;
    if (mode == 2) {  // onto the cone, then off it by a relative 1e-3 .. 1e-9 either way
      const double smean = ((a + b) + d) / 3.0;
      const double d0 = a - smean, d1 = b - smean, d3 = d - smean;
      const double sj = sqrt(c * c + 0.5 * (d0 * d0 + d1 * d1 + d3 * d3));
      const double y = kc - 3.0 * alpha2 * smean;
      if (sj > 0.0 && y > 0.0) {
        const double eps = exp2(-10.0 - 20.0 * uni(mix64(r4 ^ 9))) * ((r4 & 4) ? 1.0 : -1.0);
        const double k = (y / sj) * (1.0 + eps);
        a = smean + k * d0;
        b = smean + k * d1;
        d = smean + k * d3;
        c = k * c;
      }
    }
    if (inside_cone_f32((float)alpha2, (float)kc, a, b, c, d)) {
      nc++;
      // both returns must leave a certified stress exactly as it is
      double p0 = a, p1 = b, p2 = c, p3 = d, f0 = a, f1 = b, f2 = c, f3 = d;
      adapt_stress(alpha2, kc, p0, p1, p2, p3);
      adapt_stress_fast(alpha2, kc, alpha2 > 0.0 ? kc / (3.0 * alpha2) : 0.0, f0, f1, f2, f3);
      auto same = [](double x, double y) { return __double_as_longlong(x) == __double_as_longlong(y); };
      if (!(same(p0, a) && same(p1, b) && same(p2, c) && same(p3, d) && same(f0, a) &&
            same(f1, b) && same(f2, c) && same(f3, d)))
        nb++;
    }
  }
  if (nb) atomicAdd(bad, nb);
  if (nc) atomicAdd(certified, nc);
}

void launch_selftest_cone(Ctx& c, int64_t n, uint64_t seed, unsigned long long* d_out) {
  k_selftest_cone<<<152 * 8, 256, 0, c.stream>>>(n, seed, d_out, d_out + 1);
}

void launch_selftest_conv(Ctx& c, int64_t n, uint64_t seed, unsigned long long* d_bad) {
  k_selftest_conv<<<152 * 8, 256, 0, c.stream>>>(n, seed, d_bad);
}

void launch_selftest_div(Ctx& c, int64_t n, uint64_t seed, unsigned long long* d_bad) {
  k_selftest_div<<<152 * 8, 256, 0, c.stream>>>(n, seed, d_bad);
}

void launch_vol(Ctx& c, int lo, int hi) {
  if (hi > lo) k_vol<<<(hi - lo + kBlock - 1) / kBlock, kBlock, 0, c.stream>>>(c.d, lo, hi);
}

// the plain interpolation and derivative kernels, split by target kind like the FP32 form's
void launch_pinterp(Ctx& c) {
  const Dev& D = c.d;
  const int b = c.blk[TK_INTERP], ns = D.NT - D.NN;
  if (!D.sp_sph) {
    k_interp<0><<<c.grid_of(TK_INTERP, D.N2), b, 0, c.stream>>>(D, nullptr, 0);
    return;
  }
  c.kernels_launched += 1;
  if (ns > 0) k_interp<1><<<(ns + b - 1) / b, b, 0, c.stream>>>(D, D.tgtS, ns);
  k_interp<2><<<(D.NN + b - 1) / b, b, 0, c.stream>>>(D, D.tgtN, D.NN);
}
void launch_pderivs(Ctx& c, int stage) {
  const Dev& D = c.d;
  const int b = c.blk[TK_DERIVS], ns = D.NT - D.NN;
  if (!D.sp_sph) {
    k_derivs<0><<<c.grid_of(TK_DERIVS, D.N2), b, 0, c.stream>>>(D, stage, nullptr, 0);
    return;
  }
  c.kernels_launched += 1;
  if (ns > 0) k_derivs<1><<<(ns + b - 1) / b, b, 0, c.stream>>>(D, stage, D.tgtS, ns);
  k_derivs<2><<<(D.NN + b - 1) / b, b, 0, c.stream>>>(D, stage, D.tgtN, D.NN);
}

int launch_plain_step(Ctx& c) {
  Dev& D = c.d;
  cudaStream_t st = c.stream;
  int nbT = (D.NT + kBlock - 1) / kBlock;
  int nbN = (D.NN + kBlock - 1) / kBlock;
  c.mark("load_scalars");
  k_load_scalars<<<1, 128, 0, st>>>(D);
  launch_pair_build(c);
  if (c.step_variant & 1) {
    // the outside approach re-interpolates after a shift: stress_point_update and
    // adapt_stress2 (2_SPH_main_2018.f90:99-108)
    c.mark("interp");
    if (D.fast) launch_finterp(c);
    else launch_pinterp(c);
    if (D.cont_density) {
      c.mark("node_rho");
      k_node_rho<<<nbN, kBlock, 0, st>>>(D);
    }
    c.mark("adapt_bc");
    k_adapt_bc<<<c.grid_of(TK_ADAPT, D.NT), c.blk[TK_ADAPT], 0, st>>>(D, 0, 0);
  }
  c.mark("step_init");
  k_step_init<<<(D.N2 + kBlock - 1) / kBlock, kBlock, 0, st>>>(D);
  if (D.inside) {
    c.mark("bound");
    k_bound<<<nbN, kBlock, 0, st>>>(D);
  }
  for (int stage = 0; stage < 4; stage++) {
    c.mark("stage_begin");
    k_stage_begin<<<c.grid_of(TK_STAGE, D.NT), c.blk[TK_STAGE], 0, st>>>(D, stage);
    c.mark("interp");
    if (D.fast) launch_finterp(c);
    else launch_pinterp(c);
    if (D.cont_density && D.sp_sph) {
      c.mark("node_rho");
      k_node_rho<<<nbN, kBlock, 0, st>>>(D);
    }
    c.mark("adapt_bc");
    k_adapt_bc<<<c.grid_of(TK_ADAPT, D.NT), c.blk[TK_ADAPT], 0, st>>>(D, 1);
    if (D.art_stress) {
      c.mark("art_R");
      k_art_R<<<nbN, kBlock, 0, st>>>(D);
    }
    c.mark("derivs");
    if (D.fast) launch_fderivs(c, stage);
    else launch_pderivs(c, stage);
    if (D.fast) {
      c.mark("sp_tail");
      launch_fsp_tail(c, stage);
    }
  }
  c.mark("rk_final");
  k_rk_final<<<c.grid_of(TK_RKFINAL, D.NT), c.blk[TK_RKFINAL], 0, st>>>(D);
  c.mark("interp");
  if (D.fast) launch_finterp(c);
  else launch_pinterp(c);
  if (D.cont_density && D.sp_sph) {
    c.mark("node_rho");
    k_node_rho<<<nbN, kBlock, 0, st>>>(D);
  }
  if (D.sp_sph || D.fast) {
    c.mark("adapt_bc");
    k_adapt_bc<<<c.grid_of(TK_ADAPT, D.NT), c.blk[TK_ADAPT], 0, st>>>(D, 0);
  }
  if (D.update_x && D.xsph) {
    c.mark("xsph");
    if (D.fast) launch_fxsph(c);
    else k_xsph<<<c.grid_of(TK_XSPH, D.N2), c.blk[TK_XSPH], 0, st>>>(D);
  } else {
    c.mark("trapezoid");
    k_trapezoid<<<nbT, kBlock, 0, st>>>(D);
  }
  // get_nodes_on_free_surface after the position update (2_SPH_main_2018.f90:153); on
  // demand instead when no later step reads it (Ctx::surf_every)
  if (D.update_x && c.surf_every) launch_surface(c);
  if (D.update_x && D.outside) {
    c.mark("shift");
    k_shift<<<nbN, kBlock, 0, st>>>(D, (c.step_variant & 2) ? 1 : 0);
  }
  c.mark("displ");
  k_displ<<<nbN, kBlock, 0, st>>>(D);
  c.mark("next_step");
  k_next_step<<<1, 1, 0, st>>>(D);
  return 0;
}

}  // namespace sps
