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

namespace sps {

namespace {

constexpr int kBlock = 256;

// Normal_BCs (3_SPH_material_2018.f90:1665-1770) for one particle
__device__ __forceinline__ void apply_bcs(const Dev& D, const StepScalars& sc, int ip, double& vx,
                                          double& vy, double& s0, double& s1, double& s2) {
  if (D.no_bcs <= 0) return;
  if (D.bc_or_not[ip] != 1) return;
  const int32_t* bi = D.bc_info + 8 * (size_t)ip;
  if (bi[1] == 0) return;
  for (int r = 0; r < 5; r++) {
    int bt = bi[r + 2];
    if (bt == 0) continue;
    double val = sc.bcval[bt - 1];
    int var = D.bcvar[bt - 1];
    if (var == 5) vx = val;
    else if (var == 6) vy = val;
    else if (var == 1) s0 = val;
    else if (var == 3) s2 = val;
    else if (var == 2) s1 = val;
  }
}

__global__ void k_load_scalars(Dev D) {
  int k = *D.step_idx;
  *D.cur = D.scal_table[k];
}

__global__ void k_next_step(Dev D) { *D.step_idx += 1; }

__global__ void k_step_init(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  D.x0x[i] = D.px[i];
  D.x0y[i] = D.py[i];
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
__device__ __forceinline__ bool bound_term(const Dev& D, int i, int j, float& fx, float& fy) {
  const float cc = 20.0f;
  const float d0 = (float)(D.dx / 2.0);
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

__global__ void k_bound(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NN) return;
  constexpr int K = 8;
  int ids[K];
  float tx[K], ty[K];
  int n = 0;
  const int j0 = D.NT, j1 = D.NT + D.ndummy2;
  if (D.bound_from_lists) {
    int s = D.spos[i];
    int deg = D.degC[s];
    for (int k = 0; k < deg; k++) {
      int u = D.cross[(size_t)k * D.N2 + s].x;
      if (u < j0 || u >= j1) continue;
      float fx, fy;
      if (!bound_term(D, i, u, fx, fy)) continue;
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
    double bx = 0.0, by = 0.0;
    for (int k = 0; k < n; k++) {
      bx = bx + (double)tx[k];
      by = by + (double)ty[k];
    }
    D.fbx[i] = bx;
    D.fby[i] = by;
  } else {
    double bx = 0.0, by = 0.0;
    for (int j = j0; j < j1; j++) {
      float fx, fy;
      if (!bound_term(D, i, j, fx, fy)) continue;
      bx = bx + (double)fx;
      by = by + (double)fy;
    }
    D.fbx[i] = bx;
    D.fby[i] = by;
  }
}

__global__ void k_stage_begin(Dev D, int stage) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  const double f1rk[4] = {0.0, 0.5, 0.5, 1.0};
  const double f1dt = f1rk[stage] * D.dt;
  const StepScalars& sc = *D.cur;
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
      if (D.sle == 2) {
        double rh = -(D.hsml0[i] / (rho * 2.0)) * rr;
        D.RHSh[i] = rh;
        D.hsml[i] = D.hsml0[i] + f1dt * rh;
      }
    }
  }
  if (D.ncrit == 12) adapt_stress(D.alpha2, D.kc, a, b, c, d);
  apply_bcs(D, sc, i, vx, vy, a, b, c);
  D.vx[i] = vx;
  D.vy[i] = vy;
  D.s0[i] = a;
  D.s1[i] = b;
  D.s2[i] = c;
  D.s3[i] = d;
}

// stress_point_update (2_SPH_main_2018.f90:403-482) as a gather per target
__global__ void k_interp(Dev D) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  int t = D.sorted[s];
  int tt = D.itype[t];
  if (t >= D.NT) return;
  if (!D.sp_sph) {
    if (t >= D.NN) {
      int n = t - D.NN;
      D.vx[t] = D.vx[n];
      D.vy[t] = D.vy[n];
    } else {
      int sp = t + D.NN;
      D.s0[t] = D.s0[sp];
      D.s1[t] = D.s1[sp];
      D.s2[t] = D.s2[sp];
      D.s3[t] = D.s3[sp];
      D.iv1[t] = D.iv1[sp];
      if (D.cont_density) D.rho0[t] = D.rho[sp];
    }
    return;
  }
  int deg = D.degC[s];
  if (is_sp(tt)) {
    double v0 = 0.0, v1 = 0.0, norm = 0.0;
    for (int k = 0; k < deg; k++) {
      int4 e = D.cross[(size_t)k * D.N2 + s];
      int u = e.x;
      if (D.itype[u] != 2) continue;
      double w = (double)__int_as_float(e.y);
      double mu = D.mass[u], ru = D.rho[u];
      double h2 = (mu / ru) * w;
      v0 = v0 + D.vx[u] * h2;
      v1 = v1 + D.vy[u] * h2;
      norm = norm + (w * mu) / ru;
    }
    if (norm != 0) {
      D.vx[t] = v0 / norm;
      D.vy[t] = v1 / norm;
    }
  } else {
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0, iv = 0.0, rt = 0.0, norm = 0.0;
    for (int k = 0; k < deg; k++) {
      int4 e = D.cross[(size_t)k * D.N2 + s];
      int u = e.x;
      if (D.itype[u] != 1) continue;
      double w = (double)__int_as_float(e.y);
      double mu = D.mass[u], ru = D.rho[u];
      double h1 = (mu / ru) * w;
      a = a + D.s0[u] * h1;
      b = b + D.s1[u] * h1;
      c = c + D.s2[u] * h1;
      d = d + D.s3[u] * h1;
      iv = iv + D.iv1[u] * h1;
      if (D.cont_density) rt = rt + ru * h1;
      norm = norm + (w * mu) / ru;
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

__global__ void k_node_rho(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < D.NN) D.rho[i] = D.rho0[i];
}

__global__ void k_adapt_bc(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  const StepScalars& sc = *D.cur;
  double vx = D.vx[i], vy = D.vy[i];
  double a = D.s0[i], b = D.s1[i], c = D.s2[i], d = D.s3[i];
  if (D.ncrit == 12) adapt_stress(D.alpha2, D.kc, a, b, c, d);
  apply_bcs(D, sc, i, vx, vy, a, b, c);
  D.vx[i] = vx;
  D.vy[i] = vy;
  D.s0[i] = a;
  D.s1[i] = b;
  D.s2[i] = c;
  D.s3[i] = d;
}

// get_derivatives (2_SPH_main_2018.f90:487-648) + the per-particle stage work of RK4
__global__ void k_derivs(Dev D, int stage) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  int t = D.sorted[s];
  if (t >= D.NT) return;
  const double f2rk[4] = {1.0, 2.0, 2.0, 1.0};
  const double f2 = f2rk[stage];
  const StepScalars& sc = *D.cur;
  int tt = D.itype[t];
  int deg = D.degC[s];
  double AE[4] = {0.0, 0.0, 0.0, 0.0};
  const double xt = D.px[t], yt = D.py[t];
  if (is_sp(tt)) {
    double g[4] = {0.0, 0.0, 0.0, 0.0};  // grad1(a,b) at a + 2b
    const double vt[2] = {D.vx[t], D.vy[t]};
    for (int k = 0; k < deg; k++) {
      int4 e = D.cross[(size_t)k * D.N2 + s];
      int u = e.x;
      int ut = D.itype[u];
      double Gx = (double)__int_as_float(e.z), Gy = (double)__int_as_float(e.w);
      double mu = D.mass[u], ru = D.rho[u];
      if (ut == 2) {  // node -- stress-point (target is pair_i)
        double h1 = (Gx * mu) / ru;
        double h2 = (Gy * mu) / ru;
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
      } else if (ut == 25) {  // stress-point -- dummy (dummy is pair_i)
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
        double hh1 = (-Gx * mu) / ru;
        double hh2 = (-Gy * mu) / ru;
        g[0] = g[0] + (vt[0] - dv0) * hh1;
        g[2] = g[2] + (vt[0] - dv0) * hh2;
        g[1] = g[1] + (vt[1] - dv1) * hh1;
        g[3] = g[3] + (vt[1] - dv1) * hh2;
      }
    }
    if (D.cspm) {
      double A4 = AE[0] * AE[3] - AE[1] * AE[2];
      double A0 = AE[0], A1 = AE[1], A2 = AE[2], A3 = AE[3];
      if (fabs(A4) < (double)1e-07f) {
        A4 = 1;
        A0 = 1;
        A1 = 0;
        A2 = 0;
        A3 = 1;
      } else {
        A4 = 1.0 / A4;
      }
      for (int d = 0; d < 2; d++) {
        g[d] = A4 * (A0 * g[d] + A1 * g[d + 2]);
        g[d + 2] = A4 * (A2 * g[d] + A3 * g[d + 2]);
      }
    }
    double* gu = D.grad_u + 4 * (size_t)t;
    gu[0] = g[0];
    gu[1] = g[1];
    gu[2] = g[2];
    gu[3] = g[3];
    const double g11 = g[0], g21 = g[1], g12 = g[2], g22 = g[3];
    double div1[4];
    div1[0] = -(D.D11 * g11 + D.D12 * g22);
    div1[1] = -(D.D12 * g11 + D.D22 * g22);
    div1[2] = -(D.D33 * g21 + D.D33 * g12);
    div1[3] = -(D.D41 * g11 + D.D42 * g22);
    // plastic_terms (3_SPH_material_2018.f90:1884-1954)
    double st[4] = {D.s0[t], D.s1[t], D.s2[t], D.s3[t]};
    double Gs[4] = {0.0, 0.0, 0.0, 0.0}, der = 0.0;
    if (D.ntype_eco > 1) {
      double s2v[4] = {st[0], st[1], st[2], st[3]};
      if (D.ntype_solid == 1) s2v[3] = D.poiss * (s2v[0] + s2v[1]);
      double vivel[4] = {0.0, 0.0, 0.0, 0.0}, G2[4];
      if (D.ncrit == 12) {
        double f = D.fdp[t];
        drucker_prager(D, sc.time_sph, s2v, g, &f, G2, vivel);
        D.fdp[t] = f;
        for (int k = 0; k < 4; k++) Gs[k] = -G2[k];
      }
      der = sqrt((2.0 * ((vivel[0] * vivel[0] + vivel[1] * vivel[1]) + vivel[3] * vivel[3]) +
                  vivel[2] * vivel[2]) /
                 3.0);
    }
    double spin[4] = {0.0, 0.0, 0.0, 0.0};
    if (D.update_x) {
      double om1 = 0.5 * (g12 - g21);
      double om2 = -0.5 * (g12 - g21);
      spin[0] = 2.0 * om1 * st[2];
      spin[1] = 2.0 * om2 * st[2];
      spin[2] = om2 * st[0] + om1 * st[1];
    }
    for (int k = 0; k < 4; k++) {
      double rhs = (-div1[k] + spin[k]) + Gs[k];
      D.RHS1[k][t] = rhs;
      D.RKs[k][t] = D.RKs[k][t] + f2 * rhs;
    }
    D.RKd[t] = D.RKd[t] + der * f2;
    if (D.cont_density) {
      D.RKr[t] = D.RKr[t] + f2 * D.RHSr[t];
      if (D.sle == 2) D.RKh[t] = D.RKh[t] + f2 * D.RHSh[t];
    }
  } else if (is_node(tt)) {
    double g2[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};  // grad2(s,b) at s + 3b
    const double rt = D.rho[t];
    const double rt2 = rt * rt;
    const double at[3] = {D.s0[t] / rt2, D.s1[t] / rt2, D.s2[t] / rt2};
    const double stt[3] = {D.s0[t], D.s1[t], D.s2[t]};
    int bc_int = 0;
    for (int k = 0; k < deg; k++) {
      int4 e = D.cross[(size_t)k * D.N2 + s];
      int u = e.x;
      int ut = D.itype[u];
      double dwx = -(double)__int_as_float(e.z), dwy = -(double)__int_as_float(e.w);
      double mu = D.mass[u], ru = D.rho[u];
      double ru2 = ru * ru;
      if (ut == 1) {  // node -- stress-point (stress-point is pair_i)
        const double su[3] = {D.s0[u], D.s1[u], D.s2[u]};
        for (int q = 0; q < 3; q++) {
          double sum = at[q] + su[q] / ru2;
          g2[q] = g2[q] - mu * (dwx * sum);
          g2[q + 3] = g2[q + 3] - mu * (dwy * sum);
        }
        if (D.cspm) {
          double h1b = -((dwx * mu) / ru);
          double h2b = -((dwy * mu) / ru);
          double xu = D.px[u] - xt, yu = D.py[u] - yt;
          AE[0] = AE[0] + xu * h1b;
          AE[1] = AE[1] + yu * h1b;
          AE[2] = AE[2] + xu * h2b;
          AE[3] = AE[3] + yu * h2b;
        }
      } else if (ut == 25) {  // node -- dummy: the dummy carries the node's stress
        bc_int = 1;
        for (int q = 0; q < 3; q++) {
          double sum = at[q] + stt[q] / ru2;
          g2[q] = g2[q] - mu * (dwx * sum);
          g2[q + 3] = g2[q + 3] - mu * (dwy * sum);
        }
      }
    }
    D.bc_int[t] = bc_int;
    if (D.cspm) {
      double A4 = AE[0] * AE[3] - AE[1] * AE[2];
      double A0 = AE[0], A1 = AE[1], A2 = AE[2], A3 = AE[3];
      if (fabs(A4) < (double)1e-07f) {
        A4 = 1;
        A0 = 1;
        A1 = 0;
        A2 = 0;
        A3 = 1;
      } else {
        A4 = 1.0 / A4;
      }
      for (int d = 0; d < 2; d++) {
        g2[d] = A4 * (A0 * g2[d] + A1 * g2[d + 3]);
        g2[d + 3] = A4 * (A2 * g2[d] + A3 * g2[d + 3]);
      }
    }
    double div2x = -(g2[0] + g2[2 + 3]);
    double div2y = -(g2[2] + g2[1 + 3]);
    const double vtx = D.vx[t], vty = D.vy[t];
    double gx = (D.ic_grav == 1) ? sc.factg * D.cgrav[0] : 0.0;
    double gy = (D.ic_grav == 1) ? sc.factg * D.cgrav[1] : 0.0;
    gx = gx - D.damping * vtx;
    gy = gy - D.damping * vty;
    double avx = 0.0, avy = 0.0;
    if (D.alpha > 0 || D.beta > 0) {
      // artificial_viscosity (2_SPH_main_2018.f90:826-904): FP32 accumulators
      float ax = 0.0f, ay = 0.0f;
      int degs = D.degS[s];
      const float ht = (float)0.0;  // unused placeholder to keep types explicit
      (void)ht;
      for (int k = 0; k < degs; k++) {
        int4 e = D.same[(size_t)k * D.N2 + s];
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
          visc = (float)((-((D.alpha * 600.0) * (double)theta) + D.beta * (double)(theta * theta)) /
                         (double)rho2);
        float px = visc * __int_as_float(e.z), py = visc * __int_as_float(e.w);
        double mu = D.mass[u];
        ax = (float)((double)ax + (double)px * mu);
        ay = (float)((double)ay + (double)py * mu);
      }
      avx = -(double)ax;
      avy = -(double)ay;
    }
    double rhsx = (((-div2x + gx) + avx) + D.fbx[t]) + 0.0;
    double rhsy = (((-div2y + gy) + avy) + D.fby[t]) + 0.0;
    D.RHS2[0][t] = rhsx;
    D.RHS2[1][t] = rhsy;
    D.RKv[0][t] = D.RKv[0][t] + f2 * rhsx;
    D.RKv[1][t] = D.RKv[1][t] + f2 * rhsy;
  }
}

__global__ void k_rk_final(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  const StepScalars& sc = *D.cur;
  const double dt6 = D.dt / 6.0;
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
  if (D.ncrit == 12) adapt_stress(D.alpha2, D.kc, a, b, c, d);
  apply_bcs(D, sc, i, vx, vy, a, b, c);
  D.vx[i] = vx;
  D.vy[i] = vy;
  D.s0[i] = a;
  D.s1[i] = b;
  D.s2[i] = c;
  D.s3[i] = d;
  if (i >= D.NN) {
    if (D.cont_density) {
      D.rho[i] = D.rho0[i] + dt6 * D.RKr[i];
      if (D.sle == 2) D.hsml[i] = D.hsml0[i] + dt6 * D.RKh[i];
    }
    double dd = D.RKd[i] / 6.0;
    D.Ddev[i] = dd;
    D.iv1[i] = D.iv1[i] + D.dt * dd;  // update_strain (3_SPH_material_2018.f90:1864)
  }
}

__global__ void k_trapezoid(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NT) return;
  if (D.update_x) {
    float hx = (float)(0.5 * (D.vx0[i] + D.vx[i]));
    float hy = (float)(0.5 * (D.vy0[i] + D.vy[i]));
    double x = D.x0x[i] + (double)hx * D.dt;
    double y = D.x0y[i] + (double)hy * D.dt;
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
  int deg = D.degS[s];
  const double vt0 = D.vx[t], vt1 = D.vy[t];
  double s0 = 0.0, s1 = 0.0;
  int flag = D.bc_or_not[t];
  bool mark = false;
  for (int k = 0; k < deg; k++) {
    int4 e = D.same[(size_t)k * D.N2 + s];
    int u = e.x;
    double w = (double)__int_as_float(e.y);
    double vol = D.mass[u] / D.rho[u];
    s0 = s0 + (vol * (D.vx[u] - vt0)) * w;
    s1 = s1 + (vol * (D.vy[u] - vt1)) * w;
    if (t < D.NN && D.bc_or_not[u] == 2 && flag != 2) mark = true;
  }
  const double eps = 0.5;
  D.px[t] = D.x0x[t] + D.dt * (vt0 + eps * s0);
  D.py[t] = D.x0y[t] + D.dt * (vt1 + eps * s1);
  if (mark) D.bc_or_not[t] = 3;
}

__global__ void k_displ(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.NN) return;
  if (D.update_x) {
    if (!D.sp_sph) {
      D.px[D.NN + i] = D.px[i];
      D.py[D.NN + i] = D.py[i];
    }
    D.dispx[i] = D.px[i] - D.x00x[i];
    D.dispy[i] = D.py[i] - D.x00y[i];
  } else {
    D.dispx[i] = D.dispx[i] + (0.5 * (D.vx0[i] + D.vx[i])) * D.dt;
    D.dispy[i] = D.dispy[i] + (0.5 * (D.vy0[i] + D.vy[i])) * D.dt;
  }
}

}  // namespace

int launch_plain_step(Ctx& c) {
  Dev& D = c.d;
  cudaStream_t st = c.stream;
  int nbT = (D.NT + kBlock - 1) / kBlock;
  int nbN = (D.NN + kBlock - 1) / kBlock;
  int nb2 = (D.N2 + kBlock - 1) / kBlock;
  c.mark("load_scalars");
  k_load_scalars<<<1, 1, 0, st>>>(D);
  launch_pair_build(c);
  c.mark("step_init");
  k_step_init<<<nbT, kBlock, 0, st>>>(D);
  if (D.inside) {
    c.mark("bound");
    k_bound<<<nbN, kBlock, 0, st>>>(D);
  }
  for (int stage = 0; stage < 4; stage++) {
    c.mark("stage_begin");
    k_stage_begin<<<nbT, kBlock, 0, st>>>(D, stage);
    c.mark("interp");
    k_interp<<<nb2, kBlock, 0, st>>>(D);
    if (D.cont_density && D.sp_sph) {
      c.mark("node_rho");
      k_node_rho<<<nbN, kBlock, 0, st>>>(D);
    }
    if (D.sp_sph) {
      c.mark("adapt_bc");
      k_adapt_bc<<<nbT, kBlock, 0, st>>>(D);
    }
    c.mark("derivs");
    k_derivs<<<nb2, kBlock, 0, st>>>(D, stage);
  }
  c.mark("rk_final");
  k_rk_final<<<nbT, kBlock, 0, st>>>(D);
  c.mark("interp");
  k_interp<<<nb2, kBlock, 0, st>>>(D);
  if (D.cont_density && D.sp_sph) {
    c.mark("node_rho");
    k_node_rho<<<nbN, kBlock, 0, st>>>(D);
  }
  if (D.sp_sph) {
    c.mark("adapt_bc");
    k_adapt_bc<<<nbT, kBlock, 0, st>>>(D);
  }
  if (D.update_x && D.xsph) {
    c.mark("xsph");
    k_xsph<<<nb2, kBlock, 0, st>>>(D);
  } else {
    c.mark("trapezoid");
    k_trapezoid<<<nbT, kBlock, 0, st>>>(D);
  }
  c.mark("displ");
  k_displ<<<nbN, kBlock, 0, st>>>(D);
  c.mark("next_step");
  k_next_step<<<1, 1, 0, st>>>(D);
  return 0;
}

}  // namespace sps
