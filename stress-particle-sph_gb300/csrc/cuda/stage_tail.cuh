// stage_tail.cuh -- per-particle FP64 work shared by the plain and the FP32 forms.
//
// Normal_BCs for one particle, and the tails of get_derivatives / RK4 that follow the
// neighbour sums (2_SPH_main_2018.f90:596-648 and :727-777 of the Drucker-Prager example):
// CSPM correction, D : grad(v), plastic_terms / drucker_prager, Jaumann spin, gravity with
// damping, right-hand sides and RK4 accumulation.  In the plain form (compiled with
// -fmad=false) these reproduce the reference's rounding exactly.
#pragma once
#include "common.cuh"
#include "mlp.cuh"

namespace sps {

// BCs (3_SPH_material_2018.f90:1640-1660) for one particle: Normal_BCs (:1665-1770), then
// with ifsigman = 1 apply_stress_free (:1775-1858): a free-surface node away from the walls
// keeps only the stress component along the surface (zero normal and shear traction)
__device__ __forceinline__ void apply_bcs(const Dev& D, const StepScalars& sc, int ip, double& vx,
                                          double& vy, double& s0, double& s1, double& s2,
                                          double& s3) {
  if (D.no_bcs <= 0) return;
  const int bc = D.bc_or_not[ip];
  if (bc == 1) {
    if (D.bc_nodes_only && ip >= D.NN) return;  // Normal_BCs over 1..nnode
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
  } else if (D.ifsigman == 1 && bc == 2 && ip < D.NN && D.bc_int[ip] != 1) {
    const double costh = D.nrmx[ip], sinth = D.nrmy[ip];
    if (isnan(costh) || isnan(sinth)) return;
    const double s2_ = sinth * sinth, c2 = costh * costh, sc_ = sinth * costh;
    const double stt = (s2_ * s0 - (2.0 * sc_) * s2) + c2 * s1;
    s0 = s2_ * stt;
    s1 = c2 * stt;
    s2 = -(sc_ * stt);
    s3 = c2 * stt;
  }
}


// training capture: the exact flow rule's inputs and its plastic source Gs, scaled
__device__ __forceinline__ void capture_tuple(const Dev& D, int t, const double* s2v,
                                              const double* g, const double* Gs) {
  float x[16];
  const Real& M = real_of(D, t);
  double scale = mlp_features(s2v, g, M.tanfi, M.coh, M.young, M.poiss, D.rho[t], x);
  if (!(scale > 0.0)) return;
  unsigned long long k = atomicAdd(D.cap_cnt, 1ull);
  if ((long long)k >= D.cap_max) return;
  float* o = D.cap_buf + (size_t)k * MLP_TUPLE;
  for (int j = 0; j < MLP_NIN; j++) o[j] = x[j];
  for (int j = 0; j < MLP_NOUT; j++) o[MLP_NIN + j] = (float)(Gs[j] / scale);
}

// stress-point gradient: CSPM correction of g = grad1(a,b) (at a + 2b) with the moments AE,
// stored as grad_u
__device__ __forceinline__ void tail_sp_grad(const Dev& D, int t, double* g, const double* AE) {
    if (D.cspm) {
      double A4 = AE[0] * AE[3] - AE[1] * AE[2];
      double A0 = AE[0], A1 = AE[1], A2 = AE[2], A3 = AE[3];
      if (fabs(A4) < D.cspm_det) {
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
}

// stress-point rates after the gradient: D : grad(v), plastic_terms / drucker_prager,
// Jaumann spin, RHS and RK4 accumulation.  Gs_net (may be null): a plastic source from the
// learned surrogate that replaces the exact one (with its plastic strain rate der_net)
// FAST (the FP32 form): the mean of drucker_prager by a product, the plastic strain-rate
// norm in FP32.
// dp (FP32 form with the surrogate): drucker_prager's results for this stress-point,
// already evaluated on the same inputs by the caller: G (4), vivel (4), the updated f
template <bool FAST = false>
__device__ __forceinline__ void tail_sp_rates(const Dev& D, const StepScalars& sc, int t,
                                              const double* g, double f2,
                                              const double* Gs_net = nullptr,
                                              double der_net = 0.0,
                                              const double* dp = nullptr) {
    const Real& M = real_of(D, t);
    const double g11 = g[0], g21 = g[1], g12 = g[2], g22 = g[3];
    double div1[4];
    if (!FAST) {
      div1[0] = -(M.D11 * g11 + M.D12 * g22);
      div1[1] = -(M.D12 * g11 + M.D22 * g22);
      div1[2] = -(M.D33 * g21 + M.D33 * g12);
      div1[3] = -(M.D41 * g11 + M.D42 * g22);
    }
    // plastic_terms (3_SPH_material_2018.f90:1884-1954)
    double st[4] = {D.s0[t], D.s1[t], D.s2[t], D.s3[t]};
    double Gs[4] = {0.0, 0.0, 0.0, 0.0}, der = 0.0;
    if (M.ntype_eco > 1) {
      double s2v[4] = {st[0], st[1], st[2], st[3]};
      if (M.ntype_solid == 1) s2v[3] = M.poiss * (s2v[0] + s2v[1]);
      double vivel[4] = {0.0, 0.0, 0.0, 0.0}, G2[4];
      if (M.ncrit <= 4) {
        viscoplastic(M, s2v, D.iv1[t], vivel, Gs);
      } else if (M.ncrit == 12) {
        double f;
        if (dp) {
          for (int k = 0; k < 4; k++) {
            G2[k] = dp[k];
            vivel[k] = dp[4 + k];
          }
          f = dp[8];
        } else {
          f = D.fdp[t];
          if (FAST) drucker_prager_f32(M, sc.time_sph, s2v, g, &f, G2, vivel);
          else drucker_prager(M, sc.time_sph, s2v, g, &f, G2, vivel);
        }
        D.fdp[t] = f;
        if (FAST) {
          // negation and the non-zero test on the integer pipe (sign bit; magnitude bits)
          bool nz = false;
          for (int k = 0; k < 4; k++) {
            const long long b = __double_as_longlong(G2[k]);
            Gs[k] = __longlong_as_double(b ^ (long long)0x8000000000000000ull);
            nz = nz || (b << 1) != 0;
          }
          if (D.cap_buf && nz) capture_tuple(D, t, s2v, g, Gs);
        } else {
          for (int k = 0; k < 4; k++) Gs[k] = -G2[k];
          if (D.cap_buf && (G2[0] != 0.0 || G2[1] != 0.0 || G2[2] != 0.0 || G2[3] != 0.0))
            capture_tuple(D, t, s2v, g, Gs);
        }
      }
      if (FAST) {
        float v0 = f32_rn(vivel[0]), v1 = f32_rn(vivel[1]), v2 = f32_rn(vivel[2]),
              v3 = f32_rn(vivel[3]);
        // explicit fmaf: the same rounding in every kernel that inlines this tail
        float q = fmaf(2.0f, fmaf(v0, v0, fmaf(v1, v1, __fmul_rn(v3, v3))), __fmul_rn(v2, v2));
        der = f64_of(sqrtf(__fmul_rn(q, 1.0f / 3.0f)));
      } else {
        der = sqrt((2.0 * ((vivel[0] * vivel[0] + vivel[1] * vivel[1]) + vivel[3] * vivel[3]) +
                    vivel[2] * vivel[2]) /
                   3.0);
      }
    }
    if (Gs_net) {
      for (int k = 0; k < 4; k++) Gs[k] = Gs_net[k];
      der = der_net;
    }
    if (FAST) {
      // the FP32 form: the elastic rate, the spin and the right-hand side in FP32 (the
      // gradient comes from FP32 neighbour sums and carries their accuracy), conversions on
      // the integer pipe; only the RK accumulation stays FP64
      const float h11 = f32_rn(g11), h21 = f32_rn(g21), h12 = f32_rn(g12), h22 = f32_rn(g22);
      float r[4];
      r[0] = fmaf(M.D11f, h11, M.D12f * h22);
      r[1] = fmaf(M.D12f, h11, M.D22f * h22);
      r[2] = M.D33f * (h21 + h12);
      r[3] = fmaf(M.D41f, h11, M.D42f * h22);
      if (D.update_x) {
        const float om1 = 0.5f * (h12 - h21);
        const float t0 = f32_rn(st[0]), t1 = f32_rn(st[1]), t2 = f32_rn(st[2]);
        r[0] = fmaf(2.0f * om1, t2, r[0]);
        r[1] = fmaf(-2.0f * om1, t2, r[1]);
        r[2] = fmaf(om1, t1 - t0, r[2]);
      }
      for (int k = 0; k < 4; k++) {
        const double rhs = f64_of(r[k] + f32_rn(Gs[k]));
        D.RHS1[k][t] = rhs;
        D.RKs[k][t] = fma(f2, rhs, D.RKs[k][t]);
      }
    } else {
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
    }
    D.RKd[t] = D.RKd[t] + der * f2;
    if (D.cont_density) {
      D.RKr[t] = D.RKr[t] + f2 * D.RHSr[t];
      if (D.sle == 2) D.RKh[t] = D.RKh[t] + f2 * D.RHSh[t];
    }
}

// stress-point tail: g = grad1(a,b) at a + 2b, AE = CSPM moments (used when cspm)
__device__ __forceinline__ void tail_sp(const Dev& D, const StepScalars& sc, int t, double* g,
                                        double* AE, double f2) {
  tail_sp_grad(D, t, g, AE);
  tail_sp_rates(D, sc, t, g, f2);
}

// artificial_force (2_SPH_main_2018.f90:908-1016) on node t (sorted slot s): the node-node
// pairs in the reference's walk order, h = (dW f^n) (R_t + R_u) with f = W / W(dx, 1.2 dx)
// and n = 2.55, dW taken w.r.t. t (so t's side of the pair gets + m_u h as pair_i and
// - m_u h as pair_j, the same numbers); art_force = (T11 + T32, T31 + T22).
__device__ __forceinline__ void art_force_node(const Dev& D, int col, int t, double* afx,
                                               double* afy) {
  const Real& M = real_of(D, t);
  double w2, g0, g1;
  sph_kernel(D.skf, D.pi, M.dx, M.dx, M.dx, (double)1.2f * M.dx, &w2, &g0, &g1);
  const double n = (double)2.55f;
  const double Rt[3] = {D.artR[t], D.artR[D.NN + t], D.artR[2 * (size_t)D.NN + t]};
  double T[3][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
  const int degs = D.degS[col];
  for (int k = 0; k < degs; k++) {
    const int4 e = D.same[ell(k, col, D.N2)];
    const int u = e.x;
    const double fn = pow((double)__int_as_float(e.y) / w2, n);
    const double mu = D.mass[u];
    const double gx = (double)__int_as_float(e.z), gy = (double)__int_as_float(e.w);
    for (int q = 0; q < 3; q++) {
      const double r = Rt[q] + D.artR[(size_t)q * D.NN + u];
      T[q][0] = T[q][0] + mu * ((gx * fn) * r);
      T[q][1] = T[q][1] + mu * ((gy * fn) * r);
    }
  }
  *afx = T[0][0] + T[2][1];
  *afy = T[2][0] + T[1][1];
}

// node tail: g2 = grad2(s,b) at s + 3b, AE = CSPM moments, av = artificial viscosity,
// af = artificial force
__device__ __forceinline__ void tail_node(const Dev& D, const StepScalars& sc, int t, double* g2,
                                          double* AE, int bc_int, double avx, double avy,
                                          double f2, double afx = 0.0, double afy = 0.0) {
  D.bc_int[t] = bc_int;
  if (D.cspm) {
    double A4 = AE[0] * AE[3] - AE[1] * AE[2];
    double A0 = AE[0], A1 = AE[1], A2 = AE[2], A3 = AE[3];
    if (fabs(A4) < D.cspm_det) {
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
  const Real& M = real_of(D, t);
  double div2x = -(g2[0] + g2[2 + 3]);
  double div2y = -(g2[2] + g2[1 + 3]);
  const double vtx = D.vx[t], vty = D.vy[t];
  double gx = (M.ic_grav == 1) ? sc.factg * M.cgrav[0] : 0.0;
  double gy = (M.ic_grav == 1) ? sc.factg * M.cgrav[1] : 0.0;
  gx = gx - M.damping * vtx;
  gy = gy - M.damping * vty;
  double rhsx = (((-div2x + gx) + avx) + D.fbx[t]) + afx;
  double rhsy = (((-div2y + gy) + avy) + D.fby[t]) + afy;
  D.RHS2[0][t] = rhsx;
  D.RHS2[1][t] = rhsy;
  D.RKv[0][t] = D.RKv[0][t] + f2 * rhsx;
  D.RKv[1][t] = D.RKv[1][t] + f2 * rhsy;
}

}  // namespace sps
