// fast_step.cu -- neighbour sums of the FP32 form of the SPS step.
//
// The FP32 form keeps the particle state, the RK4 update and the stress return in FP64
// (per-particle work, shared with the plain form through stage_tail.cuh) and moves the
// neighbour sums -- the O(N x neighbours) part -- to FP32:
//   * neighbours are read from packed FP32 records written by the per-particle kernels
//     (recV: velocity as double-float hi/lo pairs, recS: stress, recI {intvar1, m/rho, rho,
//     m}, recA / recAl: sigma/rho^2 as double-float pairs and m), 16 bytes per field set;
//   * every sum is Kahan-compensated (Kahan, "Further remarks on reducing truncation
//     errors", CACM 8(1), 1965), so its error stays at a few FP32 ulps of the result
//     regardless of the neighbour count;
//   * differences of nearly equal neighbour values (velocities, sigma/rho^2) are taken in
//     double-float, and the near-cancelling sums are rearranged so that their terms are
//     small (see k_finterp and k_fderivs);
//   * the quotients (G m)/rho and (w m)/rho of the reference are formed as G (m/rho).
// The pair set is the same exact set as the plain form's; kernel values are evaluated in
// FP32 (k_half<true>).
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <string>

#include "ctx.cuh"
#include "stage_tail.cuh"

namespace sps {

namespace {

struct Kahan {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double val() const { return (double)s - (double)c; }
  // the compensated sum rounded to FP32
  __device__ __forceinline__ float fval() const { return s - c; }
};

// sum of exact FP32 products: p = RN(a b) and e = a b - p (exact, by one FMA: the
// error-free product transformation of Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26(6), 2005); p is Kahan-summed, e summed plainly
struct ProdSum {
  Kahan hi;
  float lo = 0.0f;
  __device__ __forceinline__ void add(float a, float b) {
    float p = a * b;
    float e = fmaf(a, b, -p);
    hi.add(p);
    lo += e;
  }
};

// difference of two double-float values (hi + lo) in FP32
__device__ __forceinline__ float dfdiff(float ah, float al, float bh, float bl) {
  return (ah - bh) + (al - bl);
}

// The node tail of get_derivatives / RK4 (tail_node without CSPM) in FP32: the divergence,
// gravity with damping and the right-hand side carry the FP32 accuracy of the sums they
// come from; only the RK4 accumulation of the FP64 state is FP64 (one fused multiply-add
// per component, exact in its product since f2 is 1 or 2).
__device__ __forceinline__ void tail_node_f32(const Dev& D, const StepScalars& sc, const Real& M,
                                              int t, const float* g2, int bc_int, float avx,
                                              float avy, double f2, double afx, double afy) {
  D.bc_int[t] = bc_int;
  const float div2x = -(g2[0] + g2[5]);
  const float div2y = -(g2[2] + g2[4]);
  float gx = 0.0f, gy = 0.0f;
  if (M.ic_grav == 1) {
    const float fg = f32_rn(sc.factg);
    gx = fg * f32_rn(M.cgrav[0]);
    gy = fg * f32_rn(M.cgrav[1]);
  }
  if ((__double_as_longlong(M.damping) << 1) != 0) {  // non-zero, on the integer pipe
    const float dmp = f32_rn(M.damping);
    gx = fmaf(-dmp, f32_rn(D.vx[t]), gx);
    gy = fmaf(-dmp, f32_rn(D.vy[t]), gy);
  }
  float rhsx = ((-div2x + gx) + avx) + f32_rn(D.fbx[t]);
  float rhsy = ((-div2y + gy) + avy) + f32_rn(D.fby[t]);
  if (D.art_stress) {
    rhsx += f32_rn(afx);
    rhsy += f32_rn(afy);
  }
  const double rx = f64_of(rhsx), ry = f64_of(rhsy);
  D.RHS2[0][t] = rx;
  D.RHS2[1][t] = ry;
  D.RKv[0][t] = fma(f2, rx, D.RKv[0][t]);
  D.RKv[1][t] = fma(f2, ry, D.RKv[1][t]);
}

// Walks entries 0 .. deg of list column col, KP entries a pass, software-pipelined: the
// next pass's entries are loaded while the current pass's records are gathered and summed,
// so that the entry loads (streamed from DRAM) overlap the record gathers (mostly L2 hits)
// instead of adding their latency to them.  load(e) returns the records of entry e (called
// only for entries below deg), sum(e, rec) adds one term; terms are added in list order,
// so the result does not depend on KP.
template <int KP, typename Rec, typename Load, typename Sum>
__device__ __forceinline__ void walk_list(const int4* __restrict__ list, int col, int N2,
                                          int deg, Load&& load, Sum&& sum) {
  int4 nxt[KP];
#pragma unroll
  for (int q = 0; q < KP; q++)
    nxt[q] = q < deg ? list[ell(q, col, N2)] : make_int4(0, 0, 0, 0);
  for (int k = 0; k < deg; k += KP) {
    int4 cur[KP];
    Rec rec[KP] = {};
#pragma unroll
    for (int q = 0; q < KP; q++) {
      cur[q] = nxt[q];
      if (k + q < deg) rec[q] = load(cur[q]);
    }
#pragma unroll
    for (int q = 0; q < KP; q++)
      nxt[q] = k + KP + q < deg ? list[ell(k + KP + q, col, N2)] : make_int4(0, 0, 0, 0);
#pragma unroll
    for (int q = 0; q < KP; q++)
      if (k + q < deg) sum(cur[q], rec[q]);
  }
}

// the same walk over the compact {id, W} entries (crossW: entry k of column col at
// k * N2 + col)
template <int KP, typename Rec, typename Load, typename Sum>
__device__ __forceinline__ void walk_compact(const int2* __restrict__ list, int col, int N2,
                                             int deg, Load&& load, Sum&& sum) {
  int2 nxt[KP];
#pragma unroll
  for (int q = 0; q < KP; q++) nxt[q] = q < deg ? list[(size_t)q * N2 + col] : make_int2(0, 0);
  for (int k = 0; k < deg; k += KP) {
    int2 cur[KP];
    Rec rec[KP] = {};
#pragma unroll
    for (int q = 0; q < KP; q++) {
      cur[q] = nxt[q];
      if (k + q < deg) rec[q] = load(cur[q]);
    }
#pragma unroll
    for (int q = 0; q < KP; q++)
      nxt[q] = k + KP + q < deg ? list[(size_t)(k + KP + q) * N2 + col] : make_int2(0, 0);
#pragma unroll
    for (int q = 0; q < KP; q++)
      if (k + q < deg) sum(cur[q], rec[q]);
  }
}

// records of one neighbour, as the four sums read them
struct RecVI {  // velocity (hi, lo) and m / rho
  float4 v;
  float vol;
};
struct RecSI {  // stress and {intvar1, m / rho, rho, m}
  float4 s, i;
};
struct RecA {  // sigma / rho^2 (hi with m, lo)
  float4 a, l;
};

// stress_point_update (2_SPH_main_2018.f90:403-482), FP32 sums.  A stress-point's velocity
// is the weighted mean of its nodes' velocities; it is formed as the first node's velocity
// plus the weighted mean of the deviations, which are small and exact in double-float.
// KIND 0: every particle (sorted positions); 1: the stress-point targets tgt[0..n); 2: the
// node targets (no divergence between the two branches inside a warp)
// KP: neighbours a pass whose entries and records are loaded before any is summed (the
// autotuner's look-ahead; the sum order, and so the result, does not depend on it)
template <int KIND, int KP>
__global__ void k_finterp(Dev D, const int32_t* __restrict__ tgt, int ntgt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  int s;
  if (KIND == 0) {
    s = k;
    if (s >= D.N2) return;
  } else {
    if (k >= ntgt) return;
    s = tgt[k];
  }
  int t = D.sorted[s];
  if (t >= D.NT) return;
  int tt = D.itype[t];
  if (!D.sp_sph) {
    const Real& M = real_of(D, t);
    if (t >= D.NN) {
      D.vx[t] = D.vx[node_of_sp(M, t)];
      D.vy[t] = D.vy[node_of_sp(M, t)];
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
  const int col = list_col<KIND>(D, k, s);
  int deg = D.degC[col];
  if (KIND != 0 && (D.l2_prefetch & 1)) prefetch_list_l2(D.cross, col, deg, D.N2);
  if (KIND == 1 || (KIND == 0 && is_sp(tt))) {
    Kahan v0, v1, nm;
    bool have = false;
    float4 ref = make_float4(0.f, 0.f, 0.f, 0.f);
    auto term = [&](float w, float4 r, float vol) {
      if (!have) {
        ref = r;
        have = true;
      }
      float h2 = vol * w;
      v0.add(dfdiff(r.x, r.z, ref.x, ref.z) * h2);
      v1.add(dfdiff(r.y, r.w, ref.y, ref.w) * h2);
      nm.add(h2);
    };
    auto load = [&](const auto& e) {
      RecVI r = {make_float4(0.f, 0.f, 0.f, 0.f), 0.f};
      if (e.y >= 0) {  // not a dummy partner
        r.v = D.recV[e.x];
        r.vol = D.recI[e.x].y;
      }
      return r;
    };
    auto sum = [&](const auto& e, const RecVI& r) {
      if (e.y >= 0) term(__int_as_float(e.y), r.v, r.vol);
    };
    // the compact {id, W} entries when the lists were gathered (half the bytes)
    if (KIND != 0 && D.use_crossW) walk_compact<KP, RecVI>(D.crossW, col, D.N2, deg, load, sum);
    else walk_list<KP, RecVI>(D.cross, col, D.N2, deg, load, sum);
    // the mean deviation in FP32 (its sums carry FP32 accuracy), added to the first
    // node's velocity (hi + lo, exact in FP64): two FP64 additions per target
    const float norm = nm.fval();
    if (norm != 0.0f) {
      const float rn = __frcp_rn(norm);
      D.vx[t] = (f64_of(ref.x) + f64_of(ref.z)) + f64_of(v0.fval() * rn);
      D.vy[t] = (f64_of(ref.y) + f64_of(ref.w)) + f64_of(v1.fval() * rn);
    }
  } else {
    Kahan a, b, c, d, iv, rt, nm;
    auto term = [&](float w, float4 rs, float4 ri) {
      float h1 = ri.y * w;
      a.add(rs.x * h1);
      b.add(rs.y * h1);
      c.add(rs.z * h1);
      d.add(rs.w * h1);
      iv.add(ri.x * h1);
      if (D.cont_density) rt.add(ri.z * h1);
      nm.add(h1);
    };
    auto load = [&](const auto& e) {
      RecSI r = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
      if (e.y >= 0) {
        r.s = D.recS[e.x];
        r.i = D.recI[e.x];
      }
      return r;
    };
    auto sum = [&](const auto& e, const RecSI& r) {
      if (e.y >= 0) term(__int_as_float(e.y), r.s, r.i);
    };
    if (KIND != 0 && D.use_crossW) walk_compact<KP, RecSI>(D.crossW, col, D.N2, deg, load, sum);
    else walk_list<KP, RecSI>(D.cross, col, D.N2, deg, load, sum);
    // the weighted means in FP32 (no FP64 arithmetic): the sums carry FP32 accuracy
    const float norm = nm.fval();
    if (norm != 0.0f) {
      const float rn = __frcp_rn(norm);
      D.s0[t] = f64_of(a.fval() * rn);
      D.s1[t] = f64_of(b.fval() * rn);
      D.s2[t] = f64_of(c.fval() * rn);
      D.s3[t] = f64_of(d.fval() * rn);
      D.iv1[t] = f64_of(iv.fval() * rn);
      if (D.cont_density) D.rho0[t] = f64_of(rt.fval() * rn);
    } else {
      D.vx[t] = 0.0;
      D.vy[t] = 0.0;
      if (D.cont_density) D.rho0[t] = rt.val() / nm.val();
    }
  }
}

// get_derivatives (2_SPH_main_2018.f90:487-648) with FP32 sums, then the FP64 tails.
// Node side: sum_u m (A_t + A_u) dW = sum_u m (A_u - A_t) dW + 2 A_t sum_u m dW, with
// A = sigma / rho^2.  The first sum has small terms (double-float differences); the second
// is a sum of exact products.  This keeps the near-cancelling stress divergence accurate.
// KIND 1: the stress-point targets tgt[0..n), 2: the node targets
// KP: neighbours a pass, loaded before any is summed (as in k_finterp)
// CSPM: the CSPM correction's moments (D.cspm), a template parameter so that the
// accumulators of the moments take no registers when it is off
template <int KIND, int KP, bool CSPM>
__global__ void __launch_bounds__(256, KIND == 1 ? 4 : 3) k_fderivs(Dev D, int stage,
                                                    const int32_t* __restrict__ tgt, int ntgt) {
  const int k0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (k0 >= ntgt) return;
  const int s = tgt[k0];
  int t = D.sorted[s];
  const double f2 = (stage == 1 || stage == 2) ? 2.0 : 1.0;  // RK4 weights 1, 2, 2, 1
  const Real& Mt = real_of(D, t);
  const StepScalars& sc = D.cur[D.R == 1 ? 0 : D.rid[t]];
  const int col = list_col<KIND>(D, k0, s);
  int deg = D.degC[col];
  if (D.l2_prefetch & 2) prefetch_list_l2(D.cross, col, deg, D.N2);
  const double xt = D.px[t], yt = D.py[t];
  if (KIND == 1) {
    Kahan g0, g1, g2, g3, e0, e1, e2, e3;
    const double vtx = D.vx[t], vty = D.vy[t];
    float vh0, vh1, vl0, vl1;
    f32_split(vtx, vh0, vl0);
    f32_split(vty, vh1, vl1);
    auto term = [&](const int4& e, float vol, float4 r) {
      const int u = e.x;
      const bool wall = e.y < 0;  // a dummy partner (sign bit of W)
      float Gx = __int_as_float(e.z), Gy = __int_as_float(e.w);
      if (!wall) {
        float h1 = Gx * vol, h2 = Gy * vol;
        float du0 = dfdiff(r.x, r.z, vh0, vl0), du1 = dfdiff(r.y, r.w, vh1, vl1);
        g0.add(du0 * h1);
        g2.add(du0 * h2);
        g1.add(du1 * h1);
        g3.add(du1 * h2);
        if (CSPM) {
          float xu = (float)(D.px[u] - xt), yu = (float)(D.py[u] - yt);
          e0.add(xu * h1);
          e1.add(yu * h1);
          e2.add(xu * h2);
          e3.add(yu * h2);
        }
      } else {
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
        float du0 = (float)(vtx - vtx * (1.0 - beta)), du1 = (float)(vty - vty * (1.0 - beta));
        float hh1 = -Gx * vol, hh2 = -Gy * vol;
        g0.add(du0 * hh1);
        g2.add(du0 * hh2);
        g1.add(du1 * hh1);
        g3.add(du1 * hh2);
      }
    };
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    walk_list<KP, RecVI>(
        D.cross, col, D.N2, deg,
        [&](const int4& e) {
          RecVI r;
          r.vol = D.recI[e.x].y;
          r.v = e.y >= 0 ? D.recV[e.x] : z;
          return r;
        },
        [&](const int4& e, const RecVI& r) { term(e, r.vol, r.v); });
    // the rates follow in k_fsp_tail
    if (CSPM) {
      double g[4] = {g0.val(), g1.val(), g2.val(), g3.val()};
      double AE[4] = {e0.val(), e1.val(), e2.val(), e3.val()};
      tail_sp_grad(D, t, g, AE);
    } else {  // grad_u rounded to FP32 (its sums' accuracy), no FP64 arithmetic
      double* gu = D.grad_u + 4 * (size_t)t;
      gu[0] = f64_of(g0.fval());
      gu[1] = f64_of(g1.fval());
      gu[2] = f64_of(g2.fval());
      gu[3] = f64_of(g3.fval());
    }
  } else {
    Kahan q0, q1, q2, q3, q4, q5, e0, e1, e2, e3;
    ProdSum sx, sy;
    const float4 ah = D.recA[t], al = D.recAl[t];
    int bc_int = 0;
    auto term = [&](int4 e, float4 ra, float4 rl) {
      const int u = e.x;
      const bool wall = e.y < 0;  // a dummy partner (sign bit of W)
      float dwx = -__int_as_float(e.z), dwy = -__int_as_float(e.w);
      float m, d0, d1, d2;
      if (!wall) {
        m = ra.w;
        d0 = dfdiff(ra.x, rl.x, ah.x, al.x);
        d1 = dfdiff(ra.y, rl.y, ah.y, al.y);
        d2 = dfdiff(ra.z, rl.z, ah.z, al.z);
        if (CSPM) {
          float vol = D.recI[u].y;
          float h1b = -(dwx * vol), h2b = -(dwy * vol);
          float xu = (float)(D.px[u] - xt), yu = (float)(D.py[u] - yt);
          e0.add(xu * h1b);
          e1.add(yu * h1b);
          e2.add(xu * h2b);
          e3.add(yu * h2b);
        }
      } else {
        // the dummy carries the node's stress: A_u = sigma_t / rho_d^2
        bc_int = 1;
        double ri = D.rinv[u];
        double ri2 = ri * ri;
        const double rt = D.rinv[t];
        const double rt2 = rt * rt;  // A_t = sigma_t (1/rho_t)^2, as k_adapt_bc forms it
        const double st0 = D.s0[t], st1 = D.s1[t], st2 = D.s2[t];
        m = (float)D.mass[u];
        d0 = (float)fma(st0, ri2, -(st0 * rt2));
        d1 = (float)fma(st1, ri2, -(st1 * rt2));
        d2 = (float)fma(st2, ri2, -(st2 * rt2));
      }
      float mx = m * dwx, my = m * dwy;
      q0.add(mx * d0);
      q1.add(mx * d1);
      q2.add(mx * d2);
      q3.add(my * d0);
      q4.add(my * d1);
      q5.add(my * d2);
      sx.add(m, dwx);
      sy.add(m, dwy);
    };
    // KP neighbours a pass, pipelined (walk_list)
    walk_list<KP, RecA>(
        D.cross, col, D.N2, deg,
        [&](const int4& e) {
          RecA r = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
          if (e.y >= 0) {
            r.a = D.recA[e.x];
            r.l = D.recAl[e.x];
          }
          return r;
        },
        [&](const int4& e, const RecA& r) { term(e, r.a, r.l); });
    float avx = 0.0f, avy = 0.0f;
    // alpha > 0 or beta > 0 (non-negative doubles: a positive one has a positive bit pattern)
    if (__double_as_longlong(Mt.alpha) > 0 || __double_as_longlong(Mt.beta) > 0) {
      // artificial_viscosity (2_SPH_main_2018.f90:826-904) in FP32
      Kahan ax, ay;
      int degs = D.degS[col];
      float vh0, vh1, vl0, vl1;
      f32_split(D.vx[t], vh0, vl0);
      f32_split(D.vy[t], vh1, vl1);
      const float ht = f32_rn(D.hsml[t]), rt = f32_rn(D.rho[t]);
      for (int k = 0; k < degs; k++) {
        int4 e = D.same[ell(k, col, D.N2)];
        int u = e.x;
        float4 r = D.recV[u];
        float4 ri = D.recI[u];
        float xij = (float)(xt - D.px[u]);
        float yij = (float)(yt - D.py[u]);
        float h = 0.5f * (ht + (float)D.hsml[u]);
        float rho2 = 0.5f * (rt + ri.z);
        float div_u = xij * dfdiff(vh0, vl0, r.x, r.z) + yij * dfdiff(vh1, vl1, r.y, r.w);
        float sq2 = xij * xij + yij * yij;
        float theta = (h * div_u) / (sq2 + 0.01f * (h * h));
        float visc = 0.0f;
        if (div_u < 0)
          visc = (-((float)Mt.alpha * 600.0f) * theta + (float)Mt.beta * (theta * theta)) / rho2;
        ax.add(visc * __int_as_float(e.z) * ri.w);
        ay.add(visc * __int_as_float(e.w) * ri.w);
      }
      avx = -ax.fval();
      avy = -ay.fval();
    }
    // g2 = -(q + 2 A_t S) in FP32: A_t (hi + lo) times S (hi + lo) as a double-float
    // product, so that the large, nearly cancelling part 2 A_t S keeps FP32 accuracy
    // relative to the result
    const float sxh = sx.hi.s, sxl = sx.lo - sx.hi.c, syh = sy.hi.s, syl = sy.lo - sy.hi.c;
    auto g2of = [](float q, float ah_, float al_, float sh, float sl) {
      const float p = ah_ * sh;
      const float e = fmaf(ah_, sl, fmaf(al_, sh, fmaf(ah_, sh, -p)));
      return -(fmaf(2.0f, p, q) + 2.0f * e);
    };
    float g2v[6];
    g2v[0] = g2of(q0.fval(), ah.x, al.x, sxh, sxl);
    g2v[1] = g2of(q1.fval(), ah.y, al.y, sxh, sxl);
    g2v[2] = g2of(q2.fval(), ah.z, al.z, sxh, sxl);
    g2v[3] = g2of(q3.fval(), ah.x, al.x, syh, syl);
    g2v[4] = g2of(q4.fval(), ah.y, al.y, syh, syl);
    g2v[5] = g2of(q5.fval(), ah.z, al.z, syh, syl);
    double afx = 0.0, afy = 0.0;
    if (D.art_stress) art_force_node(D, col, t, &afx, &afy);
    if (CSPM) {  // the CSPM correction in FP64 (the reference's form)
      double g2d[6];
      for (int q = 0; q < 6; q++) g2d[q] = f64_of(g2v[q]);
      double AE[4] = {e0.val(), e1.val(), e2.val(), e3.val()};
      tail_node(D, sc, t, g2d, AE, bc_int, f64_of(avx), f64_of(avy), f2, afx, afy);
    } else {
      tail_node_f32(D, sc, Mt, t, g2v, bc_int, avx, avy, f2, afx, afy);
    }
  }
}

// Stress-point rates of the FP32 form (after k_fderivs has stored grad_u): one thread per
// stress-point, one warp per 32 consecutive stress-points, so that the FP64 tail runs in
// its own kernel on contiguous stress-points instead of diverging against the node branch
// of k_fderivs.  With the learned surrogate installed (and its gate open for the step),
// loading stress-points whose inputs lie in the training envelope have been appended as
// rows by k_fsp_cand and run through the network by the tensor-core kernel (mlp_tc.cu); a
// prediction is kept when the yield-function drift it causes over one step,
//   r = dt |grad f : (D:e + Gs)| / sqrt(J2),  f = sqrt(J2) + alpha I1 - k_c,
// is at most surr_tol (the exact flow rule makes grad f : (D:e + Gs) = 0 up to rounding).
// Every other stress-point takes the exact flow rule.
// The stress-point tail of the FP32 form without the network, for the Drucker-Prager plane
// strain case (every realisation: ntype_eco > 1, ncrit 12, ntype_solid != 1, no
// continuity density, no training capture; the host checks): the arithmetic of
// tail_sp_rates<true>
// with the flow rule's outputs kept as the FP32 values they are (fewer registers, no FP64
// copies); FP64 only for the state's RK accumulation.
__device__ __forceinline__ void tail_sp_f32(const Dev& D, const StepScalars& sc, int t,
                                            double f2) {
  const Real& M = real_of(D, t);
  const double* gu = D.grad_u + 4 * (size_t)t;
  const double g[4] = {gu[0], gu[1], gu[2], gu[3]};
  const double st[4] = {D.s0[t], D.s1[t], D.s2[t], D.s3[t]};
  double f = D.fdp[t];
  float G[4], vv[4];
  drucker_prager_f32v(M, sc.time_sph, st, g, &f, G, vv);  // (no capture: see lean_tail)
  D.fdp[t] = f;
  // explicit fmaf: the same rounding as tail_sp_rates<true>
  const float q = fmaf(2.0f, fmaf(vv[0], vv[0], fmaf(vv[1], vv[1], __fmul_rn(vv[3], vv[3]))),
                       __fmul_rn(vv[2], vv[2]));
  const double der = f64_of(sqrtf(__fmul_rn(q, 1.0f / 3.0f)));
  const float h11 = f32_rn(g[0]), h21 = f32_rn(g[1]), h12 = f32_rn(g[2]), h22 = f32_rn(g[3]);
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
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const double rhs = f64_of(r[k] + -G[k]);
    D.RHS1[k][t] = rhs;
    D.RKs[k][t] = fma(f2, rhs, D.RKs[k][t]);
  }
  D.RKd[t] = D.RKd[t] + der * f2;
}

// The surrogate's view of stress-point t: the exact rule (drucker_prager, whose results dp
// = {G, vivel, f} the tail reuses), whether it is loading, and for a loading point the
// network's inputs x, their output scale and whether they lie in the training envelope.
// Deterministic, so k_fsp_cand and k_fsp_tail<true> reach the same decisions.
__device__ __forceinline__ void surr_front(const Dev& D, const Real& M, const StepScalars& sc,
                                           int t, double* g, double* s2v, float* x,
                                           double& scale, bool& loading, bool& cand,
                                           double* dp) {
  const double* gu = D.grad_u + 4 * (size_t)t;
  for (int k = 0; k < 4; k++) g[k] = gu[k];
  s2v[0] = D.s0[t];
  s2v[1] = D.s1[t];
  s2v[2] = D.s2[t];
  s2v[3] = D.s3[t];
  if (M.ntype_solid == 1) s2v[3] = M.poiss * (s2v[0] + s2v[1]);
  double f = D.fdp[t], G2[4], vivel[4];
  drucker_prager_f32(M, sc.time_sph, s2v, g, &f, G2, vivel);  // the exact rule
  loading = G2[0] != 0.0 || G2[1] != 0.0 || G2[2] != 0.0 || G2[3] != 0.0;
  for (int k = 0; k < 4; k++) {
    dp[k] = G2[k];
    dp[4 + k] = vivel[k];
  }
  dp[8] = f;
  scale = 0.0;
  cand = false;
  if (loading) {
    scale = mlp_features(s2v, g, M.tanfi, M.coh, M.young, M.poiss, D.rho[t], x);
    cand = scale > 0.0;
    for (int k = 0; k < MLP_NIN && cand; k++) cand = x[k] >= D.env_lo[k] && x[k] <= D.env_hi[k];
  }
}

// One stress-point (index i among the stress-points) of k_fsp_tail; the warp's 32 lanes
// call it together.  SURR: the network's prediction for a candidate is the row that
// k_fsp_cand appended for it this stage, computed by the tensor-core kernel in between.
template <bool SURR, bool LEAN = false>
__device__ __forceinline__ void fsp_tail_one(const Dev& D, int stage, int i) {
  const int lane = threadIdx.x & 31;
  const bool act = i < D.NT - D.NN;
  const int t = D.NN + (act ? i : 0);
  const double f2 = (stage == 1 || stage == 2) ? 2.0 : 1.0;  // RK4 weights 1, 2, 2, 1
  const Real& M = real_of(D, t);
  const StepScalars& sc = D.cur[D.R == 1 ? 0 : D.rid[t]];
  double g[4] = {0.0, 0.0, 0.0, 0.0}, s2v[4] = {0.0, 0.0, 0.0, 0.0};
  float x[16];
  double scale = 0.0;
  bool loading = false, cand = false;
  // drucker_prager's results (G, vivel, f), handed to the tail, which would repeat them
  double dp[9];
  bool have_dp = false;
  if (SURR && act && M.ntype_eco > 1 && M.ncrit == 12) {
    surr_front(D, M, sc, t, g, s2v, x, scale, loading, cand, dp);
    have_dp = true;
  }
  double Gnet[4];
  bool accept = false;
  if (SURR && cand) {
    const float* y = D.ycand + 4 * (size_t)D.cand_row[i];
    bool inside = true;
    for (int k = 0; k < MLP_NOUT; k++) {
      const float yk = y[k];
      inside = inside && fabsf(yk) <= 1.5f * D.out_max;
      Gnet[k] = (double)yk * scale;
    }
    if (inside) {
      // drift test in FP64
      double sm = ((s2v[0] + s2v[1]) + s2v[3]) / 3.0;
      double d0 = s2v[0] - sm, d1 = s2v[1] - sm, d2 = s2v[2], d3 = s2v[3] - sm;
      double sj = sqrt(d2 * d2 + 0.5 * ((d0 * d0 + d1 * d1) + d3 * d3));
      double e0 = M.D11 * g[0] + M.D12 * g[3] + Gnet[0];
      double e1 = M.D12 * g[0] + M.D22 * g[3] + Gnet[1];
      double e2 = M.D33 * g[1] + M.D33 * g[2] + Gnet[2];
      double e3 = M.D41 * g[0] + M.D42 * g[3] + Gnet[3];
      double df = (d0 * e0 + d1 * e1 + d3 * e3 + 2.0 * d2 * e2) / (2.0 * sj) +
                  M.alpha2 * (e0 + e1 + e3);
      accept = sj > 0.0 && M.dt * fabs(df) <= D.surr_tol * sj;
    } else {
      cand = false;  // counted as outside the envelope
    }
  }
  // counters: loading, answered, outside the envelope, drift-rejected
  if (SURR) {
    unsigned ml = __ballot_sync(0xffffffffu, loading), ma = __ballot_sync(0xffffffffu, accept),
             mc = __ballot_sync(0xffffffffu, cand);
    if (lane == 0 && ml) {
      atomicAdd(&D.surr_cnt[0], (unsigned long long)__popc(ml));
      atomicAdd(&D.surr_cnt[1], (unsigned long long)__popc(ma));
      atomicAdd(&D.surr_cnt[2], (unsigned long long)(__popc(ml) - __popc(mc)));
      atomicAdd(&D.surr_cnt[3], (unsigned long long)(__popc(mc) - __popc(ma)));
    }
  }
  if (!act) return;
  if (accept) {
    // plastic strain rate of the predicted source: e_p = G / (2 G_mod), shear G / G_mod
    const double gm = M.young / (2.0 * (1.0 + M.poiss));
    double v0 = -Gnet[0] / (2.0 * gm), v1 = -Gnet[1] / (2.0 * gm), v2 = -Gnet[2] / gm,
           v3 = -Gnet[3] / (2.0 * gm);
    double der = sqrt((2.0 * ((v0 * v0 + v1 * v1) + v3 * v3) + v2 * v2) / 3.0);
    tail_sp_rates<true>(D, sc, t, D.grad_u + 4 * (size_t)t, f2, Gnet, der, have_dp ? dp : nullptr);
  } else if (LEAN) {
    tail_sp_f32(D, sc, t, f2);
  } else {
    tail_sp_rates<true>(D, sc, t, D.grad_u + 4 * (size_t)t, f2, nullptr, 0.0,
                        have_dp ? dp : nullptr);
  }
}

// The stress-point tail of an RK4 stage (2_SPH_main_2018.f90:727-777): plastic_terms and
// drucker_prager (3_SPH_material_2018.f90:1884-2062), the Jaumann spin
// (2_SPH_main_2018.f90:1021-1034), the rates and their RK accumulation.  Each block strides
// over block-sized chunks of the stress-points.
// With the surrogate installed both variants are launched: the one the gate selects for
// this step runs, the other's blocks return at once.  The variant with the network runs
// over at most kTailBlocks blocks (a few SM-fulls, so that the launch costs little when the
// gate skips it); the one without over a block per 128 stress-points.
constexpr int kTailBlocks = 152 * 8;
// LEAN (without the network only): tail_sp_f32 for the Drucker-Prager plane strain case
template <bool SURR, bool LEAN = false>
__global__ void __launch_bounds__(128) k_fsp_tail(Dev D, int stage) {
  if (D.surr && (D.surr_gate->on != 0) != SURR) return;
  const int ns = D.NT - D.NN;
  for (int base = blockIdx.x * blockDim.x; base < ns; base += gridDim.x * blockDim.x)
    fsp_tail_one<SURR, LEAN>(D, stage, base + threadIdx.x);
}

// The surrogate's candidates of this stage (while the gate runs the network): every loading
// stress-point whose inputs lie in the training envelope appends its inputs (16 floats) as
// one row of xcand; cand_row[i] holds the row of stress-point i, or -1.  The rows of a warp
// are reserved with one atomic on the stage's count (reset at the start of every step).
__global__ void __launch_bounds__(128) k_fsp_cand(Dev D, int stage) {
  if (!D.surr || D.surr_gate->on == 0) return;
  const int ns = D.NT - D.NN, lane = threadIdx.x & 31;
  for (int base = blockIdx.x * blockDim.x; base < ns; base += gridDim.x * blockDim.x) {
    const int i = base + threadIdx.x;
    const bool act = i < ns;
    const int t = D.NN + (act ? i : 0);
    const Real& M = real_of(D, t);
    const StepScalars& sc = D.cur[D.R == 1 ? 0 : D.rid[t]];
    double g[4], s2v[4], scale, dp[9];
    float x[16];
    bool loading = false, cand = false;
    if (act && M.ntype_eco > 1 && M.ncrit == 12)
      surr_front(D, M, sc, t, g, s2v, x, scale, loading, cand, dp);
    const unsigned m = __ballot_sync(0xffffffffu, cand);
    int row0 = 0;
    if (lane == 0 && m) row0 = atomicAdd(&D.cand_count[stage], __popc(m));
    row0 = __shfl_sync(0xffffffffu, row0, 0);
    int row = -1;
    if (cand) {
      row = row0 + __popc(m & ((1u << lane) - 1u));
      float4* o = reinterpret_cast<float4*>(D.xcand + 16 * (size_t)row);
      for (int q = 0; q < 4; q++) o[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
    }
    if (act) D.cand_row[i] = row;
  }
}

// XSPH_update (2_SPH_main_2018.f90:189-239), FP32 sums of double-float velocity differences
__global__ void k_fxsph(Dev D) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  int t = D.sorted[s];
  if (t >= D.NT) return;
  const int col = D.lcol[s];
  int deg = D.degS[col];
  const double vt0 = D.vx[t], vt1 = D.vy[t];
  float vh0, vh1, vl0, vl1;
  f32_split(vt0, vh0, vl0);
  f32_split(vt1, vh1, vl1);
  Kahan s0, s1;
  int flag = D.bc_or_not[t];
  bool mark = false;
  for (int k = 0; k < deg; k++) {
    int4 e = D.same[ell(k, col, D.N2)];
    int u = e.x;
    float w = __int_as_float(e.y);
    float4 r = D.recV[u];
    float vw = D.recI[u].y * w;
    s0.add(dfdiff(r.x, r.z, vh0, vl0) * vw);
    s1.add(dfdiff(r.y, r.w, vh1, vl1) * vw);
    if (t < D.NN && D.bc_or_not[u] == 2 && flag != 2) mark = true;
  }
  const double eps = 0.5;
  const double dt = real_of(D, t).dt;
  D.px[t] = D.x0x[t] + dt * (vt0 + eps * s0.val());
  D.py[t] = D.x0y[t] + dt * (vt1 + eps * s1.val());
  if (mark) D.bc_or_not[t] = 3;
}

}  // namespace

// the targets split by kind (k_split_targets) after the pair build; one launch per kind
template <int KP>
void launch_finterp_kp(Ctx& c) {
  const Dev& D = c.d;
  const int ns = D.NT - D.NN, b = c.blk[TK_INTERP];
  c.kernels_launched += 1;
  if (ns > 0) k_finterp<1, KP><<<(ns + b - 1) / b, b, 0, c.stream>>>(D, D.tgtS, ns);
  k_finterp<2, KP><<<(D.NN + b - 1) / b, b, 0, c.stream>>>(D, D.tgtN, D.NN);
}
void launch_finterp(Ctx& c) {
  const Dev& D = c.d;
  if (!D.sp_sph) {
    k_finterp<0, 4><<<c.grid_of(TK_INTERP, D.N2), c.blk[TK_INTERP], 0, c.stream>>>(D, nullptr, 0);
    return;
  }
  switch (c.ahead[0]) {
    case 2: launch_finterp_kp<2>(c); break;
    case 8: launch_finterp_kp<8>(c); break;
    default: launch_finterp_kp<4>(c);
  }
}
template <int KP, bool CSPM>
void launch_fderivs_kp(Ctx& c, int stage) {
  const Dev& D = c.d;
  const int ns = D.NT - D.NN, b = c.blk[TK_DERIVS];
  c.kernels_launched += 1;
  // the stress-point sums (64 registers) load one neighbour ahead; more spill
  if (ns > 0) k_fderivs<1, 1, CSPM><<<(ns + b - 1) / b, b, 0, c.stream>>>(D, stage, D.tgtS, ns);
  k_fderivs<2, KP, CSPM><<<(D.NN + b - 1) / b, b, 0, c.stream>>>(D, stage, D.tgtN, D.NN);
}
template <int KP>
void launch_fderivs_kp(Ctx& c, int stage) {
  if (c.d.cspm) launch_fderivs_kp<KP, true>(c, stage);
  else launch_fderivs_kp<KP, false>(c, stage);
}
void launch_fderivs(Ctx& c, int stage) {
  switch (c.ahead[1]) {
    case 1: launch_fderivs_kp<1>(c, stage); break;
    case 4: launch_fderivs_kp<4>(c, stage); break;
    default: launch_fderivs_kp<2>(c, stage);
  }
}
void launch_fsp_tail(Ctx& c, int stage) {
  int ns = c.d.NT - c.d.NN;
  if (ns <= 0) return;
  const int nb = std::min((ns + 127) / 128, kTailBlocks);
  if (c.d.surr) {
    // the network's rows of this stage: candidates, then the tensor-core forward pass over
    // as many 128-row tiles as there are candidates (a grid of at most two CTAs per SM)
    c.kernels_launched += 3;
    k_fsp_cand<<<nb, 128, 0, c.stream>>>(c.d, stage);
    SPS_CUDA_CHECK(mlp_tc_forward(c.d.tc_img, c.d.tc_bias, c.d.xcand, 16, MLP_NIN,
                                  c.d.cand_count + stage, ns, c.d.ycand, MLP_NOUT, c.d.err,
                                  kErrTensorCore, c.tc_grid, c.stream));
    k_fsp_tail<true><<<nb, 128, 0, c.stream>>>(c.d, stage);
  }
  // the variant without the network over one block per 128 stress-points: when it runs
  // it does the work, and the scheduler refills SMs with fresh blocks as others wait
  if (c.lean_tail && !c.d.cap_buf)
    k_fsp_tail<false, true><<<(ns + 127) / 128, 128, 0, c.stream>>>(c.d, stage);
  else k_fsp_tail<false><<<(ns + 127) / 128, 128, 0, c.stream>>>(c.d, stage);
}
void launch_fxsph(Ctx& c) {
  k_fxsph<<<c.grid_of(TK_XSPH, c.d.N2), c.blk[TK_XSPH], 0, c.stream>>>(c.d);
}

int launch_fast_step(Ctx& c) { return launch_plain_step(c); }

}  // namespace sps
