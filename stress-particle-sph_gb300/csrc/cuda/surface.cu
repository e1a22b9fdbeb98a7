// surface.cu -- get_nodes_on_free_surface (3_SPH_material_2018.f90:1135-1430) as gathers per
// particle (compiled with -fmad=false: the reference's rounding, both forms).
//
// The routine's locals are `real` (FP32) and its module arrays normal and subset FP64; an
// FP32 accumulation with an FP64 operand is evaluated in FP64 and rounded once.  Steps 1 and
// 4 accumulate over node--stress-point and same-type pairs in the order of the reference's
// linked list: a particle merges its two neighbour lists by their walk-order keys (written
// by k_lists), which restores that order.  Step 3 (is a neighbour inside the particle's scan
// region?) does not depend on the order.
//   k_fs_normal0  steps 1-2 (:1180-1253): renormalisation matrix, kernel-gradient sums,
//                 first normal
//   k_fs_scan     step 3 (:1254-1369) + the bc_or_not update: subset (1 surface,
//                 2 inside), f_int
//   k_fs_normal   step 4 (:1370-1430): normals of surface particles from their surface
//                 neighbours
#include <cuda_runtime.h>

#include "ctx.cuh"

namespace sps {

namespace {

constexpr int kBlock = 256;

// the merged walk over a target's node--stress-point (cross, non-dummy neighbour) and
// same-type entries, in ascending key; f(u, gx, gy, is_pair_i)
template <typename F>
__device__ __forceinline__ void walk_123(const Dev& D, int col, F&& f) {
  const int nC = D.degC[col], nS = D.degS[col];
  int a = 0, b = 0;
  int32_t ka = 0, kb = 0;
  int4 ea = make_int4(0, 0, 0, 0), eb = make_int4(0, 0, 0, 0);
  auto next_cross = [&]() {
    while (a < nC) {
      ea = D.cross[ell(a, col, D.N2)];
      if (ea.y >= 0) {  // not a dummy partner (sign bit of W)
        ka = D.keyC[(size_t)a * D.N2 + col];
        return;
      }
      a++;
    }
  };
  next_cross();
  if (b < nS) {
    eb = D.same[ell(b, col, D.N2)];
    kb = D.keyS[(size_t)b * D.N2 + col];
  }
  while (a < nC || b < nS) {
    // one call site for both lists, so that a warp whose lanes take different lists runs
    // the body once
    const bool takeC = (a < nC) && (b >= nS || ka < kb);
    const int u = takeC ? ea.x : eb.x;
    const int gx = takeC ? ea.z : eb.z, gy = takeC ? ea.w : eb.w;
    const int32_t key = takeC ? ka : kb;
    f(u, __int_as_float(gx), __int_as_float(gy), (key & 1) != 0);
    if (takeC) {
      a++;
      next_cross();
    } else {
      b++;
      if (b < nS) {
        eb = D.same[ell(b, col, D.N2)];
        kb = D.keyS[(size_t)b * D.N2 + col];
      }
    }
  }
}

// hf = (m_u G / rho_u) rounded to FP32; G is the gradient with respect to the target, which
// gives the reference's hf1i (target pair_i) and hf1j = -(m_i gradW / rho_i) (target pair_j).
// The float rounding of the IEEE quotient comes from the reciprocal 1/rho_u (div_rcp_f32),
// the float -> double conversion from the integer pipe: two FP64 multiplies per value.
__device__ __forceinline__ float hf_of(double m, double rho, double rinv, float g) {
  return div_rcp_f32(m * f64_of(g), rho, rinv);
}

// (float)((double)acc + d * (double)h): the FP32 accumulation of an FP64 term, with the
// conversions on the integer pipe
__device__ __forceinline__ float acc_f64(float acc, double d, float h) {
  return f32_rn(f64_of(acc) + d * f64_of(h));
}

__global__ void k_fs_normal0(Dev D) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  const int t = D.sorted[s];
  if (t >= D.NT) return;
  const double xt = D.px[t], yt = D.py[t];
  float A0 = 0.0f, A1 = 0.0f, A2 = 0.0f, A3 = 0.0f, f0 = 0.0f, f1 = 0.0f;
  walk_123(D, D.lcol[s], [&](int u, float gx, float gy, bool) {
    const double m = D.mass[u], rho = D.rho[u], ri = D.rinv[u];
    float h1 = hf_of(m, rho, ri, gx), h2 = hf_of(m, rho, ri, gy);
    double dx = D.px[u] - xt, dy = D.py[u] - yt;
    A0 = acc_f64(A0, dx, h1);
    A1 = acc_f64(A1, dy, h1);
    A2 = acc_f64(A2, dx, h2);
    A3 = acc_f64(A3, dy, h2);
    f0 = f0 + h1;
    f1 = f1 + h2;
  });
  if (fabsf(A0) <= 1.e-8f) A0 = 0.0f;
  if (fabsf(A1) <= 1.e-8f) A1 = 0.0f;
  if (fabsf(A2) <= 1.e-8f) A2 = 0.0f;
  if (fabsf(A3) <= 1.e-8f) A3 = 0.0f;
  float v0 = -(A0 * f0 + A1 * f1);
  float v1 = -(A2 * f0 + A3 * f1);
  float v2 = sqrtf(v0 * v0 + v1 * v1);
  D.nrmx[t] = (double)(v0 / v2);
  D.nrmy[t] = (double)(v1 / v2);
}

// the scan region of particle a: its position, normal and smoothing length, the point
// T = x_a + h_a n_a and the tangent, in the precisions the reference holds them
struct ScanRegion {
  double xa, ya, nx, ny, ha;
  double tt0, tt1;  // FP32 values of T, widened
  float tau0, tau1, limit;
};
__device__ __forceinline__ ScanRegion scan_region(const Dev& D, int a) {
  ScanRegion R;
  R.xa = D.px[a];
  R.ya = D.py[a];
  R.nx = D.nrmx[a];
  R.ny = D.nrmy[a];
  R.ha = D.hsml[a];
  R.tt0 = (double)(float)(R.xa + R.ha * R.nx);
  R.tt1 = (double)(float)(R.ya + R.ha * R.ny);
  R.tau0 = (float)(-R.ny);
  R.tau1 = (float)R.nx;
  R.limit = (float)((double)sqrtf(2.0f) * R.ha);
  return R;
}

// true when a neighbour at (xb, yb) lies in the scan region (then a is not on the surface)
__device__ __forceinline__ bool in_scan_region(const ScanRegion& R, double xb, double yb) {
  double ddx = xb - R.xa, ddy = yb - R.ya;
  float xba = (float)sqrt(ddx * ddx + ddy * ddy);
  float xbt0 = f32_rn(xb - R.tt0), xbt1 = f32_rn(yb - R.tt1);
  if (xba >= R.limit) {
    float xbt_norm = sqrtf(xbt0 * xbt0 + xbt1 * xbt1);
    return (double)xbt_norm < R.ha;
  }
  if (xba < R.limit) {
    float prod = f32_rn(fabs(R.nx * f64_of(xbt0) + R.ny * f64_of(xbt1)) +
                        f64_of(fabsf(R.tau0 * xbt0 + R.tau1 * xbt1)));
    return (double)prod < R.ha;
  }
  return false;  // a NaN distance lies in neither part of the region
}

__global__ void k_fs_scan(Dev D) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  const int t = D.sorted[s];
  if (t >= D.NT) return;
  bool inside = false;
  const int col = D.lcol[s];
  const int nS = D.degS[col], nC = D.degC[col];
  const ScanRegion R = scan_region(D, t);
  for (int k = 0; k < nS && !inside; k++) {
    int u = D.same[ell(k, col, D.N2)].x;
    inside = in_scan_region(R, D.px[u], D.py[u]);
  }
  for (int k = 0; k < nC && !inside; k++) {
    const int4 e = D.cross[ell(k, col, D.N2)];
    if (e.y < 0) inside = in_scan_region(R, D.px[e.x], D.py[e.x]);  // dummy partners
  }
  int sub = inside ? 2 : 1;
  D.fint[t] = inside ? -1.0f : 0.0f;
  int bc = D.bc_or_not[t];
  if (bc != 1) bc = (sub == 1) ? 2 : 0;
  else if (sub == 1) sub = 2;
  D.bc_or_not[t] = bc;
  D.subset[t] = (int8_t)sub;
}

__global__ void k_fs_normal(Dev D) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  const int t = D.sorted[s];
  if (t >= D.NT) return;
  const bool surf = D.subset[t] == 1;
  const float ft = D.fint[t];
  const float xtf = (float)D.px[t], ytf = (float)D.py[t];
  double nx = 0.0, ny = 0.0;
  float nb = 0.0f, g0 = 0.0f, g1 = 0.0f;
  walk_123(D, D.lcol[s], [&](int u, float gx, float gy, bool pair_i) {
    if (surf && D.subset[u] == 1) {
      // the reference adds the same vector x_j - x_i to both particles of the pair
      float xu = (float)D.px[u], yu = (float)D.py[u];
      float xv = pair_i ? xu - xtf : xtf - xu;
      float yv = pair_i ? yu - ytf : ytf - yu;
      nx = nx - (double)yv;
      ny = ny + (double)xv;
      nb = nb + 1.0f;
    }
    const double m = D.mass[u], rho = D.rho[u], ri = D.rinv[u];
    float h1 = hf_of(m, rho, ri, gx), h2 = hf_of(m, rho, ri, gy);
    float df = D.fint[u] - ft;
    g0 = g0 + df * h1;
    g1 = g1 + df * h2;
  });
  if (surf) {
    nx = nx / (double)nb;
    ny = ny / (double)nb;
    float nv = (float)sqrt(nx * nx + ny * ny);
    nx = nx / (double)nv;
    ny = ny / (double)nv;
    float p = (float)((double)g0 * nx + (double)g1 * ny);
    if (p < 0) {
      nx = -nx;
      ny = -ny;
    }
  }
  D.nrmx[t] = nx;
  D.nrmy[t] = ny;
}

// ---- FP32 detection (the FP32 form's on-demand detection, for output only) -------------
// The same three steps with the arithmetic in FP32: m/rho per particle, separations from
// one FP64 subtraction each, FP32 sums.  The node--stress-point and same-type lists are
// walked one after the other instead of merged by walk-order key (the sums are FP32
// roundings apart from the exact detection's), and a pair's orientation comes from its
// type: pair_i is the stress-point of a node--stress-point pair and the creator (the lower
// sorted position) of a same-type pair, as in the walk-order keys.

__global__ void k_fs_vol32(Dev D) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < D.NT) D.vol32[t] = (float)(D.mass[t] / D.rho[t]);
}

// f(u, gx, gy, is_same) over the non-dummy cross entries, then the same-type entries
template <typename F>
__device__ __forceinline__ void walk_123_f32(const Dev& D, int col, F&& f) {
  const int nC = D.degC[col], nS = D.degS[col];
  for (int a = 0; a < nC; a++) {
    const int4 e = D.cross[ell(a, col, D.N2)];
    if (e.y >= 0) f(e.x, __int_as_float(e.z), __int_as_float(e.w), false);
  }
  for (int b = 0; b < nS; b++) {
    const int4 e = D.same[ell(b, col, D.N2)];
    f(e.x, __int_as_float(e.z), __int_as_float(e.w), true);
  }
}

// steps 1-3 (3_SPH_material_2018.f90:1180-1369) for one particle: its first normal from
// the kernel-gradient sums, then, with that normal (the scan region needs the particle's
// own normal only), whether a neighbour lies in its scan region
__global__ void k_fs_normal_scan_f32(Dev D) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  const int t = D.sorted[s];
  if (t >= D.NT) return;
  const int col = D.lcol[s];
  const double xt = D.px[t], yt = D.py[t];
  float A0 = 0.0f, A1 = 0.0f, A2 = 0.0f, A3 = 0.0f, f0 = 0.0f, f1 = 0.0f;
  walk_123_f32(D, col, [&](int u, float gx, float gy, bool) {
    const float v = D.vol32[u];
    const float h1 = v * gx, h2 = v * gy;
    const float dx = f32_rn(D.px[u] - xt), dy = f32_rn(D.py[u] - yt);
    A0 = fmaf(dx, h1, A0);
    A1 = fmaf(dy, h1, A1);
    A2 = fmaf(dx, h2, A2);
    A3 = fmaf(dy, h2, A3);
    f0 += h1;
    f1 += h2;
  });
  if (fabsf(A0) <= 1.e-8f) A0 = 0.0f;
  if (fabsf(A1) <= 1.e-8f) A1 = 0.0f;
  if (fabsf(A2) <= 1.e-8f) A2 = 0.0f;
  if (fabsf(A3) <= 1.e-8f) A3 = 0.0f;
  const float v0 = -(A0 * f0 + A1 * f1);
  const float v1 = -(A2 * f0 + A3 * f1);
  const float v2 = sqrtf(v0 * v0 + v1 * v1);
  const float nx = v0 / v2, ny = v1 / v2;
  D.nrmx[t] = (double)nx;
  D.nrmy[t] = (double)ny;
  // step 3: the scan region of t
  const int nS = D.degS[col], nC = D.degC[col];
  const float ha = (float)D.hsml[t];
  const float limit = sqrtf(2.0f) * ha;
  // T = x_t + h_t n_t relative to x_t, the tangent (-ny, nx)
  const float T0 = ha * nx, T1 = ha * ny;
  auto in_region = [&](int u) {
    const float ddx = f32_rn(D.px[u] - xt), ddy = f32_rn(D.py[u] - yt);
    const float xba = sqrtf(ddx * ddx + ddy * ddy);
    const float xbt0 = ddx - T0, xbt1 = ddy - T1;
    if (xba >= limit) return sqrtf(xbt0 * xbt0 + xbt1 * xbt1) < ha;
    if (xba < limit) return fabsf(nx * xbt0 + ny * xbt1) + fabsf(-ny * xbt0 + nx * xbt1) < ha;
    return false;
  };
  bool inside = false;
  for (int k = 0; k < nS && !inside; k++) inside = in_region(D.same[ell(k, col, D.N2)].x);
  for (int k = 0; k < nC && !inside; k++) {
    const int4 e = D.cross[ell(k, col, D.N2)];
    if (e.y < 0) inside = in_region(e.x);  // dummy partners
  }
  int sub = inside ? 2 : 1;
  D.fint[t] = inside ? -1.0f : 0.0f;
  int bc = D.bc_or_not[t];
  if (bc != 1) bc = (sub == 1) ? 2 : 0;
  else if (sub == 1) sub = 2;
  D.bc_or_not[t] = bc;
  D.subset[t] = (int8_t)sub;
}

// step 4 (3_SPH_material_2018.f90:1370-1430) of the FP32 detection: the normals of the
// surface particles from their surface neighbours
__global__ void k_fs_normal_f32(Dev D) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  const int t = D.sorted[s];
  if (t >= D.NT) return;
  const bool surf = D.subset[t] == 1;
  const bool t_sp = is_sp(D.itype[t]);
  const float ft = D.fint[t];
  const double xt = D.px[t], yt = D.py[t];
  // compensated sums (Kahan, with the exact FMA residual of each product): the normal's
  // direction and its orientation test p below are sums that can nearly cancel, and their
  // result must not depend on the order in which a list holds its neighbours
  struct Sum {
    float s = 0.0f, c = 0.0f, e = 0.0f;
    __device__ __forceinline__ void add(float x) {
      const float y = x - c;
      const float t = s + y;
      c = (t - s) - y;
      s = t;
    }
    __device__ __forceinline__ void add_prod(float a, float b) {
      const float p = __fmul_rn(a, b);
      e += fmaf(a, b, -p);
      add(p);
    }
    __device__ __forceinline__ double val() const { return ((double)s - (double)c) + (double)e; }
  };
  Sum nx, ny, g0, g1;
  float nb = 0.0f;
  walk_123_f32(D, D.lcol[s], [&](int u, float gx, float gy, bool same) {
    if (surf && D.subset[u] == 1) {
      // the reference adds the same vector x_j - x_i to both particles of the pair
      const bool pair_i = same ? s < D.spos[u] : t_sp;
      const float xv = f32_rn(pair_i ? D.px[u] - xt : xt - D.px[u]);
      const float yv = f32_rn(pair_i ? D.py[u] - yt : yt - D.py[u]);
      nx.add(-yv);
      ny.add(xv);
      nb += 1.0f;
    }
    const float v = D.vol32[u];
    const float df = D.fint[u] - ft;
    g0.add_prod(df, v * gx);
    g1.add_prod(df, v * gy);
  });
  double dnx = 0.0, dny = 0.0;
  if (surf) {
    dnx = nx.val() / (double)nb;
    dny = ny.val() / (double)nb;
    const float nv = (float)sqrt(dnx * dnx + dny * dny);
    dnx = dnx / (double)nv;
    dny = dny / (double)nv;
    const float p = (float)(g0.val() * dnx + g1.val() * dny);
    if (p < 0) {
      dnx = -dnx;
      dny = -dny;
    }
  }
  D.nrmx[t] = dnx;
  D.nrmy[t] = dny;
}

}  // namespace

void launch_surface_f32(Ctx& c) {
  const int nb = (c.d.N2 + kBlock - 1) / kBlock;
  c.mark("surface", 3);
  k_fs_vol32<<<(c.d.NT + kBlock - 1) / kBlock, kBlock, 0, c.stream>>>(c.d);
  k_fs_normal_scan_f32<<<nb, kBlock, 0, c.stream>>>(c.d);
  k_fs_normal_f32<<<nb, kBlock, 0, c.stream>>>(c.d);
}

void launch_surface(Ctx& c) {
  const int nb = (c.d.N2 + kBlock - 1) / kBlock;
  c.mark("surface", 3);
  k_fs_normal0<<<nb, kBlock, 0, c.stream>>>(c.d);
  k_fs_scan<<<nb, kBlock, 0, c.stream>>>(c.d);
  k_fs_normal<<<nb, kBlock, 0, c.stream>>>(c.d);
}

}  // namespace sps
