// neighbours.cu -- cell-linked neighbour search of the SPS step (compiled with -fmad=false).
//
// Restates grid_find_NEW (example_problems/soil_failure_bui_et_al_2008/
// 2_SPH_main_2018.f90:1199-1435), kernel (:1440) and Pint_Update
// (3_SPH_material_2018.f90:1574) as a GB300 pipeline:
//   k_bbox      Check_Out_Domain (:1170) + bounding box / max h over active particles
//   k_grid      grid parameters with the reference's arithmetic (:1245-1258)
//   k_cell_*    counting sort by cell, stable in particle id (the order list_picell holds)
//   k_half      pairs created by each particle over the half stencil (self, +x, row
//               above), in the reference's creation order, with FP32-stored W and dW
//   k_lists     per-target neighbour lists in the reference's linked-list walk order
// The distance test r < scale_k*(h_i+h_j)/2 is decided on FP32 cell-frame coordinates
// with a guard band; candidates inside the band are re-tested with the exact FP64
// expression, so the pair set equals the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>

#include "ctx.cuh"

namespace sps {

namespace {

constexpr int kBlock = 256;
// half-list entries: partner id in the low 28 bits, pair type (pint_type) in the top 4
constexpr int kHalfTypeShift = 28;
constexpr unsigned kHalfIdMask = (1u << kHalfTypeShift) - 1u;

// ---- double-float (unevaluated sum of two FP32 numbers) arithmetic: Dekker, "A floating-
// point technique for extending the available precision", Numer. Math. 18, 1971, with the
// FMA-based exact product.  Used by the FP32 form for the separations and r/h of its pairs
// (cubic_mixed).
__device__ __forceinline__ dfl df_fast2sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ dfl df_2sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dfl df_mul(dfl x, dfl y) {
  float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e += x.hi * y.lo + x.lo * y.hi;
  return df_fast2sum(p, e);
}
__device__ __forceinline__ dfl df_sqrt(dfl x) {
  if (x.hi <= 0.0f) return {0.0f, 0.0f};
  float s = x.hi * rsqrtf(x.hi);  // approximate seed, corrected below
  float p = s * s;
  float e = fmaf(s, s, -p);
  float r = ((x.hi - p) - e) + x.lo;
  return df_fast2sum(s, r * (0.5f * __frcp_rn(s)));
}
// x^2 + y^2 of two double-float values, accurate to a few units of 2^-44: the exact
// squares of the high parts (FMA residuals) summed exactly, the cross terms and residuals
// added once; sign-symmetric in x and y
__device__ __forceinline__ dfl df_sumsq(dfl x, dfl y) {
  const float px = x.hi * x.hi, ex = fmaf(x.hi, x.hi, -px);
  const float py = y.hi * y.hi, ey = fmaf(y.hi, y.hi, -py);
  dfl s = df_2sum(px, py);
  s.lo += (ex + ey) + 2.0f * fmaf(x.hi, x.lo, y.hi * y.lo);
  return df_fast2sum(s.hi, s.lo);
}
// the separation (xa + xal) - (xb + xbl) - q (c.hi + c.lo), q in {-1, 0, 1}, as a
// double-float: the two exact sums of the high parts, the low parts added once (the cell
// shift q c.hi is exact); negating every input negates the result exactly
__device__ __forceinline__ dfl df_sep(float xa, float xal, float xb, float xbl, int q, dfl c) {
  const float ch = q < 0 ? -c.hi : (q > 0 ? c.hi : 0.0f);
  const float cl = q < 0 ? -c.lo : (q > 0 ? c.lo : 0.0f);
  const dfl a = df_2sum(xa, -xb);
  const dfl b = df_2sum(a.hi, -ch);
  return df_fast2sum(b.hi, ((a.lo + b.lo) + (xal - xbl)) - cl);
}
__device__ __forceinline__ dfl df_from(double v) {
  float h = (float)v;
  return {h, (float)(v - (double)h)};
}

// ordered key of a double: unsigned order of the keys = numeric order of the values, so
// that atomicMin on keys is an exact min over doubles
__device__ __forceinline__ unsigned long long okey(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double unkey(unsigned long long k) {
  unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}
constexpr unsigned long long kNoKey = ~0ull;  // no active particle

// Check_Out_Domain (2_SPH_main_2018.f90:1170) + the bounding box of the active particles of
// every realisation: keys of (minx, miny, -maxx, -maxy, -maxh, minh), reduced over the warp
// (or the block) when it holds one realisation, then atomicMin per realisation
__global__ void k_bbox(Dev D) {
  __shared__ unsigned long long sh[kBlock / 32][6];
  __shared__ int shr[kBlock / 32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long v[6] = {kNoKey, kNoKey, kNoKey, kNoKey, kNoKey, kNoKey};
  int r = -1;
  if (i < D.N2) {
    r = D.rid[i];
    const Real& M = D.real[r];
    double x = D.px[i], y = D.py[i];
    // (x - xmin)(x - xmax) > 0 of the reference: both differences non-zero and of one sign,
    // i.e. x outside [xmin, xmax] (the product of two such differences cannot underflow to
    // zero for a domain of non-zero width; a NaN coordinate gives false), decided on the
    // integer pipe with ordered keys
    auto outside = [](double v, double lo, double hi) {
      if (f64_isnan(v)) return false;
      const long long kv = f64_key(v), kl = f64_key(lo), kh = f64_key(hi);
      return kv < min(kl, kh) || kv > max(kl, kh);
    };
    uint8_t o = D.out[i];
    if (outside(x, M.xmin_dom[0], M.xmax_dom[0]) || outside(y, M.xmin_dom[1], M.xmax_dom[1]))
      o = 1;
    D.out[i] = o;
    if (!o) {
      double h = D.hsml[i];
      v[0] = okey(x);
      v[1] = okey(y);
      v[2] = okey(-x);
      v[3] = okey(-y);
      v[4] = okey(-h);
      v[5] = okey(h);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // the realisation of the warp (-1: several, or none active)
  int r0 = __shfl_sync(0xffffffffu, r, 0);
  for (int o = 16; o; o >>= 1) r0 = max(r0, __shfl_xor_sync(0xffffffffu, r0, o));
  const bool uni = __all_sync(0xffffffffu, r < 0 || r == r0);
  if (!uni) {
    if (r >= 0 && v[0] != kNoKey)
      for (int k = 0; k < 6; k++) atomicMin(&D.bbox[6 * (size_t)r + k], v[k]);
    r0 = -1;
  } else {
    for (int k = 0; k < 6; k++)
      for (int o = 16; o; o >>= 1) {
        unsigned long long u = __shfl_xor_sync(0xffffffffu, v[k], o);
        v[k] = u < v[k] ? u : v[k];
      }
  }
  if (lane == 0) {
    shr[wid] = r0;
    for (int k = 0; k < 6; k++) sh[wid][k] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int rb = shr[0];
    bool block_uni = rb >= 0;
    for (int w = 1; w < kBlock / 32 && block_uni; w++) block_uni = shr[w] == rb;
    if (block_uni) {
      unsigned long long m[6];
      for (int k = 0; k < 6; k++) {
        m[k] = sh[0][k];
        for (int w = 1; w < kBlock / 32; w++) m[k] = sh[w][k] < m[k] ? sh[w][k] : m[k];
      }
      if (m[0] != kNoKey)
        for (int k = 0; k < 6; k++) atomicMin(&D.bbox[6 * (size_t)rb + k], m[k]);
    } else {
      for (int w = 0; w < kBlock / 32; w++)
        if (shr[w] >= 0 && sh[w][0] != kNoKey)
          for (int k = 0; k < 6; k++) atomicMin(&D.bbox[6 * (size_t)shr[w] + k], sh[w][k]);
    }
  }
}

// grid parameters of every realisation (2_SPH_main_2018.f90:1230-1260) and the numbering
// of their cells (one block; the bounding-box keys are reset for the next step)
__global__ void k_grid(Dev D) {
  __shared__ int sc[kBlock];
  __shared__ int carry, bad;
  const int tid = threadIdx.x;
  if (tid == 0) {
    carry = 0;
    bad = 0;
  }
  __syncthreads();
  for (int base = 0; base < D.R; base += kBlock) {
    const int r = base + tid;
    int nc = 0;
    Grid g;
    if (r < D.R) {
      double red[6];
      for (int k = 0; k < 6; k++) {
        unsigned long long key = D.bbox[6 * (size_t)r + k];
        D.bbox[6 * (size_t)r + k] = kNoKey;
        red[k] = key == kNoKey ? 1e300 : unkey(key);
      }
      double hmax = -red[4];
      if (red[0] > 1e299) hmax = 0.0;  // no active particle
      double cellsz = hmax * 2.0;
      double ncd = 1.0;
      for (int d = 0; d < 2; d++) {
        double xmin = red[d] > 1e299 ? (double)1.e10f : red[d];
        double xmax = red[d] > 1e299 ? -(double)1.e10f : -red[2 + d];
        double length = xmax - xmin;
        double qd = length / cellsz + 1.0;
        int ndiv = (qd >= 1.0 && qd < 1.0e9) ? (int)qd : 1;
        double length_new = (double)ndiv * cellsz;
        g.xmin[d] = (xmin - (length_new - length) / 2.0) - (double)0.001f * length;
        g.deltx[d] = cellsz;
        g.rdeltx[d] = 1.0 / cellsz;
        g.ndiv[d] = ndiv;
        ncd *= ndiv;
      }
      g.overflow = (ncd > (double)D.cell_cap || !(cellsz > 0.0)) ? 1 : 0;
      nc = g.overflow ? 0 : (int)ncd;
      if (g.overflow) bad = 1;
      // uniform smoothing length: (h + h) / 2 == h, so every pair's kernel shares these
      g.uniform_h = (D.skf == 1 && red[5] == hmax && hmax > 0.0) ? 1 : 0;
      double h = hmax;
      g.h = h;
      g.yh = 1.0 / h;
      g.hh = h * h;
      g.yhh = 1.0 / g.hh;
      g.factor = 15.0 / (7.0 * D.pi * h * h);
      g.factor6 = g.factor / 6.0;
      g.c3 = g.factor6 * 3.0;
      g.df_h = df_from(g.h);
      g.df_yh = df_from(g.yh);
      g.df_yhh = df_from(g.yhh);
      g.df_factor = df_from(g.factor);
      g.df_factor6 = df_from(g.factor6);
      g.df_c3 = df_from(g.c3);
      g.df_cell[0] = df_from(g.deltx[0]);
      g.df_cell[1] = df_from(g.deltx[1]);
      // FP32 prefilter band: cell-relative offsets and the cell-corner shift each carry
      // |err| <= 2^-24 * 2 cells; the band covers eight times that relative to the support
      double ext = 2.0 * fmax(g.deltx[0], g.deltx[1]);
      double smin = (double)D.scale_k * red[5];
      g.tau = (float)((smin > 0) ? 8.0 * ext * 1.1920929e-07 / smin + 4e-6 : 1.0);
    }
    sc[tid] = nc;
    __syncthreads();
    for (int off = 1; off < kBlock; off <<= 1) {
      int add = tid >= off ? sc[tid - off] : 0;
      __syncthreads();
      sc[tid] += add;
      __syncthreads();
    }
    if (r < D.R) {
      g.ncells = nc;
      g.cell0 = carry + sc[tid] - nc;
      D.grid[r] = g;
    }
    __syncthreads();
    if (tid == kBlock - 1) carry += sc[tid];
    __syncthreads();
  }
  if (tid == 0) {
    GridTotal gt;
    gt.overflow = (bad || carry > D.cell_cap) ? 1 : 0;
    gt.ncells = gt.overflow ? 0 : carry;
    gt.nactive = 0;
    *D.gtot = gt;
    if (gt.overflow) atomicOr(D.err, ERR_CELLS);
  }
}

// (x - xmin) / deltx of the reference's cell index (2_SPH_main_2018.f90:1280), correctly
// rounded by div_rcp from the cell size's reciprocal (an IEEE division costs GB300's FP64
// pipe about ten times as much); non-finite offsets take the IEEE division
__device__ __forceinline__ double cell_quot(double a, double b, double y) {
  const bool finite = (__double_as_longlong(a) & 0x7FF0000000000000ll) != 0x7FF0000000000000ll;
  return finite ? div_rcp(a, b, y) : a / b;
}

// (int)q for 1 <= q < 2^31, truncating, on the integer pipe (the significand shifted by
// the exponent)
__device__ __forceinline__ int trunc_pos(double q) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(q);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;  // 0 .. 30
  const unsigned long long m = (b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
  return (int)(m >> (52 - e));
}

// (double)n for 0 <= n < 2^31, exact, on the integer pipe
__device__ __forceinline__ double i2d_pos(int n) {
  if (n == 0) return 0.0;
  const int e = 31 - __clz(n);  // the leading bit
  const unsigned long long m = ((unsigned long long)(unsigned)n << (52 - e)) & 0x000FFFFFFFFFFFFFull;
  return __longlong_as_double((long long)(((unsigned long long)(e + 1023) << 52) | m));
}

// local cell of a position in a realisation's grid: q = (x - xmin) / delta + 1 with the
// reference's rounding, then its integer part clamped to [1, ndiv]; the comparisons and
// conversions on the integer pipe (ordered keys; q >= 1 is positive, below 2^31)
__device__ __forceinline__ int cell_index(const Grid& g, double x, double y) {
  const double qx = cell_quot(x - g.xmin[0], g.deltx[0], g.rdeltx[0]) + 1.0;
  const double qy = cell_quot(y - g.xmin[1], g.deltx[1], g.rdeltx[1]) + 1.0;
  // particles inside the bounding box give 1 <= q < ndiv + 1; the clamps only guard
  // against non-finite coordinates (a NaN q takes cell 1, as the FP64 comparisons did)
  auto idx = [](double q, int nd) {
    if (f64_isnan(q)) return 1;
    const long long k = f64_key(q);
    if (!(k >= f64_key(1.0))) return 1;
    return k < f64_key(i2d_pos(nd)) ? trunc_pos(q) : nd;
  };
  const int ix = idx(qx, g.ndiv[0]), iy = idx(qy, g.ndiv[1]);
  return g.ndiv[0] * (iy - 1) + (ix - 1);
}

// Task 2 of grid_find_NEW (2_SPH_main_2018.f90:1275-1286): the cell of every particle
// inside the domain, and the cells' counts
__global__ void k_cell_count(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N2) return;
  const GridTotal gt = *D.gtot;
  int c;
  const Grid& g = D.grid[D.rid[i]];
  if (D.out[i] || gt.overflow) {
    c = gt.ncells;  // out-of-domain bucket, after every real cell
  } else {
    double x = D.px[i], y = D.py[i];
    int cl = cell_index(g, x, y);
    // FP32 offsets from the particle's own cell corner (|offset| <= one cell)
    int ix = cl % g.ndiv[0], iy = cl / g.ndiv[0];
    double ox = x - (g.xmin[0] + i2d_pos(ix) * g.deltx[0]);
    double oy = y - (g.xmin[1] + i2d_pos(iy) * g.deltx[1]);
    // the conversions on the integer pipe (f32_split: hi = (float)ox and lo = (float)(ox -
    // hi), the same bits as the hardware conversions, which GB300 issues at its FP64 rate)
    float oxh, oxl, oyh, oyl;
    f32_split(ox, oxh, oxl);
    f32_split(oy, oyh, oyl);
    D.xr[i] = oxh;
    D.yr[i] = oyh;
    if (D.fast) {
      D.xrl[i] = oxl;
      D.yrl[i] = oyl;
    }
    D.hr[i] = f32_rn(D.hsml[i]);
    c = g.cell0 + cl;
  }
  D.cell_of[i] = c;
  atomicAdd(&D.cell_cnt[c], 1);
}

// the cells' particle lists (list_picell, 2_SPH_main_2018.f90:1288-1305), filled in any
// order here and put in ascending id order by k_cell_sort
__global__ void k_cell_fill(Dev D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N2) return;
  int c = D.cell_of[i];
  int slot = atomicAdd(&D.cell_cursor[c], 1);
  D.spos[D.cell_start[c] + slot] = i;  // spos used as scratch here
}

// per cell: sort the ids ascending (list_picell order, 2_SPH_main_2018.f90:1299-1305),
// write sorted[] and spos[]
__global__ void k_cell_sort(Dev D) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  const GridTotal g = *D.gtot;
  if (c > g.ncells) return;
  int st = D.cell_start[c], n = D.cell_cnt[c];
  for (int a = 0; a < n; a++) {
    int v = D.spos[st + a];
    int b = a - 1;
    while (b >= 0 && D.sorted[st + b] > v) {
      D.sorted[st + b + 1] = D.sorted[st + b];
      b--;
    }
    D.sorted[st + b + 1] = v;
  }
  if (c == g.ncells) D.gtot->nactive = st;
}

// sorted position of every particle, and the pair search's per-particle values in sorted
// order (the candidates of a cell are then read contiguously)
__global__ void k_spos(Dev D) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  const int t = D.sorted[s];
  D.spos[t] = s;
  D.srec[s] = make_float4(D.xr[t], D.yr[t], D.hr[t], __int_as_float(D.itype[t]));
  if (D.fast) D.srecl[s] = make_float2(D.xrl[t], D.yrl[t]);
}

// exact distance test of the reference (2_SPH_main_2018.f90:1345-1353) on the pair
// (a = creator, b); returns true and r, dx, dy, mhsml when the pair is accepted
__device__ __forceinline__ bool exact_test(const Dev& D, int a, int b, double& r, double& dx,
                                           double& dy, double& mh) {
  dx = D.px[a] - D.px[b];
  double driac = dx * dx;
  dy = D.py[a] - D.py[b];
  driac = driac + dy * dy;
  mh = (D.hsml[a] + D.hsml[b]) * 0.5;  // / 2.0, exactly
  r = sqrt(driac);
  // r < scale_k mh with the conversion and the comparison on the integer pipe (r >= 0)
  return !f64_isnan(r) && f64_key(r) < f64_key(i2d_pos(D.scale_k) * mh);
}

// 0 = reject, 1 = accept, 2 = undecided (inside the guard band).  (cx, cy) is the corner
// of b's cell relative to a's in FP32 (multiples of the cell size); fx, fy return the
// FP32 separation x_a - x_b.
__device__ __forceinline__ int prefilter(const Dev& D, float xa, float ya, float ha, float4 rb,
                                         float cx, float cy, float tau, float& fx, float& fy) {
  fx = (xa - rb.x) - cx;
  fy = (ya - rb.y) - cy;
  float d2 = fx * fx + fy * fy;
  float s = (float)D.scale_k * ((ha + rb.z) * 0.5f);
  float s2 = s * s;
  if (d2 < s2 * (1.0f - tau)) return 1;
  if (d2 > s2 * (1.0f + tau)) return 0;
  return 2;
}

// FP32 cubic / Gaussian / quintic kernel of the FP32 form (same formulas as the reference's
// kernel routine, evaluated in single precision)
__device__ __forceinline__ void sph_kernel_f32(int skf, float pi, float r, float dx0, float dx1,
                                               float h, float* w, float* dw0, float* dw1) {
  float q = r / h;
  *w = 0.0f;
  *dw0 = 0.0f;
  *dw1 = 0.0f;
  if (skf == 1) {
    float factor = 15.0f / (7.0f * pi * h * h);
    if (q <= 1.0f) {
      *w = factor * ((2.0f / 3.0f - q * q) + (q * q * q) * 0.5f);
      float a = (factor * (-2.0f + 1.5f * q)) / (h * h);
      *dw0 = a * dx0;
      *dw1 = a * dx1;
    } else if (q <= 2.0f) {
      float t = 2.0f - q;
      *w = (factor / 6.0f) * (t * t * t);
      float a = -(factor * 0.5f) * (t * t) / (h * r);
      *dw0 = a * dx0;
      *dw1 = a * dx1;
    }
  } else if (skf == 2) {
    float factor = 1.0f / (h * h * pi);
    if (q <= 3.0f) {
      *w = factor * expf(-(q * q));
      *dw0 = *w * (-2.0f * dx0 / (h * h));
      *dw1 = *w * (-2.0f * dx1 / (h * h));
    }
  } else {
    float factor = 7.0f / (478.0f * pi * h * h);
    float a = 3.0f - q, b = 2.0f - q, c1 = 1.0f - q;
    float a2 = a * a, b2 = b * b, c2 = c1 * c1;
    float a4 = a2 * a2, b4 = b2 * b2;
    float a5 = a4 * a, b5 = b4 * b, c5 = c2 * c2 * c1;
    if (q <= 1.0f) {
      *w = factor * ((a5 - 6.0f * b5) + 15.0f * c5);
      float g = factor * ((-120.0f + 120.0f * q) - 50.0f * (q * q)) / (h * h);
      *dw0 = g * dx0;
      *dw1 = g * dx1;
    } else if (q <= 2.0f) {
      *w = factor * (a5 - 6.0f * b5);
      float g = factor * (-5.0f * a4 + 30.0f * b4) / (h * r);
      *dw0 = g * dx0;
      *dw1 = g * dx1;
    } else if (q <= 3.0f) {
      *w = factor * a5;
      float g = factor * (-5.0f * a4) / (h * r);
      *dw0 = g * dx0;
      *dw1 = g * dx1;
    }
  }
}

// the reference's cubic kernel for a uniform h (2_SPH_main_2018.f90:1468-1492) for the FP32
// form: the separation, r and q = r/h in double-float, which removes the cancellations (of
// the cell-relative offsets and of 2 - q near the edge of the support), then the
// polynomial and the gradient in FP32 from the accurate q: W and dW within a few FP32 ulps
// of the FP64 evaluation
__device__ __forceinline__ void cubic_mixed(const Grid& g, dfl dx, dfl dy, float* w, float* dw0,
                                            float* dw1) {
  const dfl r = df_sqrt(df_sumsq(dx, dy));
  const dfl q = df_mul(r, g.df_yh);
  *w = 0.0f;
  *dw0 = 0.0f;
  *dw1 = 0.0f;
  if (q.hi < 1.0f || (q.hi == 1.0f && q.lo <= 0.0f)) {
    const float qh = q.hi, q2 = qh * qh;
    *w = g.df_factor.hi * ((2.0f / 3.0f - q2) + 0.5f * (q2 * qh));
    const float a = (g.df_factor.hi * (-2.0f + 1.5f * qh)) * g.df_yhh.hi;
    *dw0 = a * dx.hi;
    *dw1 = a * dy.hi;
  } else if (q.hi < 2.0f || (q.hi == 2.0f && q.lo <= 0.0f)) {
    const float t = (2.0f - q.hi) - q.lo;  // 2 - q.hi is exact
    const float t2 = t * t;
    *w = g.df_factor6.hi * (t2 * t);
    const float ar = ((g.df_c3.hi * t2) * g.df_yh.hi) / r.hi;
    *dw0 = -(ar * dx.hi);
    *dw1 = -(ar * dy.hi);
  }
}

// Pairs created by the particle at sorted position s, in the reference's creation order:
// the rest of its own cell, the cell to its right, then the three cells of the row above.
// FAST = false: W and dW from the reference's FP64 kernel, stored in FP32 (the plain
// form); FAST = true: the FP32 form's evaluation (cubic_mixed, or FP32 for a varying h).
// The pair set is the same.
// Kernel values of one accepted pair (creator a at sorted position s, partner at sorted
// position bs in stencil cell q), packed as the finished half-list entry.
template <bool FAST>
__device__ __forceinline__ int4 half_entry(const Dev& D, const Grid& g, int a, int ta, float xa,
                                           float ya, float ha, float xal, float yal, int bs,
                                           int q) {
  const int b = D.sorted[bs];
  const float cw = (float)g.deltx[0], ch = (float)g.deltx[1];
  // the stencil cell's offset (cells[q]) without indexing a local array
  const int qx = (q == 1 || q == 4) ? 1 : (q == 2 ? -1 : 0), qy = q >= 2 ? 1 : 0;
  const float cx = (float)qx * cw, cy = (float)qy * ch;
  const float4 rb = D.srec[bs];
  const float fx = (xa - rb.x) - cx, fy = (ya - rb.y) - cy;
  double r, dx, dy, mh;
  if (!FAST) exact_test(D, a, b, r, dx, dy, mh);
  float wf, d0f, d1f;
  if (!FAST) {
    double w, dw0, dw1;
    if (g.uniform_h) cubic_uniform(g, r, dx, dy, &w, &dw0, &dw1);
    else sph_kernel(D.skf, D.pi, r, dx, dy, mh, &w, &dw0, &dw1);
    wf = f32_rn(w);  // the same bits as (float), on the integer pipe
    d0f = f32_rn(dw0);
    d1f = f32_rn(dw1);
  } else if (g.uniform_h) {
    // separation as double-float from the cell-relative hi/lo offsets
    // x_a - x_b = (offset_a - offset_b) - (cell shift) with every term in double-float
    const float2 rl = D.srecl[bs];
    cubic_mixed(g, df_sep(xa, xal, rb.x, rl.x, qx, g.df_cell[0]),
                df_sep(ya, yal, rb.y, rl.y, qy, g.df_cell[1]), &wf, &d0f, &d1f);
  } else {
    float hm = (ha + rb.z) * 0.5f;
    float rf = sqrtf(fx * fx + fy * fy);
    sph_kernel_f32(D.skf, (float)D.pi, rf, fx, fy, hm, &wf, &d0f, &d1f);
  }
  const int pt = pint_type(ta, D.itype[b]);
  return make_int4((int)((unsigned)b | ((unsigned)pt << kHalfTypeShift)), __float_as_int(wf),
                   __float_as_int(d0f), __float_as_int(d1f));
}

// Phase 2 of the plain form, warp-cooperative.  The FP64 kernel values are the plain form's
// cost (FP64 pipe), and a warp whose lanes each evaluate their own creator's pairs runs as
// many iterations as its longest list with the other lanes idle (17.8 of 32 lanes active
// per instruction in the per-lane loop).  Here the warp's accepted pairs are numbered
// creator by creator (a warp scan of the counts) and evaluated 32 at a time, one per lane:
// lane l takes pair base + l, finds its creator among the warp's lanes by a binary search
// over the scanned counts, and writes the finished entry into that creator's list at the
// same place.  Every entry is computed by the same arithmetic as before.  All 32 lanes call
// this (inactive ones with kk = 0).
__device__ __forceinline__ void half_phase2_coop(const Dev& D, int s, int kk, int a, int ta,
                                                 float xa, float ya, float ha) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int incl = kk;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += v;
  }
  const int excl = incl - kk;
  const int total = __shfl_sync(full, incl, 31);
  __syncwarp();  // the phase-1 entries of every lane are visible to the others
  for (int base = 0; base < total; base += 32) {
    const int p = base + lane;
    // the last lane whose first pair is at or before p (it owns p: p < its excl + kk)
    int lo = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int e = __shfl_sync(full, excl, lo + step);
      if (e <= p) lo += step;
    }
    const int so = __shfl_sync(full, s, lo), ao = __shfl_sync(full, a, lo);
    const int tao = __shfl_sync(full, ta, lo), eo = __shfl_sync(full, excl, lo);
    const float xo = __shfl_sync(full, xa, lo), yo = __shfl_sync(full, ya, lo);
    const float ho = __shfl_sync(full, ha, lo);
    if (p < total) {
      int4* out = D.half + (size_t)so * D.capH;
      const int m = p - eo;
      const int4 e0 = out[m];
      const Grid& g = D.grid[D.rid[ao]];
      out[m] = half_entry<false>(D, g, ao, tao, xo, yo, ho, 0.0f, 0.0f, e0.x, e0.y);
    }
  }
  __syncwarp();
}

// Phase 1 for the creator at sorted position s: the accepted partners in creation order
// (sorted position, stencil cell) into its half list, its pair count and its list-build
// record.  Returns the number of entries held (at most capH) and the creator's id, type and
// FP32 cell-relative offsets.
template <bool FAST>
__device__ __forceinline__ int half_phase1(const Dev& D, int s, int& a, int& ta, float& xa,
                                           float& ya, float& ha) {
  a = D.sorted[s];
  const Grid& g = D.grid[D.rid[a]];
  const float tau = g.tau;
  int c = D.cell_of[a] - g.cell0;  // local cell in the realisation's grid
  int nx = g.ndiv[0], ny = g.ndiv[1];
  int ix = c % nx, iy = c / nx;
  xa = D.xr[a];
  ya = D.yr[a];
  ha = D.hr[a];
  ta = D.itype[a];
  const float cw = (float)g.deltx[0], ch = (float)g.deltx[1];
  int k = 0;
  int4* out = D.half + (size_t)s * D.capH;
  // stencil cells in creation order: (dix, diy) and the first sorted position to scan
  int cells[5][2] = {{0, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
  int gstart[5] = {0, 0, 0, 0, 0};  // where each stencil cell's pairs start in the list
  for (int q = 0; q < 5; q++) {
    gstart[q] = min(k, D.capH);
    int jx = ix + cells[q][0], jy = iy + cells[q][1];
    if (jx < 0 || jx >= nx || jy >= ny) continue;
    int cc = g.cell0 + jy * nx + jx;
    int lo = (q == 0) ? s + 1 : D.cell_start[cc];
    int hi = D.cell_start[cc] + D.cell_cnt[cc];
    float cx = (float)cells[q][0] * cw, cy = (float)cells[q][1] * ch;
    // the kernel values follow in phase 2, so that the lanes of a warp evaluate them
    // together instead of each time one lane accepts a candidate
    for (int bs = lo; bs < hi; bs++) {
      float fx, fy;
      int pf = prefilter(D, xa, ya, ha, D.srec[bs], cx, cy, tau, fx, fy);
      if (pf == 0) continue;
      if (pf == 2) {
        double r, dx, dy, mh;
        if (!exact_test(D, a, D.sorted[bs], r, dx, dy, mh)) continue;
      }
      if (k < D.capH) out[k] = make_int4(bs, q, 0, 0);
      k++;
    }
  }
  if (k > D.capH) {
    atomicOr(D.err, ERR_HALF_CAP);
    k = D.capH;
  }
  D.half_cnt[s] = k;
  // what the list build reads of a creator, in one 16-byte record: where its pairs with
  // stencil cells 1-4 start, its pair count and its id
  D.half_meta[s] = make_int4((int)((unsigned)gstart[1] | ((unsigned)gstart[2] << 16)),
                             (int)((unsigned)gstart[3] | ((unsigned)gstart[4] << 16)), k, a);
  return k;
}

// Task 3 of grid_find_NEW (2_SPH_main_2018.f90:1307-1403): the half-stencil search
// (:1322-1341), the exact test (:1345-1353), kernel (:1371, :1440-1538) and the pair types
// of Pint_Update (3_SPH_material_2018.f90:1574-1634).
// Phase 2 turns each accepted (partner, stencil cell) into the finished entry: the
// partner's id with the pair type in its top bits (kHalfIdMask), so that the list build
// needs neither the partner's id nor its type from memory, and W, dW/dx, dW/dy; within one
// stencil cell the entries ascend in id (a cell is sorted by id) as they do in sorted
// position.  The FP32 form's lanes each finish their own list; the plain form's warps
// share the work (half_phase2_coop), so all of a warp's lanes stay to the end.
template <bool FAST>
__global__ void k_half(Dev D) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = s < D.N2 && s < D.gtot->nactive;
  if (!active && s < D.N2) D.half_cnt[s] = 0;
  if (FAST) {
    if (!active) return;
    int a, ta;
    float xa, ya, ha;
    const int kk = half_phase1<true>(D, s, a, ta, xa, ya, ha);
    const Grid& g = D.grid[D.rid[a]];
    const float xal = D.xrl[a], yal = D.yrl[a];
    int4* out = D.half + (size_t)s * D.capH;
    for (int m = 0; m < kk; m++) {
      const int4 e0 = out[m];
      out[m] = half_entry<true>(D, g, a, ta, xa, ya, ha, xal, yal, e0.x, e0.y);
    }
  } else {
    int a = 0, ta = 0, kk = 0;
    float xa = 0.0f, ya = 0.0f, ha = 0.0f;
    if (active) kk = half_phase1<false>(D, s, a, ta, xa, ya, ha);
    half_phase2_coop(D, s, kk, a, ta, xa, ya, ha);
  }
}

// entries 2j and 2j+1 of a list column in one 32-byte store (ell(): one sector, 32-byte
// aligned), so that no sector of the lists is ever written in halves
__device__ __forceinline__ void store_pair(int4* dst, int4 a, int4 b) {
  asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(dst), "r"(a.x),
               "r"(a.y), "r"(a.z), "r"(a.w), "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w)
               : "memory");
}

// ---------------------------------------------------------------- FP32 form: direct lists
// The FP32 form builds each target's lists straight from its 3 x 3 cell stencil, without
// the half lists and the search through them.  Scanning the stencil's cells in ascending
// sorted position visits a target's partners in the reference's creation order of their
// pairs: first the creators before it (the row below, the cell to its left, its own cell
// up to it), one pair each, then its own half list (the rest of its cell, the cell to its
// right, the row above).  The lists hold that order; the FP32 form's sums use it in every
// step (the plain form's walk order reverses the newest pairs in steps where the pair
// count reaches a new maximum).
// The pair test is the same symmetric test (prefilter and exact FP64 band test), and the
// kernel values are evaluated with the target in the creator's role: the separation is
// negated exactly (double-float additions and the cell shift are sign-symmetric), so W is
// the same bits as the creator's evaluation and the gradient its exact negation.  Every
// target also counts the partners after it, which is its half-list length (half_cnt), for
// the pair count bookkeeping; dummies and inactive positions are counted by k_fgather_rest.

// the list entry of partner bs (cell offset qx, qy) of a target of type ta with FP32
// cell-relative offsets (xa, xal), (ya, yal) and smoothing length ha: {partner id, W (sign
// bit set for a dummy partner), dW/dx, dW/dy} with the gradient with respect to the target.
// f32: the kernel values in FP32 from the FP32 separation (same-kind entries that only the
// FP32 free-surface detection reads), otherwise r and r/h in double-float (cubic_mixed)
__device__ __forceinline__ int4 gather_entry(const Dev& D, const Grid& g, int ta, float xa,
                                             float ya, float ha, float xal, float yal, int bs,
                                             int qx, int qy, bool f32 = false) {
  const int b = D.sorted[bs];
  const float4 rb = D.srec[bs];
  float wf, d0f, d1f;
  if (g.uniform_h && !f32) {
    const float2 rl = D.srecl[bs];
    cubic_mixed(g, df_sep(xa, xal, rb.x, rl.x, qx, g.df_cell[0]),
                df_sep(ya, yal, rb.y, rl.y, qy, g.df_cell[1]), &wf, &d0f, &d1f);
  } else {
    // the cell shift qx * (float)deltx without conversions on the FP64 pipe
    const float cw = f32_rn(g.deltx[0]), ch = f32_rn(g.deltx[1]);
    const float cx = qx < 0 ? -cw : (qx > 0 ? cw : 0.0f);
    const float cy = qy < 0 ? -ch : (qy > 0 ? ch : 0.0f);
    const float fx = (xa - rb.x) - cx, fy = (ya - rb.y) - cy;
    const float hm = (ha + rb.z) * 0.5f;
    const float rf = sqrtf(fx * fx + fy * fy);
    sph_kernel_f32(D.skf, f32_rn(D.pi), rf, fx, fy, hm, &wf, &d0f, &d1f);
  }
  const int pt = pint_type(ta, __float_as_int(rb.w));
  const int w = __float_as_int(wf);
  return make_int4(b, (pt == 6 || pt == 9) ? (int)((unsigned)w | 0x80000000u) : w,
                   __float_as_int(d0f), __float_as_int(d1f));
}

// the accepted-partner test of the pair search, from either side of the pair
__device__ __forceinline__ bool gather_accept(const Dev& D, int a, float xa, float ya, float ha,
                                              float4 rb, int bs, float cx, float cy, float tau) {
  float fx, fy;
  const int pf = prefilter(D, xa, ya, ha, rb, cx, cy, tau, fx, fy);
  if (pf == 0) return false;
  if (pf == 2) {
    double r, dx, dy, mh;
    return exact_test(D, a, D.sorted[bs], r, dx, dy, mh);
  }
  return true;
}

// FP32 form: Task 3 of grid_find_NEW (2_SPH_main_2018.f90:1307-1403), kernel (:1440-1538)
// and Pint_Update (3_SPH_material_2018.f90:1574-1634) per target, gathering its entries
// from the 3 x 3 cell stencil directly in creation order.
// KIND 1: the stress-point targets tgt[0..n), 2: the node targets.  SAME: the same-kind
// entries are written too (the steps that read them: XSPH, artificial viscosity or stress,
// the FP32 free-surface detection); without them degS holds 0 unless the outside approach
// reads the counts.  Phase 1 tests the stencil's candidates and keeps the
// accepted ones (sorted position and cell offset) in shared memory; phase 2 evaluates the
// kernel values, so that a warp's lanes evaluate together.  Dynamic shared memory:
// (capC + SAME capS) ints per thread, entry k of thread j at k * blockDim + j.
template <int KIND, bool SAME>
__global__ void __launch_bounds__(512, 2) k_fgather(Dev D, const int32_t* __restrict__ tgt,
                                                    int ntgt) {
  extern __shared__ int gbuf[];
  const int k0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (k0 >= ntgt) return;
  const int bd = blockDim.x, tid = threadIdx.x;
  int* bufC = gbuf;
  int* bufS = gbuf + (size_t)D.capC * bd;
  const int s = tgt[k0];
  const int col = list_col<KIND>(D, k0, s);
  int nC = 0, nS = 0, nHalf = 0;
  if (s < D.gtot->nactive) {
    const int a = D.sorted[s];
    const int ta = D.itype[a];
    const Grid& g = D.grid[D.rid[a]];
    const float tau = g.tau;
    const int c = D.cell_of[a] - g.cell0;
    const int nx = g.ndiv[0], ny = g.ndiv[1];
    const int ix = c % nx, iy = c / nx;
    const float xa = D.xr[a], ya = D.yr[a], ha = D.hr[a];
    const float cw = (float)g.deltx[0], ch = (float)g.deltx[1];
    // same-kind partners before the target matter only for the full same-kind count
    // (the same lists, or the outside approach's isolated-node test); otherwise only the
    // ones after it are tested, for the half-list count
    const bool all_same = SAME || D.outside;
    // a uniform smoothing length makes the prefilter's bounds constant (the same FP32
    // expressions as prefilter(), so the same decisions)
    float s2lo = 0.0f, s2hi = 0.0f;
    if (g.uniform_h) {
      const float sv = (float)D.scale_k * ((ha + ha) * 0.5f);
      const float s2 = sv * sv;
      s2lo = s2 * (1.0f - tau);
      s2hi = s2 * (1.0f + tau);
    }
    // the stencil row by row: a row's three cells are one contiguous run of sorted
    // positions; a candidate's cell follows from the run's cell boundaries
    for (int qy = -1; qy <= 1; qy++) {
      const int jy = iy + qy;
      if (jy < 0 || jy >= ny) continue;
      const int row0 = g.cell0 + jy * nx;
      const int cr = row0 + (ix + 1 < nx ? ix + 1 : ix);
      const int lo = D.cell_start[row0 + (ix > 0 ? ix - 1 : 0)];
      const int hi = D.cell_start[cr] + D.cell_cnt[cr];
      const int b0 = D.cell_start[row0 + ix];                         // the centre cell
      const int b1 = ix + 1 < nx ? D.cell_start[row0 + ix + 1] : hi;  // the right cell
      const float cy = qy < 0 ? -ch : (qy > 0 ? ch : 0.0f);  // (float)qy * ch
      for (int bs = lo; bs < hi; bs++) {
        if (bs == s) continue;
        const float4 rb = D.srec[bs];
        const bool same = __float_as_int(rb.w) == ta;
        if (same && !all_same && bs < s) continue;
        const int qx = bs < b0 ? -1 : (bs < b1 ? 0 : 1);
        const float cx = qx < 0 ? -cw : (qx > 0 ? cw : 0.0f);  // (float)qx * cw
        bool acc;
        if (g.uniform_h) {
          const float fx = (xa - rb.x) - cx, fy = (ya - rb.y) - cy;
          const float d2 = fx * fx + fy * fy;
          if (d2 > s2hi) continue;
          acc = d2 < s2lo;
          if (!acc) {
            double r, dx, dy, mh;
            acc = exact_test(D, a, D.sorted[bs], r, dx, dy, mh);
          }
        } else {
          acc = gather_accept(D, a, xa, ya, ha, rb, bs, cx, cy, tau);
        }
        if (!acc) continue;
        nHalf += bs > s;
        const int code = (qy + 1) * 3 + (qx + 1);  // cell offset, kept in the top 4 bits
        if (same) {
          if (SAME && nS < D.capS) bufS[(size_t)nS * bd + tid] = bs | (code << kHalfTypeShift);
          nS++;
        } else {
          if (nC < D.capC) bufC[(size_t)nC * bd + tid] = bs | (code << kHalfTypeShift);
          nC++;
        }
      }
    }
    if (!all_same) nS = 0;  // not counted: no step kernel reads the same-kind lists or counts
    if (nHalf > D.capH) {
      atomicOr(D.err, ERR_HALF_CAP);
      nHalf = D.capH;
    }
    if (nC > D.capC || nS > D.capS) {
      atomicOr(D.err, ERR_LIST_CAP);
      nC = min(nC, D.capC);
      nS = min(nS, D.capS);
    }
    const float xal = D.xrl[a], yal = D.yrl[a];
    // phase 2: the entries, stored in pairs (whole 32-byte sectors)
    auto finish = [&](const int* buf, int n, int4* list, int2* compact, bool f32) {
      int4 pend = make_int4(0, 0, 0, 0);
      for (int k = 0; k < n; k++) {
        const unsigned v = (unsigned)buf[(size_t)k * bd + tid];
        const int code = (int)(v >> kHalfTypeShift);
        const int4 e = gather_entry(D, g, ta, xa, ya, ha, xal, yal, (int)(v & kHalfIdMask),
                                    code % 3 - 1, code / 3 - 1, f32);
        if (k & 1) store_pair(list + ell(k - 1, col, D.N2), pend, e);
        else pend = e;
        // the lanes of a warp write entry k of adjacent columns together: whole sectors
        if (compact) compact[(size_t)k * D.N2 + col] = make_int2(e.x, e.y);
      }
      if (n & 1) list[ell(n - 1, col, D.N2)] = pend;
    };
    finish(bufC, nC, D.cross, D.use_crossW ? D.crossW : nullptr, false);
    // same-kind entries that no step kernel reads serve the FP32 free-surface detection
    // only: FP32 kernel values
    if (SAME) finish(bufS, nS, D.same, nullptr, !D.same_entries);
  }
  D.degC[col] = nC;
  D.degS[col] = nS;
  D.half_cnt[s] = nHalf;
}

// every sorted position that is not a stress-point or node target: the half-list length
// of an active dummy (its pairs with the particles after it in its half stencil), zero
// counts for inactive positions and dummies' list columns
__global__ void k_fgather_rest(Dev D) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  const int a = D.sorted[s];
  if (a < D.NT) return;  // a stress-point or node target: k_fgather
  const int col = D.lcol[s];
  D.degC[col] = 0;
  D.degS[col] = 0;
  int k = 0;
  if (s < D.gtot->nactive) {
    const Grid& g = D.grid[D.rid[a]];
    const int c = D.cell_of[a] - g.cell0;
    const int nx = g.ndiv[0], ny = g.ndiv[1];
    const int ix = c % nx, iy = c / nx;
    const float xa = D.xr[a], ya = D.yr[a], ha = D.hr[a];
    const float cw = (float)g.deltx[0], ch = (float)g.deltx[1];
    const int cells[5][2] = {{0, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
    for (int q = 0; q < 5; q++) {
      const int jx = ix + cells[q][0], jy = iy + cells[q][1];
      if (jx < 0 || jx >= nx || jy >= ny) continue;
      const int cc = g.cell0 + jy * nx + jx;
      const int lo = q == 0 ? s + 1 : D.cell_start[cc];
      const int hi = D.cell_start[cc] + D.cell_cnt[cc];
      const float cx = (float)cells[q][0] * cw, cy = (float)cells[q][1] * ch;
      for (int bs = lo; bs < hi; bs++)
        k += gather_accept(D, a, xa, ya, ha, D.srec[bs], bs, cx, cy, g.tau);
    }
    if (k > D.capH) {
      atomicOr(D.err, ERR_HALF_CAP);
      k = D.capH;
    }
  }
  D.half_cnt[s] = k;
}

// pair counts of every realisation (its pairs are the half lists of its sorted range)
__global__ void k_pair_meta(Dev D) {
  const GridTotal gt = *D.gtot;
  for (int r = threadIdx.x; r < D.R; r += blockDim.x) {
    const Grid& g = D.grid[r];
    int64_t lo = 0, hi = 0;
    if (!gt.overflow) {
      lo = D.half_off[D.cell_start[g.cell0]];
      hi = D.half_off[D.cell_start[g.cell0 + g.ncells]];
    }
    PairMeta m = D.meta[r];
    m.m_prev = m.m;
    m.n = hi - lo;
    m.base = lo;
    if (m.n > m.m) m.m = m.n;
    D.meta[r] = m;
  }
  // walk-order keys hold 2 x position in 32 bits
  if (threadIdx.x == 0 && D.half_off[D.N2] > 1073741823LL) atomicOr(D.err, ERR_NPAIRS);
}

template <bool KEYS>
__device__ __forceinline__ void reverse_ell(int4* base, int32_t* key, int N2, int col, int lo,
                                            int hi) {
  // reverse entries [lo, hi) of list column col (and their keys)
  hi--;
  while (lo < hi) {
    int4 t = base[ell(lo, col, N2)];
    base[ell(lo, col, N2)] = base[ell(hi, col, N2)];
    base[ell(hi, col, N2)] = t;
    if (KEYS) {
      int32_t k = key[(size_t)lo * N2 + col];
      key[(size_t)lo * N2 + col] = key[(size_t)hi * N2 + col];
      key[(size_t)hi * N2 + col] = k;
    }
    lo++;
    hi--;
  }
}

// Per-target lists.  The pairs a target t meets, in creation order, are: first the pairs
// created by particles before t in sorted order (each holds t in its half list), then
// t's own half list.  The linked list of the reference is walked as: pairs created this
// step beyond the previous list length m (newest first), then pairs 0..m-1 in creation
// order; the lists are written in that walk order.
// KEYS: also write the walk-order key of every entry (for the free-surface detection)
template <bool KEYS>
__device__ __forceinline__ void lists_target(const Dev& D, int s, int4& pendC, int4& pendS) {
  int nC = 0, nS = 0, newC = 0, newS = 0;
  const int col = D.lcol[s];
  if (s < D.gtot->nactive) {
    int t = D.sorted[s];
    int tt = D.itype[t];
    if (!is_dummy(tt)) {
      const int r = D.rid[t];
      const Grid& g = D.grid[r];
      const PairMeta meta = D.meta[r];
      const bool reorder = meta.n > meta.m_prev;
      const int c0g = g.cell0;
      int c = D.cell_of[t] - c0g;  // local cell
      int nx = g.ndiv[0];
      int ix = c % nx, iy = c / nx;
      int lo[2], hi[2];
      if (iy > 0) {
        int c0 = c0g + (iy - 1) * nx + (ix > 0 ? ix - 1 : 0);
        int c1 = c0g + (iy - 1) * nx + (ix + 1 < nx ? ix + 1 : ix);
        lo[0] = D.cell_start[c0];
        hi[0] = D.cell_start[c1] + D.cell_cnt[c1];
      } else {
        lo[0] = hi[0] = 0;
      }
      lo[1] = D.cell_start[c0g + (ix > 0 ? c - 1 : c)];
      hi[1] = s;
      // key of an entry: its position in the walk order of the realisation's list, and
      // whether the target is pair_i (creator of a same-type pair; the stress-point of a
      // node--stress-point pair)
      auto push = [&](int u, int pt, int w, float gx, float gy, int64_t cidx, bool own) {
        bool same = (pt == 2 || pt == 3);
        // a wall (dummy) partner (pair types 6 and 9 of a non-dummy target) is marked by the
        // sign bit of W (W >= 0): readers skip or branch on it without loading its type
        int4 e = make_int4(u, (pt == 6 || pt == 9) ? (int)((unsigned)w | 0x80000000u) : w,
                           __float_as_int(gx), __float_as_int(gy));
        const int64_t rel = cidx - meta.base;
        bool isnew = reorder && rel >= meta.m_prev;
        int64_t wp = !reorder ? rel : isnew ? meta.n - 1 - rel : (meta.n - meta.m_prev) + rel;
        int role = same ? (own ? 1 : 0) : (pt == 1 && is_sp(tt) ? 1 : 0);
        int32_t key = (int32_t)(2 * wp + role);
        // an even entry waits in pendS / pendC for its odd partner, and the two are stored
        // together; a last even entry is stored alone after the walk
        if (same) {
          if (nS < D.capS && (KEYS || D.same_entries)) {
            if (nS & 1) store_pair(D.same + ell(nS - 1, col, D.N2), pendS, e);
            else pendS = e;
            if (KEYS) D.keyS[(size_t)nS * D.N2 + col] = key;
          }
          nS++;
          newS += isnew;
        } else if (pt != 0) {
          if (nC < D.capC) {
            if (nC & 1) store_pair(D.cross + ell(nC - 1, col, D.N2), pendC, e);
            else pendC = e;
            if (KEYS) D.keyC[(size_t)nC * D.N2 + col] = key;
          }
          nC++;
          newC += isnew;
        }
      };
      // the creators before s, in ascending sorted position: each holds s at most once in
      // its (ascending) half list, among the pairs it made with s's cell, whose place in
      // the list k_half recorded (half_meta: the starts of its five stencil cells).  The
      // stencil cell of s seen from a creator follows from the creator's cell: below-left,
      // below, below-right (region 0), left, own (region 1).  kG lower-bound searches run
      // interleaved, so that their dependent loads overlap; the hits are pushed in creator
      // order.
      constexpr int kG = 4;
      const int n0 = hi[0] - lo[0], ncand = n0 + (hi[1] - lo[1]);
      const int rowb = c0g + (iy - 1) * nx;  // first cell of the row below
      const int b1 = iy > 0 ? D.cell_start[rowb + ix] : 0;  // the cell below s's cell
      const int b2 = (iy > 0 && ix + 1 < nx) ? D.cell_start[rowb + ix + 1] : hi[0];
      const int own0 = D.cell_start[c0g + c];
      for (int i0 = 0; i0 < ncand; i0 += kG) {
        int as[kG], pos[kG], len[kG], cnt[kG], cid[kG];
        int4 mt[kG];
#pragma unroll
        for (int q = 0; q < kG; q++) {
          const int i = i0 + q;
          as[q] = i < n0 ? lo[0] + i : lo[1] + (i - n0);
          mt[q] = i < ncand ? D.half_meta[as[q]] : make_int4(0, 0, 0, 0);
          cnt[q] = mt[q].z;
          cid[q] = mt[q].w;
        }
#pragma unroll
        for (int q = 0; q < kG; q++) {
          const int i = i0 + q;
          const unsigned g12 = (unsigned)mt[q].x, g34 = (unsigned)mt[q].y;
          const int gs[6] = {0, (int)(g12 & 0xFFFFu), (int)(g12 >> 16), (int)(g34 & 0xFFFFu),
                             (int)(g34 >> 16), cnt[q]};
          // stencil cell of s from the creator: 0 own, 1 right, 2 up-left, 3 up, 4 up-right
          const int st = i < n0 ? (as[q] < b1 ? 4 : as[q] < b2 ? 3 : 2) : (as[q] < own0 ? 1 : 0);
          const int g0 = st == 0 ? gs[0] : st == 1 ? gs[1] : st == 2 ? gs[2] : st == 3 ? gs[3] : gs[4];
          const int g1 = st == 0 ? gs[1] : st == 1 ? gs[2] : st == 2 ? gs[3] : st == 3 ? gs[4] : gs[5];
          pos[q] = g0;
          len[q] = i < ncand ? max(g1 - g0, 0) : 0;
        }
        bool more = true;
        while (more) {
          int v[kG];
#pragma unroll
          for (int q = 0; q < kG; q++)
            v[q] = len[q] > 0 ? (int)((unsigned)D.half[(size_t)as[q] * D.capH + pos[q] +
                                                       (len[q] >> 1)].x & kHalfIdMask)
                              : 0;
          more = false;
#pragma unroll
          for (int q = 0; q < kG; q++)
            if (len[q] > 0) {
              const int half = len[q] >> 1;
              if (v[q] < t) {
                pos[q] += half + 1;
                len[q] -= half + 1;
              } else {
                len[q] = half;
              }
              more |= len[q] > 0;
            }
        }
#pragma unroll
        for (int q = 0; q < kG; q++)
          if (pos[q] < cnt[q]) {
            const int4 e = D.half[(size_t)as[q] * D.capH + pos[q]];
            if ((int)((unsigned)e.x & kHalfIdMask) == t)
              push(cid[q], (int)((unsigned)e.x >> kHalfTypeShift), e.y,
                   -__int_as_float(e.z), -__int_as_float(e.w), D.half_off[as[q]] + pos[q], false);
          }
      }
      {
        int n = D.half_cnt[s];
        const int4* h = D.half + (size_t)s * D.capH;
        for (int k = 0; k < n; k++) {
          int4 e = h[k];
          push((int)((unsigned)e.x & kHalfIdMask), (int)((unsigned)e.x >> kHalfTypeShift), e.y,
               __int_as_float(e.z), __int_as_float(e.w), D.half_off[s] + k, true);
        }
      }
      {
        const int wc = min(nC, D.capC), ws = min(nS, D.capS);
        if (wc & 1) D.cross[ell(wc - 1, col, D.N2)] = pendC;
        if ((ws & 1) && (KEYS || D.same_entries)) D.same[ell(ws - 1, col, D.N2)] = pendS;
      }
      if (nC > D.capC || nS > D.capS) {
        atomicOr(D.err, ERR_LIST_CAP);
        nC = min(nC, D.capC);
        nS = min(nS, D.capS);
        newC = newS = 0;
      }
      // walk order: [new entries, descending creation] + [old entries, ascending]
      if (newC > 0) {
        reverse_ell<KEYS>(D.cross, D.keyC, D.N2, col, 0, nC);
        reverse_ell<KEYS>(D.cross, D.keyC, D.N2, col, newC, nC);
      }
      if (newS > 0 && (KEYS || D.same_entries)) {
        reverse_ell<KEYS>(D.same, D.keyS, D.N2, col, 0, nS);
        reverse_ell<KEYS>(D.same, D.keyS, D.N2, col, newS, nS);
      }
    }
  }
  D.degC[col] = nC;
  D.degS[col] = nS;
}

// every target's cross and same lists, built from the creators' half lists in the walk
// order of the reference's pair linked list (its reuse and relinking,
// 2_SPH_main_2018.f90:1309-1401).
// dynamic shared memory: 2 x blockDim int4, the waiting even entries of each thread's two
// lists (in registers they cost the list build, which waits on its gathers, an eighth of
// its resident warps)
template <bool KEYS>
__global__ void k_lists(Dev D) {
  extern __shared__ int4 lists_pend[];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < D.N2)
    lists_target<KEYS>(D, s, lists_pend[threadIdx.x], lists_pend[blockDim.x + threadIdx.x]);
}

// ------------------------------------------------------------------------ scans
template <typename TI, typename TO>
__global__ void k_scan_blocks(const TI* in, TO* out, TO* bsum, int n, int per_block) {
  // each block scans per_block elements (per_block = blockDim.x * items)
  __shared__ TO sh[kBlock];
  int base = blockIdx.x * per_block;
  int items = per_block / blockDim.x;
  int i0 = base + threadIdx.x * items;
  TO local = 0;
  for (int k = 0; k < items; k++) {
    int i = i0 + k;
    if (i < n) local += (TO)in[i];
  }
  sh[threadIdx.x] = local;
  __syncthreads();
  for (int o = 1; o < blockDim.x; o <<= 1) {
    TO v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += v;
    __syncthreads();
  }
  TO run = sh[threadIdx.x] - local;  // exclusive prefix of this thread
  for (int k = 0; k < items; k++) {
    int i = i0 + k;
    if (i < n) {
      out[i] = run;
      run += (TO)in[i];
    }
  }
  if (threadIdx.x == blockDim.x - 1) bsum[blockIdx.x] = sh[threadIdx.x];
}

template <typename TO>
__global__ void k_scan_top(TO* bsum, int nb, TO* total) {
  // single block: exclusive scan of block sums (sequential chunks of blockDim)
  __shared__ TO sh[kBlock];
  __shared__ TO carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += blockDim.x) {
    int i = base + threadIdx.x;
    TO v = i < nb ? bsum[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < blockDim.x; o <<= 1) {
      TO u = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += u;
      __syncthreads();
    }
    if (i < nb) bsum[i] = sh[threadIdx.x] - v + carry;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += sh[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

template <typename TO>
__global__ void k_scan_add(TO* out, const TO* bsum, int n, int per_block) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += bsum[i / per_block];
}

template <typename TI, typename TO>
void scan_impl(Ctx& c, const TI* in, TO* out, int n) {
  const int per_block = kBlock * 16;
  int nb = (n + per_block - 1) / per_block;
  TO* bsum = reinterpret_cast<TO*>(c.d.scan_tmp);
  k_scan_blocks<TI, TO><<<nb, kBlock, 0, c.stream>>>(in, out, bsum, n, per_block);
  k_scan_top<TO><<<1, kBlock, 0, c.stream>>>(bsum, nb, out + n);
  k_scan_add<TO><<<(n + kBlock - 1) / kBlock, kBlock, 0, c.stream>>>(out, bsum, n, per_block);
}

}  // namespace

void scan_i32_to_i32(Ctx& c, const int32_t* in, int32_t* out, int n) { scan_impl(c, in, out, n); }
void scan_i32_to_i64(Ctx& c, const int32_t* in, int64_t* out, int n) { scan_impl(c, in, out, n); }

// flags (stress-point, node) of every sorted position, for the compaction below
__global__ void k_target_flags(Dev D) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  int t = D.sorted[s];
  D.tflag[s] = (t >= D.NN && t < D.NT) ? 1 : 0;
  D.tflag[D.N2 + s] = t < D.NN ? 1 : 0;
}
__global__ void k_target_scatter(Dev D) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.N2) return;
  const int a = D.toff[s], b = D.toff[D.N2 + 1 + s];  // stress-points, nodes before s
  int col;
  if (D.tflag[s]) {
    D.tgtS[a] = s;
    col = a;
  } else if (D.tflag[D.N2 + s]) {
    D.tgtN[b] = s;
    col = (D.NT - D.NN) + b;
  } else {
    col = D.NT + (s - a - b);
  }
  D.lcol[s] = col;
}

// per-target lists (k_lists), one thread per sorted position; keys: with the walk-order
// keys (and the same-kind entries); same: the same-kind entries even when no step kernel
// reads them (the FP32 free-surface detection does)
void launch_lists(Ctx& c, bool keys, bool same = false) {
  Dev D = c.d;
  if (same) D.same_entries = 1;
  const size_t pend = 2 * sizeof(int4) * (size_t)c.blk[TK_LISTS];
  if (keys) k_lists<true><<<c.grid_of(TK_LISTS, D.N2), c.blk[TK_LISTS], pend, c.stream>>>(D);
  else k_lists<false><<<c.grid_of(TK_LISTS, D.N2), c.blk[TK_LISTS], pend, c.stream>>>(D);
}

// the targets split by kind: their sorted positions (tgtS, tgtN) and every position's list
// column (lcol)
void split_targets(Ctx& c) {
  const Dev& D = c.d;
  const int nb = (D.N2 + kBlock - 1) / kBlock;
  k_target_flags<<<nb, kBlock, 0, c.stream>>>(D);
  scan_i32_to_i32(c, D.tflag, D.toff, D.N2);
  scan_i32_to_i32(c, D.tflag + D.N2, D.toff + D.N2 + 1, D.N2);
  k_target_scatter<<<nb, kBlock, 0, c.stream>>>(D);
}

// FP32 form: the lists straight from the cell stencil (k_fgather, one launch per target
// kind) and the remaining positions' counts; the block size is the tuned pair-search size,
// lowered until each thread's candidate lists fit 48 KB of shared memory
void launch_gather(Ctx& c, bool same, const Dev& D) {
  const size_t per_thread = sizeof(int) * (size_t)(D.capC + (same ? D.capS : 0));
  int b = std::min(c.blk[TK_HALF], 512);  // k_fgather's launch bounds
  while (b > 32 && per_thread * (size_t)b > 49152) b >>= 1;
  const size_t sm = per_thread * (size_t)b;
  const int ns = D.NT - D.NN;
  c.kernels_launched += 2;
  if (same) {
    if (ns > 0) k_fgather<1, true><<<(ns + b - 1) / b, b, sm, c.stream>>>(D, D.tgtS, ns);
    if (D.NN > 0) k_fgather<2, true><<<(D.NN + b - 1) / b, b, sm, c.stream>>>(D, D.tgtN, D.NN);
  } else {
    if (ns > 0) k_fgather<1, false><<<(ns + b - 1) / b, b, sm, c.stream>>>(D, D.tgtS, ns);
    if (D.NN > 0) k_fgather<2, false><<<(D.NN + b - 1) / b, b, sm, c.stream>>>(D, D.tgtN, D.NN);
  }
  k_fgather_rest<<<(D.N2 + kBlock - 1) / kBlock, kBlock, 0, c.stream>>>(D);
}

int launch_pair_build(Ctx& c) {
  Dev& D = c.d;
  cudaStream_t st = c.stream;
  int nb = (D.N2 + kBlock - 1) / kBlock;
  c.mark("bbox");
  k_bbox<<<nb, kBlock, 0, st>>>(D);
  c.mark("grid");
  k_grid<<<1, kBlock, 0, st>>>(D);
  c.mark("cell_count");
  cudaMemsetAsync(D.cell_cnt, 0, sizeof(int32_t) * (D.cell_cap + 2), st);
  cudaMemsetAsync(D.cell_cursor, 0, sizeof(int32_t) * (D.cell_cap + 2), st);
  k_cell_count<<<nb, kBlock, 0, st>>>(D);
  c.mark("scan_cells", 3);
  scan_i32_to_i32(c, D.cell_cnt, D.cell_start, D.cell_cap + 1);
  c.mark("cell_fill");
  k_cell_fill<<<nb, kBlock, 0, st>>>(D);
  c.mark("cell_sort");
  k_cell_sort<<<(D.cell_cap + 1 + kBlock - 1) / kBlock, kBlock, 0, st>>>(D);
  c.mark("spos");
  k_spos<<<nb, kBlock, 0, st>>>(D);
  // variant bit 2: a download follows most steps; the exact detection wants the keys, the
  // FP32 detection only the same-kind entries
  const bool want = (c.step_variant & 4) != 0;
  if (c.lists_direct()) {
    c.mark("split_targets", 8);
    split_targets(c);
    c.mark("gather");
    launch_gather(c, D.same_entries || want, D);
    c.mark("scan_half", 3);
    scan_i32_to_i64(c, D.half_cnt, D.half_off, D.N2);
    c.mark("pair_meta");
    k_pair_meta<<<1, 128, 0, st>>>(D);
    c.half_stale = true;
    return 0;
  }
  c.mark("half");
  if (c.precision == SPS_PREC_FP32_FAST)
    k_half<true><<<c.grid_of(TK_HALF, D.N2), c.blk[TK_HALF], 0, st>>>(D);
  else k_half<false><<<c.grid_of(TK_HALF, D.N2), c.blk[TK_HALF], 0, st>>>(D);
  c.mark("scan_half", 3);
  scan_i32_to_i64(c, D.half_cnt, D.half_off, D.N2);
  c.mark("pair_meta");
  k_pair_meta<<<1, 128, 0, st>>>(D);
  c.mark("split_targets", 8);
  split_targets(c);
  c.mark("lists");
  launch_lists(c, c.surf_every || (want && !c.surface_f32()), want);
  c.half_stale = false;
  return 0;
}

// The device view of the last pair build for a rebuild after the step: the FP64 positions
// the build's exact band test read (x0x, x0y hold them from the step's start, before
// anything moved; the smoothing lengths are constant when the lists are gathered), so the
// rebuild decides every pair as the build did.  The cell-frame offsets and sorted records
// are the build's own.
Dev build_view(const Ctx& c) {
  Dev D = c.d;
  D.px = D.x0x;
  D.py = D.x0y;
  return D;
}

// the half lists of the last pair build, when it gathered the lists directly (the FP32
// form): the same pairs, counts and creation order
void ensure_half_lists(Ctx& c) {
  if (!c.half_stale) return;
  k_half<true><<<c.grid_of(TK_HALF, c.d.N2), c.blk[TK_HALF], 0, c.stream>>>(build_view(c));
  c.half_stale = false;
}

// the lists of the last step again, now with their walk-order keys (the on-demand
// free-surface detection; the lists are rebuilt identically)
void launch_lists_keys(Ctx& c) {
  ensure_half_lists(c);
  launch_lists(c, true);
}

// the lists of the last step again with the same-kind entries (the FP32 detection)
void launch_lists_same(Ctx& c) {
  if (c.lists_direct() && c.half_stale) launch_gather(c, true, build_view(c));
  else launch_lists(c, false, true);
}

}  // namespace sps
