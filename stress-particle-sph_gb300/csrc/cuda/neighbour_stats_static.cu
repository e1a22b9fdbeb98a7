// neighbour_stats_static.cu -- sps_neighbour_stats_static: for every particle of a set, the
// number of partners the step's pair test accepts and the sum of their FP32 kernel values,
// computed without allocating device memory.
//
// It is a variant of the step's neighbour search (cell binning + the exact pair test of
// 2_SPH_main_2018.f90:1345-1353, kernel of 2_SPH_main_2018.f90:1458-1560 stored in FP32),
// meant for callers that cannot call cudaMalloc: hosts whose device memory is all reserved
// by their own pool allocator (a caching allocator that has claimed the device's free
// memory, so that a further cudaMalloc fails although the pool has room), and loops with a
// latency bound that may not take the device-wide synchronisation cudaMalloc and cudaFree
// can imply.  A caller uses it to check a particle configuration, e.g. the neighbour count
// that sizes sps_params.max_neighbours, before (or without) creating a context.
//
// All device scratch -- the copied positions and smoothing lengths, the cell arrays, the
// per-particle results -- lives in one file-scope array of SPS_STATIC_SCRATCH_BYTES in this
// library's device code.  No call allocates device memory, through the runtime or any
// library.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.cuh"

namespace {

constexpr int kMaxP = SPS_STATIC_MAX_PARTICLES;
constexpr int kMaxC = SPS_STATIC_MAX_CELLS;
constexpr int kBlock = 256;
constexpr int kScanThreads = 1024;

constexpr size_t up256(size_t b) { return (b + 255) & ~size_t(255); }
// byte offsets of the scratch regions (each 256-byte aligned)
constexpr size_t kOffX = 0;                                              // double x[2][kMaxP]
constexpr size_t kOffH = kOffX + up256(sizeof(double) * 2 * kMaxP);     // double h[kMaxP]
constexpr size_t kOffCell = kOffH + up256(sizeof(double) * kMaxP);      // int cell[kMaxP]
constexpr size_t kOffSorted = kOffCell + up256(sizeof(int) * kMaxP);    // int sorted[kMaxP]
constexpr size_t kOffDeg = kOffSorted + up256(sizeof(int) * kMaxP);     // int degree[kMaxP]
constexpr size_t kOffWsum = kOffDeg + up256(sizeof(int) * kMaxP);       // double wsum[kMaxP]
constexpr size_t kOffCnt = kOffWsum + up256(sizeof(double) * kMaxP);    // int cnt[kMaxC]
constexpr size_t kOffFill = kOffCnt + up256(sizeof(int) * kMaxC);       // int fill[kMaxC]
constexpr size_t kOffStart = kOffFill + up256(sizeof(int) * kMaxC);     // int start[kMaxC]
constexpr size_t kScratchBytes = kOffStart + up256(sizeof(int) * kMaxC);
static_assert(kScratchBytes == SPS_STATIC_SCRATCH_BYTES, "scratch layout and header disagree");

// The scratch shared by every call on a device.  Host code never takes this symbol as a
// device address: the address comes from cudaGetSymbolAddress (scratch_on_current_device).
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;  // serialises calls: they share g_scratch

// The device address of g_scratch in the current device's context, looked up on every call
// (cheap once this library's device code is loaded there): an address kept from an earlier
// call would be stale after the context was reset (cudaDeviceReset), since the module is
// then loaded again.  The first lookup on a device may load the device code.  Called with
// g_mu held.
cudaError_t scratch_on_current_device(unsigned char** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<unsigned char*>(p);
  return cudaSuccess;
}

// cell of each particle: the step's grid (grid_find_NEW, 2_SPH_main_2018.f90:1230-1300),
// whose cells are 2 hmax wide
__global__ void k_st_cells(int n, const double* x, double gx0, double gy0, double cs, int nx,
                           int ny, int* cell, int* cnt) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  double qx = (x[2 * a] - gx0) / cs + 1.0;
  double qy = (x[2 * a + 1] - gy0) / cs + 1.0;
  int ix = (qx >= 1.0) ? (qx < (double)nx ? (int)qx : nx) : 1;
  int iy = (qy >= 1.0) ? (qy < (double)ny ? (int)qy : ny) : 1;
  int c = nx * (iy - 1) + (ix - 1);
  cell[a] = c;
  atomicAdd(&cnt[c], 1);
}

// exclusive scan of the ncell cell counts by one block
__global__ void k_st_scan(int ncell, const int* cnt, int* start) {
  __shared__ int part[kScanThreads];
  const int t = threadIdx.x;
  const int per = (ncell + kScanThreads - 1) / kScanThreads;
  const int lo = min(t * per, ncell), hi = min(lo + per, ncell);
  int s = 0;
  for (int i = lo; i < hi; i++) s += cnt[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < kScanThreads; off <<= 1) {
    int v = (t >= off) ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = part[t] - s;
  for (int i = lo; i < hi; i++) {
    start[i] = run;
    run += cnt[i];
  }
}

__global__ void k_st_fill(int n, const int* cell, const int* start, int* fill, int* sorted) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  int c = cell[a];
  sorted[start[c] + atomicAdd(&fill[c], 1)] = a;
}

// one thread per particle: the 3 x 3 cells around its own, the reference's FP64 pair test,
// the kernel value rounded to FP32 as the step stores it.  Like the step, only adjacent
// cells are searched: with a kernel of support 3h (skf 2, 3) partners more than one cell
// away are not paired.
__global__ void k_st_stats(int n, const double* x, const double* h, int skf, double pi,
                           double scale_k, int nx, int ny, const int* cell, const int* start,
                           const int* cnt, const int* sorted, int* degree, double* wsum) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const double xa = x[2 * a], ya = x[2 * a + 1], ha = h[a];
  const int c = cell[a], ix = c % nx, iy = c / nx;
  int deg = 0;
  double ws = 0.0;
  for (int jy = max(iy - 1, 0); jy <= min(iy + 1, ny - 1); jy++)
    for (int jx = max(ix - 1, 0); jx <= min(ix + 1, nx - 1); jx++) {
      const int cc = jy * nx + jx;
      for (int k = start[cc], e = start[cc] + cnt[cc]; k < e; k++) {
        const int b = sorted[k];
        if (b == a) continue;
        double dx = xa - x[2 * b];
        double driac = dx * dx;
        double dy = ya - x[2 * b + 1];
        driac = driac + dy * dy;
        double mh = (ha + h[b]) / 2.0;
        double r = sqrt(driac);
        if (!(r < scale_k * mh)) continue;
        double w, d0, d1;
        sps::sph_kernel(skf, pi, r, dx, dy, mh, &w, &d0, &d1);
        deg++;
        ws += (double)(float)w;
      }
    }
  degree[a] = deg;
  wsum[a] = ws;
}

int say(char* msg, int32_t len, int rc, const char* fmt, ...) {
  if (msg && len > 0) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(msg, (size_t)len, fmt, ap);
    va_end(ap);
  }
  return rc;
}

}  // namespace

extern "C" int sps_neighbour_stats_static(int32_t n, const double* x, const double* hsml,
                                          int32_t skf, double pi, void* stream,
                                          int32_t* degree, double* wsum, int64_t* npairs,
                                          char* msg, int32_t msg_len) {
  if (msg && msg_len > 0) msg[0] = '\0';
  if (!npairs || n < 0 || (n > 0 && (!x || !hsml || !degree || !wsum)))
    return say(msg, msg_len, SPS_ERR_ARG,
               "sps_neighbour_stats_static: a required pointer is NULL or n < 0 (n = %d)", n);
  if (skf < 1 || skf > 3)
    return say(msg, msg_len, SPS_ERR_ARG, "sps_neighbour_stats_static: unknown kernel skf = %d",
               skf);
  if (n > kMaxP)
    return say(msg, msg_len, SPS_ERR_CAPACITY,
               "sps_neighbour_stats_static: n = %d particles exceeds the fixed device scratch "
               "(at most %d particles)",
               n, kMaxP);
  *npairs = 0;
  if (n == 0) return SPS_OK;

  // the step's grid on the host, from the host arrays, with the step's arithmetic
  double xmin = x[0], xmax = x[0], ymin = x[1], ymax = x[1], hmax = 0.0;
  for (int a = 0; a < n; a++) {
    double px = x[2 * a], py = x[2 * a + 1], ha = hsml[a];
    if (!std::isfinite(px) || !std::isfinite(py) || !std::isfinite(ha) || !(ha > 0.0))
      return say(msg, msg_len, SPS_ERR_ARG,
                 "sps_neighbour_stats_static: non-finite position or non-positive smoothing "
                 "length (particle %d)",
                 a);
    xmin = std::min(xmin, px);
    xmax = std::max(xmax, px);
    ymin = std::min(ymin, py);
    ymax = std::max(ymax, py);
    hmax = std::max(hmax, ha);
  }
  const double scale_k = skf == 1 ? 2.0 : 3.0;
  const double cs = hmax * 2.0;
  const double lo[2] = {xmin, ymin}, hi[2] = {xmax, ymax};
  double g0[2];
  int ndiv[2];
  for (int d = 0; d < 2; d++) {
    double length = hi[d] - lo[d];
    double qd = length / cs + 1.0;
    ndiv[d] = (qd >= 1.0 && qd < 1.0e9) ? (int)qd : 1;
    double length_new = (double)ndiv[d] * cs;
    g0[d] = (lo[d] - (length_new - length) / 2.0) - (double)0.001f * length;
  }
  if ((double)ndiv[0] * (double)ndiv[1] > (double)kMaxC)
    return say(msg, msg_len, SPS_ERR_CAPACITY,
               "sps_neighbour_stats_static: the particles span %d x %d cells of width 2 hmax, "
               "more than the fixed device scratch holds (at most %d cells)",
               ndiv[0], ndiv[1], kMaxC);
  const int nx = ndiv[0], ny = ndiv[1], ncell = nx * ny;

  std::lock_guard<std::mutex> lock(g_mu);
  unsigned char* base = nullptr;
  cudaError_t e = scratch_on_current_device(&base);
  if (e != cudaSuccess)
    return say(msg, msg_len, SPS_ERR_CUDA,
               "sps_neighbour_stats_static: scratch address lookup failed: %s",
               cudaGetErrorString(e));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* dx_ = reinterpret_cast<double*>(base + kOffX);
  double* dh = reinterpret_cast<double*>(base + kOffH);
  int* dcell = reinterpret_cast<int*>(base + kOffCell);
  int* dsorted = reinterpret_cast<int*>(base + kOffSorted);
  int* ddeg = reinterpret_cast<int*>(base + kOffDeg);
  double* dws = reinterpret_cast<double*>(base + kOffWsum);
  int* dcnt = reinterpret_cast<int*>(base + kOffCnt);
  int* dfill = reinterpret_cast<int*>(base + kOffFill);
  int* dstart = reinterpret_cast<int*>(base + kOffStart);
  const int nb = (n + kBlock - 1) / kBlock;
  // the cell counters and fill cursors must start at zero on every call; every other
  // region is written in full before it is read
  if ((e = cudaMemsetAsync(dcnt, 0, sizeof(int) * ncell, st)) == cudaSuccess &&
      (e = cudaMemsetAsync(dfill, 0, sizeof(int) * ncell, st)) == cudaSuccess &&
      (e = cudaMemcpyAsync(dx_, x, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, st)) ==
          cudaSuccess &&
      (e = cudaMemcpyAsync(dh, hsml, sizeof(double) * n, cudaMemcpyHostToDevice, st)) ==
          cudaSuccess) {
    k_st_cells<<<nb, kBlock, 0, st>>>(n, dx_, g0[0], g0[1], cs, nx, ny, dcell, dcnt);
    k_st_scan<<<1, kScanThreads, 0, st>>>(ncell, dcnt, dstart);
    k_st_fill<<<nb, kBlock, 0, st>>>(n, dcell, dstart, dfill, dsorted);
    k_st_stats<<<nb, kBlock, 0, st>>>(n, dx_, dh, skf, pi, scale_k, nx, ny, dcell, dstart, dcnt,
                                      dsorted, ddeg, dws);
    if ((e = cudaGetLastError()) == cudaSuccess &&
        (e = cudaMemcpyAsync(degree, ddeg, sizeof(int) * n, cudaMemcpyDeviceToHost, st)) ==
            cudaSuccess &&
        (e = cudaMemcpyAsync(wsum, dws, sizeof(double) * n, cudaMemcpyDeviceToHost, st)) ==
            cudaSuccess)
      e = cudaStreamSynchronize(st);
  }
  if (e != cudaSuccess) {
    // wait for what this call enqueued before the failure, so that none of its work still
    // uses the scratch array when the lock is released (the first error is the one reported)
    cudaStreamSynchronize(st);
    return say(msg, msg_len, SPS_ERR_CUDA, "sps_neighbour_stats_static: %s",
               cudaGetErrorString(e));
  }
  int64_t total = 0;
  for (int a = 0; a < n; a++) total += degree[a];
  *npairs = total / 2;
  return SPS_OK;
}
