// mlp_train.cu -- training of the constitutive surrogate (include/sps_surrogate.h):
// forward, backward and Adam kernels, the BF16 fragment packing, and the tensor-core
// prediction path.
//
// Every layer is handled as one matrix product with the bias folded in: the activations
// carry a trailing column of ones and the parameters of a layer, W (K x N) followed by b
// (N), are read as one (K + 1) x N matrix.  So
//   forward   Z   = [A, 1] . [W; b]
//   backward  d[W; b] = [A, 1]^T . dZ,   dA = dZ . W^T
// with one tiled FP32 product kernel (k_gemm) for all three shapes.  The weight gradient
// splits its long reduction (over the minibatch rows) into partial products that a
// second kernel sums in a fixed order, so training is deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "common.cuh"
#include "mlp.cuh"
#include "sps_surrogate.h"

static_assert(sps::MLP_NPARAM == SPS_MLP_NPARAM, "parameter count");
static_assert(sps::MLP_TUPLE == SPS_MLP_TUPLE, "tuple size");

namespace {

using namespace sps;

constexpr int kSplit = 16;  // partial products of a weight gradient

#define MLP_CHECK(call)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      throw std::runtime_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
  } while (0)

__device__ __forceinline__ float bf16r(float v) {
  return __bfloat162float(__float2bfloat16_rn(v));
}

// layer geometry: parameter offset, input width K, output width N
struct Layer {
  int off, K, N;
};
constexpr Layer kLayers[4] = {{MLP_W1, MLP_IN, MLP_H},
                              {MLP_W2, MLP_H, MLP_H},
                              {MLP_W3, MLP_H, MLP_H},
                              {MLP_W4, MLP_H, MLP_OUT}};

// C(m, n) = sum over k in this block's split of A(m, k) B(k, n);  A(m, k) = A[m sam + k sak],
// B(k, n) = B[k sbk + n sbn], C(m, n) at C[(z M + m) ldc + n] for split z = blockIdx.z.
// 64 x 64 tiles, 256 threads with 4 x 4 outputs each.
__global__ void __launch_bounds__(256) k_gemm(const float* __restrict__ A, long sam, long sak,
                                              const float* __restrict__ B, long sbk, long sbn,
                                              float* __restrict__ C, int ldc, int M, int N,
                                              int K, int kchunk) {
  __shared__ float As[16][68];
  __shared__ float Bs[16][68];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
  float acc[4][4] = {};
  for (int kb = kbeg; kb < kend; kb += 16) {
    for (int e = tid; e < 1024; e += 256) {
      int mm, kk;
      if (sam == 1) {
        mm = e & 63;
        kk = e >> 6;
      } else {
        kk = e & 15;
        mm = e >> 4;
      }
      int m = m0 + mm, k = kb + kk;
      As[kk][mm] = (m < M && k < kend) ? A[m * sam + k * sak] : 0.0f;
      int nn, k2;
      if (sbn == 1) {
        nn = e & 63;
        k2 = e >> 6;
      } else {
        k2 = e & 15;
        nn = e >> 4;
      }
      int n = n0 + nn, kk2 = kb + k2;
      Bs[k2][nn] = (n < N && kk2 < kend) ? B[kk2 * sbk + n * sbn] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  float* Cz = C + (size_t)blockIdx.z * M * ldc;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int n = n0 + tx * 4 + j;
      if (n < N) Cz[(size_t)m * ldc + n] = acc[i][j];
    }
  }
}

// out[i] = sum over the splits of part[z n + i], in split order
__global__ void k_sum_splits(const float* __restrict__ part, int nsplit, int n,
                             float* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int z = 0; z < nsplit; z++) s += part[(size_t)z * n + i];
  out[i] = s;
}

__device__ __forceinline__ bool is_bias(int i) {
  return (i >= MLP_B1 && i < MLP_W2) || (i >= MLP_B2 && i < MLP_W3) ||
         (i >= MLP_B3 && i < MLP_W4) || i >= MLP_B4;
}

// the weights the forward pass uses: BF16-rounded weights (quantize), FP32 biases
__global__ void k_quantize(const float* __restrict__ P, float* __restrict__ Wq, int quantize) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= MLP_NPARAM) return;
  float v = P[i];
  Wq[i] = (quantize && !is_bias(i)) ? bf16r(v) : v;
}

// minibatch rows r < n: X = [inputs (14), 0, 0, 1] (17 columns), T = targets (4)
__global__ void k_gather(const float* __restrict__ data, const int* __restrict__ perm,
                         long start, int n, int quantize, float* __restrict__ X,
                         float* __restrict__ T) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const float* src = data + (size_t)perm[start + r] * MLP_TUPLE;
  float* x = X + (size_t)r * (MLP_IN + 1);
  for (int k = 0; k < MLP_NIN; k++) x[k] = quantize ? bf16r(src[k]) : src[k];
  x[14] = 0.0f;
  x[15] = 0.0f;
  x[16] = 1.0f;
  for (int k = 0; k < MLP_NOUT; k++) T[(size_t)r * MLP_NOUT + k] = src[MLP_NIN + k];
}

// H = [silu(Z), 1] (129 columns), BF16-rounded when quantize
__global__ void k_act(const float* __restrict__ Z, float* __restrict__ H, int n, int quantize) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= (long)n * (MLP_H + 1)) return;
  long r = i / (MLP_H + 1);
  int c = (int)(i % (MLP_H + 1));
  float v = 1.0f;
  if (c < MLP_H) {
    v = silu(Z[r * MLP_H + c]);
    if (quantize) v = bf16r(v);
  }
  H[i] = v;
}

// dZ = dH * silu'(Z)
__global__ void k_act_bwd(const float* __restrict__ dH, const float* __restrict__ Z,
                          float* __restrict__ dZ, int n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= (long)n * MLP_H) return;
  float z = Z[i];
  float sg = 1.0f / (1.0f + expf(-z));
  dZ[i] = dH[i] * (sg * (1.0f + z * (1.0f - sg)));
}

// dY = 2 (Y - T) / (4 n) on the 4 used outputs (0 on the padding); per-block sum of the
// squared errors into lossp[blockIdx.x]
__global__ void k_loss(const float* __restrict__ Y, const float* __restrict__ T,
                       float* __restrict__ dY, int n, float* __restrict__ lossp) {
  __shared__ float sh[256];
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (r < n) {
    const float sc = 2.0f / (4.0f * (float)n);
    for (int c = 0; c < MLP_OUT; c++) {
      float d = 0.0f;
      if (c < MLP_NOUT) {
        d = Y[(size_t)r * MLP_OUT + c] - T[(size_t)r * MLP_NOUT + c];
        l += d * d;
      }
      dY[(size_t)r * MLP_OUT + c] = sc * d;
    }
  }
  sh[threadIdx.x] = l;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) lossp[blockIdx.x] = sh[0];
}

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ Mo,
                       float* __restrict__ Vo, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= MLP_NPARAM) return;
  float g = G[i];
  float m = b1 * Mo[i] + (1.0f - b1) * g;
  float v = b2 * Vo[i] + (1.0f - b2) * (g * g);
  Mo[i] = m;
  Vo[i] = v;
  P[i] = P[i] - lr * (m / bc1) / (sqrtf(v / bc2) + eps);
}

// B-operand registers of mma.m16n8k16 (row.col, BF16) for every tile and lane:
// lane = 4 g + t holds {W[k0 + 2t][n0 + g], W[k0 + 2t + 1][n0 + g]} and the same at
// k0 + 8 + 2t; biases copied as FP32
__global__ void k_pack(const float* __restrict__ P, uint2* __restrict__ frag,
                       float* __restrict__ bias) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < MLP_BIAS) {
    int src = i < MLP_H ? MLP_B1 + i
              : i < 2 * MLP_H ? MLP_B2 + (i - MLP_H)
              : i < 3 * MLP_H ? MLP_B3 + (i - 2 * MLP_H)
                              : MLP_B4 + (i - 3 * MLP_H);
    bias[i] = P[src];
  }
  if (i >= MLP_FRAG_U2) return;
  int tile = i >> 5, lane = i & 31, g = lane >> 2, t = lane & 3;
  int off, N, local, NT;
  if (tile < MLP_T1) {
    off = MLP_W1, N = MLP_H, NT = 16, local = tile;
  } else if (tile < MLP_T1 + MLP_T2) {
    off = MLP_W2, N = MLP_H, NT = 16, local = tile - MLP_T1;
  } else if (tile < MLP_T1 + MLP_T2 + MLP_T3) {
    off = MLP_W3, N = MLP_H, NT = 16, local = tile - MLP_T1 - MLP_T2;
  } else {
    off = MLP_W4, N = MLP_OUT, NT = 1, local = tile - MLP_T1 - MLP_T2 - MLP_T3;
  }
  int kt = local / NT, nt = local % NT;
  int n = nt * 8 + g, k = kt * 16 + 2 * t;
  const float* W = P + off;
  frag[i] = make_uint2(pack_bf16(W[k * N + n], W[(k + 1) * N + n]),
                       pack_bf16(W[(k + 8) * N + n], W[(k + 9) * N + n]));
}

// y (n x 4) = network(x (n x 14)) by the tensor-core code of the step; 4 warps per
// block, 32 rows per warp, every lane of a warp takes part in both 16-row tiles
__global__ void __launch_bounds__(128) k_predict(const uint2* __restrict__ frag,
                                                 const float* __restrict__ bias,
                                                 const float* __restrict__ x, int n,
                                                 float* __restrict__ y) {
  __shared__ float xs[4][32][16];
  __shared__ float ys[4][32][8];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long row = (blockIdx.x * 4L + w) * 32 + lane;
  for (int k = 0; k < 16; k++)
    xs[w][lane][k] = (row < n && k < MLP_NIN) ? x[row * MLP_NIN + k] : 0.0f;
  __syncwarp();
  mlp_tile16(frag, bias, &xs[w][0][0], &ys[w][0][0], lane);
  mlp_tile16(frag, bias, &xs[w][16][0], &ys[w][16][0], lane);
  __syncwarp();
  if (row < n)
    for (int k = 0; k < MLP_NOUT; k++) y[row * MLP_NOUT + k] = ys[w][lane][k];
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double uniform01(uint64_t& s) { return (splitmix(s) >> 11) * 0x1.0p-53; }

}  // namespace

struct sps_mlp {
  sps_mlp_config cfg{};
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  float *P = nullptr, *Wq = nullptr, *G = nullptr, *Mo = nullptr, *Vo = nullptr;
  float *part = nullptr, *X = nullptr, *T = nullptr, *Y = nullptr, *dY = nullptr;
  float *Z[3] = {}, *H[3] = {}, *dH = nullptr, *dZ = nullptr;
  float* lossp = nullptr;
  int lossp_cap = 0;
  float* data = nullptr;
  int64_t ndata = 0, data_cap = 0;
  int* perm = nullptr;
  int64_t perm_cap = 0;
  int* ident = nullptr;
  float* gtuples = nullptr;
  uint2* frag = nullptr;
  float* bias = nullptr;
  void* tc_img = nullptr;   // the network as the tensor-core kernel's shared-memory image
  float* tc_bias = nullptr;
  int* tc_err = nullptr;
  float *px = nullptr, *py = nullptr;
  int64_t pred_cap = 0;
  bool tensor_memory_path = true;  // sps_mlp_predict: tcgen05 (else the warp-level mma.sync)
  int64_t adam_t = 0;
  uint64_t rng = 0;
  std::string err;

  template <typename T>
  T* alloc(size_t n) {
    void* p = nullptr;
    MLP_CHECK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    allocs.push_back(p);
    return static_cast<T*>(p);
  }
  void release(void* p) {
    if (!p) return;
    for (auto& a : allocs)
      if (a == p) {
        cudaFree(a);
        a = nullptr;
      }
  }
  ~sps_mlp() {
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : allocs)
      if (p) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }

  void gemm(const float* A, long sam, long sak, const float* B, long sbk, long sbn, float* C,
            int ldc, int M, int N, int K, int nsplit) {
    int kchunk = ((K + nsplit - 1) / nsplit + 15) / 16 * 16;
    nsplit = (K + kchunk - 1) / kchunk;
    dim3 grid((N + 63) / 64, (M + 63) / 64, nsplit);
    k_gemm<<<grid, 256, 0, stream>>>(A, sam, sak, B, sbk, sbn, C, ldc, M, N, K, kchunk);
  }
  void weight_grad(const float* Aext, int K, const float* dZ_, int N, int n, int off) {
    // d[W; b] ((K + 1) x N) = Aext^T (n x (K + 1)) . dZ (n x N), split over rows
    int kchunk = ((n + kSplit - 1) / kSplit + 15) / 16 * 16;
    int nsplit = (n + kchunk - 1) / kchunk;
    dim3 grid((N + 63) / 64, (K + 1 + 63) / 64, nsplit);
    k_gemm<<<grid, 256, 0, stream>>>(Aext, 1, K + 1, dZ_, N, 1, part, N, K + 1, N, n, kchunk);
    int tot = (K + 1) * N;
    k_sum_splits<<<(tot + 255) / 256, 256, 0, stream>>>(part, nsplit, tot, G + off);
  }

  // forward + loss + backward for n gathered rows (X, T); gradient into G, per-block
  // squared errors into lossp[lo ...]
  void fwd_bwd(int n, int lo) {
    const int q = cfg.quantize;
    const float* A = X;
    int K = MLP_IN;
    for (int l = 0; l < 3; l++) {
      gemm(A, K + 1, 1, Wq + kLayers[l].off, MLP_H, 1, Z[l], MLP_H, n, MLP_H, K + 1, 1);
      long tot = (long)n * (MLP_H + 1);
      k_act<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(Z[l], H[l], n, q);
      A = H[l];
      K = MLP_H;
    }
    gemm(A, MLP_H + 1, 1, Wq + MLP_W4, MLP_OUT, 1, Y, MLP_OUT, n, MLP_OUT, MLP_H + 1, 1);
    k_loss<<<(n + 255) / 256, 256, 0, stream>>>(Y, T, dY, n, lossp + lo);
    // output layer
    weight_grad(H[2], MLP_H, dY, MLP_OUT, n, MLP_W4);
    // dH3 = dY . W4^T (first 128 columns)
    gemm(dY, MLP_OUT, 1, Wq + MLP_W4, 1, MLP_OUT, dH, MLP_H, n, MLP_H, MLP_OUT, 1);
    for (int l = 2; l >= 0; l--) {
      long tot = (long)n * MLP_H;
      k_act_bwd<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(dH, Z[l], dZ, n);
      const float* Ain = l > 0 ? H[l - 1] : X;
      int Kin = l > 0 ? MLP_H : MLP_IN;
      weight_grad(Ain, Kin, dZ, MLP_H, n, kLayers[l].off);
      if (l > 0)  // dA = dZ . W^T
        gemm(dZ, MLP_H, 1, Wq + kLayers[l].off, 1, MLP_H, dH, MLP_H, n, MLP_H, MLP_H, 1);
    }
  }
  void quantize() {
    k_quantize<<<(MLP_NPARAM + 255) / 256, 256, 0, stream>>>(P, Wq, cfg.quantize);
  }
  void ensure_lossp(int n) {
    if (n <= lossp_cap) return;
    release(lossp);
    lossp = alloc<float>(n);
    lossp_cap = n;
  }
};

namespace {

int mfail(sps_mlp* m, int rc, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (m) m->err = buf;
  return rc;
}

}  // namespace

namespace sps {
// used by the step's surrogate installation (sps_api.cu)
void mlp_pack(sps_mlp* m, uint2* frag, float* bias, cudaStream_t st) {
  k_pack<<<(MLP_FRAG_U2 + 255) / 256, 256, 0, st>>>(m->P, frag, bias);
}
cudaStream_t mlp_stream(sps_mlp* m) { return m->stream; }
const float* mlp_params(sps_mlp* m) { return m->P; }
}  // namespace sps

extern "C" {

int sps_mlp_create(const sps_mlp_config* cfg, sps_mlp** out) {
  if (!cfg || !out) return SPS_ERR_ARG;
  *out = nullptr;
  if (cfg->batch < 64 || cfg->batch > 65536 || cfg->batch % 64) return SPS_ERR_ARG;
  sps_mlp* m = new (std::nothrow) sps_mlp;
  if (!m) return SPS_ERR_CUDA;
  try {
    m->cfg = *cfg;
    m->rng = cfg->seed;
    MLP_CHECK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    const int B = cfg->batch;
    m->P = m->alloc<float>(MLP_NPARAM);
    m->Wq = m->alloc<float>(MLP_NPARAM);
    m->G = m->alloc<float>(MLP_NPARAM);
    m->Mo = m->alloc<float>(MLP_NPARAM);
    m->Vo = m->alloc<float>(MLP_NPARAM);
    m->part = m->alloc<float>((size_t)kSplit * (MLP_H + 1) * MLP_H);
    m->X = m->alloc<float>((size_t)B * (MLP_IN + 1));
    m->T = m->alloc<float>((size_t)B * MLP_NOUT);
    m->Y = m->alloc<float>((size_t)B * MLP_OUT);
    m->dY = m->alloc<float>((size_t)B * MLP_OUT);
    for (int l = 0; l < 3; l++) {
      m->Z[l] = m->alloc<float>((size_t)B * MLP_H);
      m->H[l] = m->alloc<float>((size_t)B * (MLP_H + 1));
    }
    m->dH = m->alloc<float>((size_t)B * MLP_H);
    m->dZ = m->alloc<float>((size_t)B * MLP_H);
    m->ident = m->alloc<int>(B);
    m->gtuples = m->alloc<float>((size_t)B * MLP_TUPLE);
    m->frag = m->alloc<uint2>(MLP_FRAG_U2);
    m->tc_img = m->alloc<uint8_t>(sps::mlp_tc_image_bytes());
    m->tc_bias = m->alloc<float>(sps::mlp_tc_bias_count());
    m->tc_err = m->alloc<int>(1);
    m->bias = m->alloc<float>(MLP_BIAS);
    m->ensure_lossp((B + 255) / 256);
    // Glorot-uniform weights, zero biases and padding
    std::vector<float> p(MLP_NPARAM, 0.0f);
    uint64_t s = cfg->seed ^ 0x5eed5eed5eedull;
    for (const Layer& L : kLayers) {
      int kin = (L.off == MLP_W1) ? MLP_NIN : L.K;
      int nout = (L.off == MLP_W4) ? MLP_NOUT : L.N;
      double a = std::sqrt(6.0 / (kin + nout));
      for (int k = 0; k < kin; k++)
        for (int n = 0; n < nout; n++) p[L.off + k * L.N + n] = (float)((2.0 * uniform01(s) - 1.0) * a);
    }
    std::vector<int> id(B);
    for (int i = 0; i < B; i++) id[i] = i;
    MLP_CHECK(cudaMemcpyAsync(m->P, p.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, m->stream));
    MLP_CHECK(cudaMemcpyAsync(m->ident, id.data(), sizeof(int) * B, cudaMemcpyHostToDevice, m->stream));
    MLP_CHECK(cudaMemsetAsync(m->Mo, 0, sizeof(float) * MLP_NPARAM, m->stream));
    MLP_CHECK(cudaMemsetAsync(m->Vo, 0, sizeof(float) * MLP_NPARAM, m->stream));
    MLP_CHECK(cudaStreamSynchronize(m->stream));
  } catch (const std::exception& e) {
    delete m;
    return SPS_ERR_CUDA;
  }
  *out = m;
  return SPS_OK;
}

int sps_mlp_get_params(sps_mlp* m, float* params) {
  if (!m || !params) return SPS_ERR_ARG;
  try {
    MLP_CHECK(cudaMemcpyAsync(params, m->P, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, m->stream));
    MLP_CHECK(cudaStreamSynchronize(m->stream));
  } catch (const std::exception& e) {
    return mfail(m, SPS_ERR_CUDA, "%s", e.what());
  }
  return SPS_OK;
}

int sps_mlp_set_params(sps_mlp* m, const float* params) {
  if (!m || !params) return SPS_ERR_ARG;
  try {
    MLP_CHECK(cudaMemcpyAsync(m->P, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, m->stream));
    MLP_CHECK(cudaMemsetAsync(m->Mo, 0, sizeof(float) * MLP_NPARAM, m->stream));
    MLP_CHECK(cudaMemsetAsync(m->Vo, 0, sizeof(float) * MLP_NPARAM, m->stream));
    MLP_CHECK(cudaStreamSynchronize(m->stream));
    m->adam_t = 0;
  } catch (const std::exception& e) {
    return mfail(m, SPS_ERR_CUDA, "%s", e.what());
  }
  return SPS_OK;
}

int sps_mlp_set_data(sps_mlp* m, const float* tuples, int64_t n) {
  if (!m || n < 0 || (n > 0 && !tuples)) return SPS_ERR_ARG;
  if (n > (int64_t)1 << 30) return mfail(m, SPS_ERR_CAPACITY, "at most 2^30 tuples");
  try {
    if (n > m->data_cap) {
      m->release(m->data);
      m->release(m->perm);
      m->data = m->alloc<float>((size_t)n * MLP_TUPLE);
      m->perm = m->alloc<int>(n);
      m->data_cap = m->perm_cap = n;
    }
    if (n)
      MLP_CHECK(cudaMemcpyAsync(m->data, tuples, sizeof(float) * MLP_TUPLE * n,
                                cudaMemcpyHostToDevice, m->stream));
    MLP_CHECK(cudaStreamSynchronize(m->stream));
    m->ndata = n;
  } catch (const std::exception& e) {
    return mfail(m, SPS_ERR_CUDA, "%s", e.what());
  }
  return SPS_OK;
}

int sps_mlp_train(sps_mlp* m, int32_t epochs, float lr, float* loss) {
  if (!m || epochs < 0) return SPS_ERR_ARG;
  const int B = m->cfg.batch;
  const int64_t nmb = m->ndata / B;
  if (epochs > 0 && nmb == 0) return mfail(m, SPS_ERR_STATE, "fewer tuples than one minibatch");
  const int per = (B + 255) / 256;
  if (!(lr > 0.0f)) lr = m->cfg.lr;
  try {
    m->ensure_lossp((int)(nmb * per));
    std::vector<int> perm(m->ndata);
    std::vector<float> lp;
    for (int ep = 0; ep < epochs; ep++) {
      for (int64_t i = 0; i < m->ndata; i++) perm[i] = (int)i;
      for (int64_t i = m->ndata - 1; i > 0; i--) {  // Fisher-Yates
        int64_t j = (int64_t)(splitmix(m->rng) % (uint64_t)(i + 1));
        std::swap(perm[i], perm[j]);
      }
      MLP_CHECK(cudaMemcpyAsync(m->perm, perm.data(), sizeof(int) * m->ndata,
                                cudaMemcpyHostToDevice, m->stream));
      for (int64_t b = 0; b < nmb; b++) {
        m->quantize();
        k_gather<<<(B + 255) / 256, 256, 0, m->stream>>>(m->data, m->perm, b * B, B,
                                                         m->cfg.quantize, m->X, m->T);
        m->fwd_bwd(B, (int)(b * per));
        m->adam_t++;
        float bc1 = (float)(1.0 - std::pow((double)m->cfg.beta1, (double)m->adam_t));
        float bc2 = (float)(1.0 - std::pow((double)m->cfg.beta2, (double)m->adam_t));
        k_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, m->stream>>>(
            m->P, m->G, m->Mo, m->Vo, lr, m->cfg.beta1, m->cfg.beta2, m->cfg.eps, bc1,
            bc2);
      }
      MLP_CHECK(cudaGetLastError());
      lp.resize(nmb * per);
      MLP_CHECK(cudaMemcpyAsync(lp.data(), m->lossp, sizeof(float) * lp.size(),
                                cudaMemcpyDeviceToHost, m->stream));
      MLP_CHECK(cudaStreamSynchronize(m->stream));
      double s = 0.0;
      for (float v : lp) s += v;
      if (loss) loss[ep] = (float)(s / ((double)nmb * B * MLP_NOUT));
    }
  } catch (const std::exception& e) {
    return mfail(m, SPS_ERR_CUDA, "%s", e.what());
  }
  return SPS_OK;
}

int sps_mlp_grad(sps_mlp* m, const float* tuples, int32_t n, float* grad, float* loss) {
  if (!m || !tuples || !grad || n <= 0 || n > m->cfg.batch) return SPS_ERR_ARG;
  try {
    MLP_CHECK(cudaMemcpyAsync(m->gtuples, tuples, sizeof(float) * MLP_TUPLE * n,
                              cudaMemcpyHostToDevice, m->stream));
    m->quantize();
    k_gather<<<(n + 255) / 256, 256, 0, m->stream>>>(m->gtuples, m->ident, 0, n,
                                                     m->cfg.quantize, m->X, m->T);
    m->fwd_bwd(n, 0);
    MLP_CHECK(cudaGetLastError());
    std::vector<float> lp((n + 255) / 256);
    MLP_CHECK(cudaMemcpyAsync(grad, m->G, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, m->stream));
    MLP_CHECK(cudaMemcpyAsync(lp.data(), m->lossp, sizeof(float) * lp.size(), cudaMemcpyDeviceToHost, m->stream));
    MLP_CHECK(cudaStreamSynchronize(m->stream));
    double s = 0.0;
    for (float v : lp) s += v;
    if (loss) *loss = (float)(s / (4.0 * n));
  } catch (const std::exception& e) {
    return mfail(m, SPS_ERR_CUDA, "%s", e.what());
  }
  return SPS_OK;
}

int sps_mlp_predict(sps_mlp* m, const float* x, int32_t n, float* y) {
  if (!m || n < 0 || (n > 0 && (!x || !y))) return SPS_ERR_ARG;
  if (n == 0) return SPS_OK;
  try {
    if (n > m->pred_cap) {
      m->release(m->px);
      m->release(m->py);
      m->px = m->alloc<float>((size_t)n * MLP_NIN);
      m->py = m->alloc<float>((size_t)n * MLP_NOUT);
      m->pred_cap = n;
    }
    MLP_CHECK(cudaMemcpyAsync(m->px, x, sizeof(float) * MLP_NIN * n, cudaMemcpyHostToDevice, m->stream));
    int herr = 0;
    if (m->tensor_memory_path) {
      // the step's inference: 128-row tiles on tcgen05 with tensor-memory accumulators
      int dev = 0, nsm = 0;
      MLP_CHECK(cudaGetDevice(&dev));
      MLP_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      MLP_CHECK(sps::mlp_tc_prepare());
      sps::mlp_tc_pack(m->P, m->tc_img, m->tc_bias, m->stream);
      MLP_CHECK(cudaMemsetAsync(m->tc_err, 0, sizeof(int), m->stream));
      MLP_CHECK(sps::mlp_tc_forward(m->tc_img, m->tc_bias, m->px, MLP_NIN, MLP_NIN, nullptr, n,
                                    m->py, MLP_NOUT, m->tc_err, 1, sps::mlp_tc_grid(n, nsm),
                                    m->stream));
      MLP_CHECK(cudaMemcpyAsync(&herr, m->tc_err, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    } else {
      // the warp-level mma.sync inference
      sps::mlp_pack(m, m->frag, m->bias, m->stream);
      k_predict<<<(n + 127) / 128, 128, 0, m->stream>>>(m->frag, m->bias, m->px, n, m->py);
    }
    MLP_CHECK(cudaGetLastError());
    MLP_CHECK(cudaMemcpyAsync(y, m->py, sizeof(float) * MLP_NOUT * n, cudaMemcpyDeviceToHost, m->stream));
    MLP_CHECK(cudaStreamSynchronize(m->stream));
    if (herr) return mfail(m, SPS_ERR_CUDA, "tensor-core inference: a wait ran out");
  } catch (const std::exception& e) {
    return mfail(m, SPS_ERR_CUDA, "%s", e.what());
  }
  return SPS_OK;
}

int sps_mlp_set_inference(sps_mlp* m, int32_t tensor_memory) {
  if (!m || (tensor_memory != 0 && tensor_memory != 1)) return SPS_ERR_ARG;
  m->tensor_memory_path = tensor_memory == 1;
  return SPS_OK;
}

int sps_mlp_last_error(sps_mlp* m, char* buf, int32_t len) {
  if (!m || !buf || len <= 0) return 0;
  std::snprintf(buf, (size_t)len, "%s", m->err.c_str());
  return (int)m->err.size();
}

void sps_mlp_destroy(sps_mlp* m) { delete m; }

}  // extern "C"
