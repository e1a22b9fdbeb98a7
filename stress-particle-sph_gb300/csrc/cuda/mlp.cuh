// mlp.cuh -- the learned constitutive surrogate: a 14-128-128-128-4 MLP (SiLU, BF16 weights
// and activations, FP32 accumulation) standing in for the plastic source of the
// Drucker-Prager update (drucker_prager, 3_SPH_material_2018.f90:2047-2060) on loading
// stress-points.
//
// Inputs (scale-free):  stress direction s/|s| (4), strain-rate direction (e11, e22, e12, 0)/|e|
//   (4), spin w/|e| (1), material: tan(phi), c/|s|, nu, log10(E) - 7, rho/2000 - 1 (5).
// Output: the plastic source Gs (the -G of drucker_prager) divided by G_mod |e| (4).
// |e| = sqrt(e11^2 + e22^2 + 2 e12^2), G_mod = E / (2 (1 + nu)).
//
// Device inference runs one warp per 32 stress-points as two 16-row tiles of
// mma.sync.m16n8k16 (BF16 in, FP32 accumulate); a layer's FP32 accumulators are rounded to
// BF16 and reused in registers as the next layer's A fragments.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace sps {

constexpr int MLP_NIN = 14, MLP_IN = 16, MLP_H = 128, MLP_NOUT = 4, MLP_OUT = 8;
// FP32 master parameter layout (row-major W[k][n], k = input, n = output)
constexpr int MLP_W1 = 0;
constexpr int MLP_B1 = MLP_W1 + MLP_IN * MLP_H;
constexpr int MLP_W2 = MLP_B1 + MLP_H;
constexpr int MLP_B2 = MLP_W2 + MLP_H * MLP_H;
constexpr int MLP_W3 = MLP_B2 + MLP_H;
constexpr int MLP_B3 = MLP_W3 + MLP_H * MLP_H;
constexpr int MLP_W4 = MLP_B3 + MLP_H;
constexpr int MLP_B4 = MLP_W4 + MLP_H * MLP_OUT;
constexpr int MLP_NPARAM = MLP_B4 + MLP_OUT;
// fragment-packed BF16 weights: per layer (k-tiles x n-tiles) tiles of 16 x 8, each held
// as 32 lanes x uint2 (the B operand registers of mma.m16n8k16 for that lane), tile
// (kt, nt) at index kt * n-tiles + nt
constexpr int MLP_T1 = 1 * 16, MLP_T2 = 8 * 16, MLP_T3 = 8 * 16, MLP_T4 = 8 * 1;
constexpr int MLP_TILES = MLP_T1 + MLP_T2 + MLP_T3 + MLP_T4;
constexpr int MLP_FRAG_U2 = MLP_TILES * 32;
constexpr int MLP_BIAS = 3 * MLP_H + MLP_OUT;  // b1, b2, b3 (128 each), b4 (8), FP32
constexpr int MLP_TUPLE = MLP_NIN + MLP_NOUT;  // training tuple: 14 inputs, 4 targets

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }

// inputs of one stress-point; returns the output scale G_mod |e| (0 when undefined)
__device__ __forceinline__ double mlp_features(const double* s, const double* gu, double tanfi,
                                               double coh, double young, double poiss,
                                               double rho, float* x) {
  double S = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + s[3] * s[3]);
  double e11 = gu[0], e22 = gu[3], e12 = 0.5 * (gu[2] + gu[1]), w = 0.5 * (gu[2] - gu[1]);
  double en = sqrt(e11 * e11 + e22 * e22 + 2.0 * e12 * e12);
  if (!(S > 0.0) || !(en > 0.0)) return 0.0;
  for (int k = 0; k < 4; k++) x[k] = (float)(s[k] / S);
  x[4] = (float)(e11 / en);
  x[5] = (float)(e22 / en);
  x[6] = (float)(e12 / en);
  x[7] = 0.0f;
  x[8] = (float)(w / en);
  x[9] = (float)tanfi;
  x[10] = (float)(coh / S);
  x[11] = (float)poiss;
  x[12] = (float)(log10(young) - 7.0);
  x[13] = (float)(rho / 2000.0 - 1.0);
  x[14] = 0.0f;
  x[15] = 0.0f;
  return (young / (2.0 * (1.0 + poiss))) * en;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One hidden layer: acc = bias + A (16 x 16 KT) * W (16 KT x 128), then SiLU, repacked as
// the BF16 A fragments of the next layer (the accumulator layout of n-tiles 2j, 2j+1 is the
// A layout of k-tile j).  frag, bias: global memory (read-only, L1-cached).
template <int KT>
__device__ __forceinline__ void mlp_hidden(const uint2* __restrict__ frag,
                                           const float* __restrict__ bias,
                                           const uint32_t (*ain)[4], uint32_t (*aout)[4],
                                           int lane) {
  const int t = lane & 3;
#pragma unroll
  for (int np = 0; np < 8; np++) {  // pairs of n-tiles form one k-tile of the next layer
    float c[2][4];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      int nt = 2 * np + h;
      float b0 = __ldg(bias + nt * 8 + t * 2), b1 = __ldg(bias + nt * 8 + t * 2 + 1);
      c[h][0] = b0;
      c[h][1] = b1;
      c[h][2] = b0;
      c[h][3] = b1;
#pragma unroll
      for (int kt = 0; kt < KT; kt++) {
        const uint2 f = __ldg(frag + (kt * 16 + nt) * 32 + lane);
        mma_bf16(c[h], ain[kt], f.x, f.y);
      }
    }
    aout[np][0] = pack_bf16(silu(c[0][0]), silu(c[0][1]));
    aout[np][1] = pack_bf16(silu(c[0][2]), silu(c[0][3]));
    aout[np][2] = pack_bf16(silu(c[1][0]), silu(c[1][1]));
    aout[np][3] = pack_bf16(silu(c[1][2]), silu(c[1][3]));
  }
}

// Forward pass for 16 rows: xs = 16 x 16 inputs (shared memory, row stride 16, rounded to
// BF16 here), ys = 16 x 8 outputs (shared memory).  All 32 lanes of the warp must call it
// together.  frag / bias: the packed network (global memory).
__device__ __forceinline__ void mlp_tile16(const uint2* __restrict__ frag,
                                           const float* __restrict__ bias, const float* xs,
                                           float* ys, int lane) {
  const int g = lane >> 2, t = lane & 3;
  uint32_t a0[1][4];
  a0[0][0] = pack_bf16(xs[g * 16 + t * 2], xs[g * 16 + t * 2 + 1]);
  a0[0][1] = pack_bf16(xs[(g + 8) * 16 + t * 2], xs[(g + 8) * 16 + t * 2 + 1]);
  a0[0][2] = pack_bf16(xs[g * 16 + t * 2 + 8], xs[g * 16 + t * 2 + 9]);
  a0[0][3] = pack_bf16(xs[(g + 8) * 16 + t * 2 + 8], xs[(g + 8) * 16 + t * 2 + 9]);
  uint32_t a1[8][4], a2[8][4];
  const uint2* f1 = frag;
  const uint2* f2 = f1 + MLP_T1 * 32;
  const uint2* f3 = f2 + MLP_T2 * 32;
  const uint2* f4 = f3 + MLP_T3 * 32;
  mlp_hidden<1>(f1, bias, a0, a1, lane);
  mlp_hidden<8>(f2, bias + MLP_H, a1, a2, lane);
  mlp_hidden<8>(f3, bias + 2 * MLP_H, a2, a1, lane);
  float c[4];
  float b0 = __ldg(bias + 3 * MLP_H + t * 2), b1 = __ldg(bias + 3 * MLP_H + t * 2 + 1);
  c[0] = b0;
  c[1] = b1;
  c[2] = b0;
  c[3] = b1;
#pragma unroll
  for (int kt = 0; kt < 8; kt++) {
    const uint2 f = __ldg(f4 + kt * 32 + lane);
    mma_bf16(c, a1[kt], f.x, f.y);
  }
  ys[g * 8 + t * 2] = c[0];
  ys[g * 8 + t * 2 + 1] = c[1];
  ys[(g + 8) * 8 + t * 2] = c[2];
  ys[(g + 8) * 8 + t * 2 + 1] = c[3];
}

}  // namespace sps

// the trainer's parameters packed for the step (mlp_train.cu)
typedef struct sps_mlp sps_mlp;
namespace sps {
void mlp_pack(sps_mlp* m, uint2* frag, float* bias, cudaStream_t st);
cudaStream_t mlp_stream(sps_mlp* m);
const float* mlp_params(sps_mlp* m);

// the tensor-core (tcgen05) forward pass of mlp_tc.cu: the network as a shared-memory
// image (mlp_tc_image_bytes) and padded biases (mlp_tc_bias_count floats) packed from the
// trainer's FP32 parameters P, then y[r * out_stride + 0..3] = network(x[r * in_stride +
// 0 .. nin)) for r < *count (count on the device; n_max when count is null, and the bound
// of *count), on grid CTAs (mlp_tc_grid: at most two per SM); err (device) gets err_bit
// when a wait ran out.  mlp_tc_prepare raises the kernel's shared-memory limit (once per
// device, before any launch or capture).
size_t mlp_tc_image_bytes();
int mlp_tc_bias_count();
void mlp_tc_pack(const float* P, void* img, float* bias, cudaStream_t st);
cudaError_t mlp_tc_prepare();
int mlp_tc_grid(int n_max, int num_sms);
cudaError_t mlp_tc_forward(const void* img, const float* bias, const float* x, int in_stride,
                           int nin, const int* count, int n_max, float* y, int out_stride,
                           int* err, int err_bit, int grid, cudaStream_t st);
}  // namespace sps
