// mlp_tc.cu -- the surrogate network's forward pass on the 5th-generation tensor cores
// (tcgen05): 128-row tiles, operands in shared memory, accumulators in tensor memory.
//
// Network: 14(16) -> 128 -> 128 -> 128 -> 4(16), SiLU on the hidden layers, BF16 weights and
// activations, FP32 accumulation and biases (the same numbers as the trainer's quantized
// forward pass and the warp-level inference of mlp.cuh).
//
// One CTA of 256 threads (8 warps) holds the whole network in shared memory (73,728 B of
// BF16 weights, 1,600 B of biases) and loops over 128-row tiles of its inputs.  Per tile:
//   - the 128 x 16 input tile is rounded to BF16 into shared memory;
//   - layer by layer, one elected thread issues tcgen05.mma (kind::f16, M = 128, K = 16 per
//     instruction, N = 128 for the hidden layers, 16 for the output layer) with the
//     activation tile as A and the layer's weights as B, accumulating in 128 columns of
//     tensor memory, and commits the group to an mbarrier;
//   - every thread waits for the mbarrier, reads half of its row of the accumulator with
//     tcgen05.ld (warp w reads tensor-memory lanes 32 (w % 4) .. + 31, the sub-partition
//     it may access, and columns 64 (w / 4) .. + 63), adds the bias, applies SiLU and writes
//     the BF16 activation back into shared memory as the next layer's A.
// Shared-memory operands use the no-swizzle K-major layout of 8 x 16-byte core matrices:
// element (r, k) of an R x K operand sits at byte ((r / 8) (K / 8) + k / 8) 128 + (r % 8) 16
// + (k % 8) 2, so the leading (K) byte offset between core matrices is 128 and the stride
// (8-row group) byte offset is 16 K.
//
// Every wait is bounded: a wait that runs out sets an error flag, waits once more (also
// bounded) for the tensor core to finish, releases the tensor memory and returns.
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.cuh"

namespace sps {

namespace {

constexpr int kTcRows = 128;                       // rows per tile (the MMA's M)
constexpr uint32_t kImgW1 = 0;                     // 128 (n) x 16 (k)
constexpr uint32_t kImgW2 = kImgW1 + 128 * 16 * 2; // 128 x 128
constexpr uint32_t kImgW3 = kImgW2 + 128 * 128 * 2;
constexpr uint32_t kImgW4 = kImgW3 + 128 * 128 * 2;  // 16 x 128 (rows 4 .. 15 zero)
constexpr uint32_t kImgBytes = kImgW4 + 16 * 128 * 2;
constexpr int kTcBias = 3 * MLP_H + 16;            // b1, b2, b3, b4 padded to 16

// dynamic shared memory of one CTA
struct TcSmem {
  alignas(128) uint8_t w[kImgBytes];     // B operands W1 .. W4 (transposed, core layout)
  alignas(128) uint8_t a0[kTcRows * 16 * 2];  // input tile (K = 16)
  alignas(128) uint8_t ah[kTcRows * 128 * 2]; // hidden activation tile (K = 128)
  float bias[kTcBias];
  alignas(8) unsigned long long mbar;
  uint32_t tmem;
  int abort;
};

__host__ __device__ constexpr uint32_t core_off(int r, int k, int K) {
  return (uint32_t)(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading (K) and stride (8-row) byte
// offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy writes to shared memory made visible to the tensor core (async proxy)
__device__ __forceinline__ void proxy_fence() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's tensor-memory lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// bounded wait for the mbarrier phase with the given parity; false when it ran out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > (1ll << 32)) return false;  // about two seconds
  }
}

// writes 16 consecutive BF16 values (columns k0 .. k0 + 15) of row r into a K = 128 tile
__device__ __forceinline__ void put16(uint8_t* tile, int r, int k0, const float* v) {
  uint4 lo = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                        pack_bf16(v[6], v[7]));
  uint4 hi = make_uint4(pack_bf16(v[8], v[9]), pack_bf16(v[10], v[11]),
                        pack_bf16(v[12], v[13]), pack_bf16(v[14], v[15]));
  *reinterpret_cast<uint4*>(tile + core_off(r, k0, 128)) = lo;
  *reinterpret_cast<uint4*>(tile + core_off(r, k0 + 8, 128)) = hi;
}

// SiLU as z sigmoid(z) = h + h tanh(h), h = z / 2, with one hardware tanh (tanh.approx.f32,
// relative error about 2^-11): one multi-function-unit operation per element instead of an
// exponential and a reciprocal; the activation is rounded to BF16 (2^-9) right after
__device__ __forceinline__ float silu_fast(float z) {
  const float h = 0.5f * z;
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
  return fmaf(h, t, h);
}

constexpr int kTcThreads = 256;  // 8 warps: warp w reads lanes 32 (w % 4) .., columns 64 (w / 4) ..

// y[row, 0..3] = network(x[row, 0..nin)) for rows [0, n), n = *count when count is given
__global__ void __launch_bounds__(kTcThreads, 2) k_mlp_tc(const uint4* __restrict__ img,
                                                   const float* __restrict__ bias,
                                                   const float* __restrict__ x, int in_stride,
                                                   int nin, const int* __restrict__ count,
                                                   int n_fixed, float* __restrict__ y,
                                                   int out_stride, int* __restrict__ err,
                                                   int err_bit) {
  extern __shared__ __align__(128) uint8_t tc_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(tc_raw);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int n = count ? *count : n_fixed;
  const int ntiles = (n + kTcRows - 1) / kTcRows;
  if ((int)blockIdx.x >= ntiles) return;  // the whole block: nothing allocated yet

  // network into shared memory; tensor memory (128 columns) and the mbarrier
  for (uint32_t i = tid; i < kImgBytes / 16; i += blockDim.x)
    reinterpret_cast<uint4*>(S.w)[i] = img[i];
  for (int i = tid; i < kTcBias; i += blockDim.x) S.bias[i] = bias[i];
  const uint32_t mbar = smem_u32(&S.mbar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    S.abort = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&S.tmem)),
                 "r"(128)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  proxy_fence();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem;
  // this warp's tensor-memory lanes (its sub-partition) and its half of the columns
  const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
  const int r = 32 * (warp & 3) + (tid & 31), chalf = 64 * (warp >> 2);
  const uint32_t a0 = smem_u32(S.a0), ah = smem_u32(S.ah), w = smem_u32(S.w);
  const uint32_t id_h = instr_desc(128, 128), id_o = instr_desc(128, 16);
  uint32_t phase = 0;

  // issue one layer's MMAs (thread 0), wait for them (every thread); false, for every thread
  // alike, when a wait ran out
  auto layer = [&](int which) -> bool {
    if (tid == 0) {
      tc_fence_after();
      if (which == 1) {
        tc_mma(tmem, smem_desc(a0, 128, 256), smem_desc(w + kImgW1, 128, 256), id_h, 0);
      } else {
        const uint32_t wb = which == 2 ? kImgW2 : which == 3 ? kImgW3 : kImgW4;
        const uint32_t id = which == 4 ? id_o : id_h;
#pragma unroll
        for (int kk = 0; kk < 8; kk++)
          tc_mma(tmem, smem_desc(ah + kk * 256, 128, 2048), smem_desc(w + wb + kk * 256, 128, 2048),
                 id, kk > 0);
      }
      tc_commit(mbar);
    }
    const bool ok = mbar_wait(mbar, phase & 1);
    phase++;
    if (!ok) S.abort = 1;
    __syncthreads();  // every thread takes the same branch afterwards
    tc_fence_after();
    return S.abort == 0;
  };
  // the accumulator of a hidden layer: bias, SiLU, BF16 into the activation tile
  auto hidden_epilogue = [&](const float* b) {
#pragma unroll 1
    for (int c0 = chalf; c0 < chalf + 64; c0 += 16) {
      float v[16];
      tc_ld16(trow + c0, v);
#pragma unroll
      for (int i = 0; i < 16; i++) v[i] = silu_fast(v[i] + b[c0 + i]);
      put16(S.ah, r, c0, v);
    }
  };
  // ordering between this thread's tensor-memory reads / shared-memory writes and the next
  // MMAs, which other threads' data feed
  auto sync_for_mma = [&]() {
    tc_fence_before();
    proxy_fence();
    __syncthreads();
  };

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    // input rows, rounded to BF16 into the K = 16 tile: thread r, column half chalf / 64
    const long row = (long)tile * kTcRows + r;
    {
      const int k0 = chalf / 8;  // columns 0-7 (warps 0-3) or 8-15 (warps 4-7)
      float v[8];
#pragma unroll
      for (int k = 0; k < 8; k++)
        v[k] = (row < n && k0 + k < nin) ? x[row * in_stride + k0 + k] : 0.0f;
      *reinterpret_cast<uint4*>(S.a0 + core_off(r, k0, 16)) =
          make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                     pack_bf16(v[6], v[7]));
    }
    sync_for_mma();
    if (!layer(1)) break;
    hidden_epilogue(S.bias);
    sync_for_mma();
    if (!layer(2)) break;
    hidden_epilogue(S.bias + MLP_H);
    sync_for_mma();
    if (!layer(3)) break;
    hidden_epilogue(S.bias + 2 * MLP_H);
    sync_for_mma();
    if (!layer(4)) break;
    if (warp < 4) {  // the output columns 0-15, by the first four warps
      float o[16];
      tc_ld16(trow, o);
      if (row < n)
        for (int k = 0; k < MLP_NOUT; k++) y[row * out_stride + k] = o[k] + S.bias[3 * MLP_H + k];
    }
    tc_fence_before();
    __syncthreads();
    if (S.abort) break;
  }
  __syncthreads();
  if (S.abort) {
    if (tid == 0) atomicOr(err, err_bit);
    // the tensor core may still be running the timed-out group: wait once more (bounded)
    // before the tensor memory is released
    mbar_wait(mbar, (phase - 1) & 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128)
                 : "memory");
}

// W^T of every layer in BF16 in the shared-memory image (core layout, K-major), and the
// biases with b4 padded to 16; P: the trainer's FP32 parameters (row-major W[k][n])
__global__ void k_pack_tc(const float* __restrict__ P, uint8_t* __restrict__ img,
                          float* __restrict__ bias) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kTcBias) {
    float b = 0.0f;
    if (i < MLP_H) b = P[MLP_B1 + i];
    else if (i < 2 * MLP_H) b = P[MLP_B2 + i - MLP_H];
    else if (i < 3 * MLP_H) b = P[MLP_B3 + i - 2 * MLP_H];
    else if (i - 3 * MLP_H < MLP_OUT) b = P[MLP_B4 + i - 3 * MLP_H];
    bias[i] = b;
  }
  // element e of the image: layer, output n, input k
  int e = i, base, off, K, N;
  if (e < 128 * 16) {
    base = kImgW1, off = MLP_W1, K = 16, N = MLP_H;
  } else if ((e -= 128 * 16) < 128 * 128) {
    base = kImgW2, off = MLP_W2, K = 128, N = MLP_H;
  } else if ((e -= 128 * 128) < 128 * 128) {
    base = kImgW3, off = MLP_W3, K = 128, N = MLP_H;
  } else if ((e -= 128 * 128) < 16 * 128) {
    base = kImgW4, off = MLP_W4, K = 128, N = MLP_OUT;
  } else {
    return;
  }
  const int nn = e / K, k = e % K;
  const float v = nn < N ? P[off + k * N + nn] : 0.0f;
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  *reinterpret_cast<__nv_bfloat16*>(img + base + core_off(nn, k, K)) = h;
}

}  // namespace

size_t mlp_tc_image_bytes() { return kImgBytes; }
int mlp_tc_bias_count() { return kTcBias; }

void mlp_tc_pack(const float* P, void* img, float* bias, cudaStream_t st) {
  const int n = 128 * 16 + 2 * 128 * 128 + 16 * 128;
  k_pack_tc<<<(n + 255) / 256, 256, 0, st>>>(P, static_cast<uint8_t*>(img), bias);
}

cudaError_t mlp_tc_prepare() {
  return cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(TcSmem));
}

// two CTAs per SM (2 x 112 KB of shared memory, 2 x 128 tensor-memory columns): one CTA's
// epilogue runs while the other's MMAs do
int mlp_tc_grid(int n_max, int num_sms) {
  const int ntiles = (n_max + kTcRows - 1) / kTcRows;
  return ntiles < 2 * num_sms ? ntiles : 2 * num_sms;
}

cudaError_t mlp_tc_forward(const void* img, const float* bias, const float* x, int in_stride,
                           int nin, const int* count, int n_max, float* y, int out_stride,
                           int* err, int err_bit, int grid, cudaStream_t st) {
  if (n_max <= 0 || grid <= 0) return cudaSuccess;
  k_mlp_tc<<<grid, kTcThreads, sizeof(TcSmem), st>>>(static_cast<const uint4*>(img), bias, x,
                                              in_stride, nin, count, n_max, y, out_stride, err,
                                              err_bit);
  return cudaGetLastError();
}

}  // namespace sps
