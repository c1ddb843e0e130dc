// wg_mlp.cu -- the calibration-step network: a 4-layer MLP of width 128 (BF16
// weights and activations, FP32 accumulation), trained and evaluated on the GPU
// by the kernels of this file.
//
// Every matrix product runs on the 5th-generation tensor cores: one thread of
// the CTA issues tcgen05.mma (kind::f16, BF16 x BF16 -> FP32) on operand tiles
// that the CTA has staged in shared memory in the canonical no-swizzle K-major
// layout, the accumulator lives in tensor memory (TMEM), and the four warps read
// it back with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31, i.e. the rows of
// its 32 samples) for the epilogue (bias, ReLU, BF16 rounding, gradients).
//
// Layers: x[128] -> 128 -> 128 -> 128 -> out[16] (inputs zero-padded to 128
// features, outputs to 16; the caller uses the first in_dim / out_dim).  One CTA
// of 128 threads handles a tile of 128 samples, thread t = sample t.
//
// Waits on the MMA-completion mbarrier are bounded; a wait that runs out sets
// the error word and the kernel still releases its TMEM before returning.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <random>
#include <vector>

#include "../../include/wg_mlp.h"

namespace wg {
namespace mlp {

constexpr int kTile = 128;                 // samples per CTA (MMA M)
constexpr int kW = 128;                    // hidden width = padded input width
constexpr int kOut = 16;                   // padded output width
constexpr int kTileBytes = kTile * kW * 2; // one 128 x 128 BF16 operand tile
constexpr uint32_t kTmemCols = 256;        // two 128-column FP32 accumulators
constexpr unsigned kWaitLimit = 1u << 24;

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, k) of a [rows x K] BF16 operand in the canonical
// no-swizzle K-major layout: 8 x 8 core matrices of 128 contiguous bytes (8 rows
// of 16 bytes); core matrices adjacent in K are 128 bytes apart (leading byte
// offset), those adjacent in rows K * 16 bytes apart (stride byte offset).
__device__ __forceinline__ uint32_t cm_off(int row, int k, int K) {
  return (uint32_t)((((row >> 3) * (K >> 3) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor (tcgen05): start >> 4 [0,14), leading byte
// offset >> 4 [16,30), stride byte offset >> 4 [32,46), version 1 at bit 46,
// base offset 0, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A BF16 (7-9 = 1),
// B BF16 (10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait for the phase `parity` of bar; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
  for (unsigned i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor cores (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes: thread = lane = row
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 16 columns (the output layer)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------- tile staging
// Copy a row-major [rows x K] BF16 matrix from global memory into the canonical
// layout at smem; 16-byte pieces, all threads of the CTA.
__device__ __forceinline__ void stage(char *smem, const __nv_bfloat16 *g, int rows, int K) {
  const int pieces = rows * (K >> 3);
  for (int p = threadIdx.x; p < pieces; p += blockDim.x) {
    const int row = p / (K >> 3), k8 = p % (K >> 3);
    const uint4 v = *reinterpret_cast<const uint4 *>(g + (size_t)row * K + k8 * 8);
    *reinterpret_cast<uint4 *>(smem + cm_off(row, k8 * 8, K)) = v;
  }
}

// D[128 x N] (TMEM columns col0..) = A[128 x K] * B[K x N], A and B staged K-major
// (B as [N][K]); issued by thread 0, completion signalled on bar.
__device__ __forceinline__ void gemm(uint32_t tmem, uint32_t col0, const char *A, const char *B, int N, int K,
                                     uint64_t *bar) {
  if (threadIdx.x == 0) {
    fence_after_sync();
    const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
    const uint32_t idesc = idesc_bf16(kTile, N);
    for (int k = 0; k < K; k += 16) {
      // two core matrices along K per instruction: advance by 2 x 128 bytes
      const uint64_t da = sdesc(a0 + (uint32_t)(k >> 3) * 128u, 128u, (uint32_t)K * 16u);
      const uint64_t db = sdesc(b0 + (uint32_t)(k >> 3) * 128u, 128u, (uint32_t)K * 16u);
      mma_bf16(tmem + col0, da, db, idesc, k > 0);
    }
    mma_commit(bar);
  }
}

struct Ctx {
  uint64_t *bar;
  unsigned phase;
  int *err;
  bool ok;
  // wait for the last committed MMA group; every thread
  __device__ __forceinline__ void wait() {
    if (ok && !mbar_wait(bar, phase & 1u)) {
      ok = false;
      atomicExch(err, 1);
    }
    phase++;
    fence_after_sync();
  }
};

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Network parameters on the device.  Master weights are FP32 (layer l: [out][in]);
// the tensor cores read BF16 copies W (as [out][in]) and, for the backward pass,
// WT (as [in][out]).
struct Params {
  const __nv_bfloat16 *W[4];    // [128][128] x 3, [16][128]
  const __nv_bfloat16 *WT[4];   // [128][128] x 3, [128][16]
  const float *b[4];            // [128] x 3, [16]
};

// -------------------------------------------------------------- the kernels
// Shared memory: bar (8) | tmem addr (4) | pad to 1024 | W tile 32 KB | act tile
// 32 KB | second act tile 32 KB | transposed tile 32 KB
constexpr int kSmemHead = 1024;
constexpr int kSmemBytes = kSmemHead + 4 * kTileBytes;

// Forward pass of the tiles of n samples (x: [n][128] BF16).  Writes y [n][16]
// (FP32) and, when h is non-null, the hidden activations h[l][n][128] (BF16, after
// ReLU) for the backward pass.
__global__ void __launch_bounds__(128, 1) k_mlp_forward(Params P, const __nv_bfloat16 *x, int n, float *y,
                                                        __nv_bfloat16 *h, int *err) {
  extern __shared__ __align__(1024) char smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + 8);
  char *wt = smem + kSmemHead;
  char *act = wt + kTileBytes;
  const int t = threadIdx.x, warp = t >> 5;
  if (t == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tslot, kTmemCols);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  Ctx cx{bar, 0u, err, true};
  for (int tile = blockIdx.x; tile * kTile < n; tile += gridDim.x) {
    const int s0 = tile * kTile;
    const int rows = min(kTile, n - s0);
    // input tile (rows beyond n are zero)
    for (int p = t; p < kTile * (kW >> 3); p += blockDim.x) {
      const int row = p / (kW >> 3), k8 = p % (kW >> 3);
      uint4 v = make_uint4(0, 0, 0, 0);
      if (row < rows) v = *reinterpret_cast<const uint4 *>(x + (size_t)(s0 + row) * kW + k8 * 8);
      *reinterpret_cast<uint4 *>(act + cm_off(row, k8 * 8, kW)) = v;
    }
    for (int l = 0; l < 4; ++l) {
      const int N = l < 3 ? kW : kOut;
      stage(wt, P.W[l], N, kW);
      fence_async_smem();
      fence_before_sync();
      __syncthreads();
      gemm(tmem, 0, act, wt, N, kW, bar);
      cx.wait();
      __syncthreads();   // every thread past the wait before act is rewritten
      if (l < 3) {
        for (int c = 0; c < kW; c += 32) {
          float v[32];
          tmem_ld32(tmem + lane_base + (uint32_t)c, v);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const float z = v[j] + P.b[l][c + j];
            const __nv_bfloat16 hb = __float2bfloat16_rn(z > 0.f ? z : 0.f);
            *reinterpret_cast<__nv_bfloat16 *>(act + cm_off(t, c + j, kW)) = hb;
            if (h && t < rows) h[((size_t)l * n + s0 + t) * kW + c + j] = hb;
          }
        }
      } else {
        float v[16];
        tmem_ld16(tmem + lane_base, v);
        if (t < rows)
          for (int j = 0; j < kOut; ++j) y[(size_t)(s0 + t) * kOut + j] = v[j] + P.b[3][j];
      }
      fence_before_sync();
      __syncthreads();
    }
  }
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// Backward pass of the loss sum_i ||y_i[:out_dim] - target_i||^2 / n_total
// for the tiles of n samples, after k_mlp_forward wrote y and h.  Accumulates the
// gradient of every parameter into grad (FP32, atomics; the caller zeroes it):
// grad layout = W0 [128][128], b0 [128], W1, b1, W2, b2, W3 [16][128], b3 [16].
__global__ void __launch_bounds__(128, 1) k_mlp_backward(Params P, const __nv_bfloat16 *x, const __nv_bfloat16 *h,
                                                         const float *y, const float *target, int out_dim, int n,
                                                         float inv_n_total, float *grad, float *loss, int *err) {
  extern __shared__ __align__(1024) char smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + 8);
  char *wt = smem + kSmemHead;              // W_l^T tile (B of the input-gradient GEMM)
  char *dz = wt + kTileBytes;               // dZ_l [sample][out] (A of the input-gradient GEMM)
  char *dzT = dz + kTileBytes;              // dZ_l as [out][sample] (B of the weight-gradient GEMM)
  char *hT = dzT + kTileBytes;              // H_{l-1} as [in][sample] (A of the weight-gradient GEMM)
  const int t = threadIdx.x, warp = t >> 5;
  if (t == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tslot, kTmemCols);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  Ctx cx{bar, 0u, err, true};
  size_t goff[4], gboff[4];
  {
    size_t o = 0;
    for (int l = 0; l < 4; ++l) {
      const int N = l < 3 ? kW : kOut;
      goff[l] = o;
      o += (size_t)N * kW;
      gboff[l] = o;
      o += N;
    }
  }
  for (int tile = blockIdx.x; tile * kTile < n; tile += gridDim.x) {
    const int s0 = tile * kTile;
    const int rows = min(kTile, n - s0);
    const bool live = t < rows;
    // dL/dy of this thread's sample, FP32 (16 columns, zero beyond out_dim)
    float g[kW];
    float lsum = 0.f;
#pragma unroll
    for (int j = 0; j < kOut; ++j) {
      float d = 0.f;
      if (live && j < out_dim) {
        const float e = y[(size_t)(s0 + t) * kOut + j] - target[(size_t)(s0 + t) * out_dim + j];
        lsum += e * e;
        d = 2.f * e * inv_n_total;
      }
      g[j] = d;
    }
    if (lsum != 0.f) atomicAdd(loss, lsum * inv_n_total);
    for (int l = 3; l >= 0; --l) {
      const int N = l < 3 ? kW : kOut;   // this layer's outputs
      // dZ_l: the incoming gradient times the ReLU mask of H_l (none on the output layer)
      for (int j = 0; j < N; ++j) {
        float d = g[j];
        if (l < 3 && live && !(__bfloat162float(h[((size_t)l * n + s0 + t) * kW + j]) > 0.f)) d = 0.f;
        if (!live) d = 0.f;
        const __nv_bfloat16 db = __float2bfloat16_rn(d);
        *reinterpret_cast<__nv_bfloat16 *>(dz + cm_off(t, j, N)) = db;       // [sample][out], K = N
        *reinterpret_cast<__nv_bfloat16 *>(dzT + cm_off(j, t, kTile)) = db;  // [out][sample], K = 128
        if (d != 0.f) atomicAdd(&grad[gboff[l] + j], d);                     // bias gradient
      }
      // H_{l-1} (the layer's input) as [in][sample]
      for (int i = 0; i < kW; ++i) {
        __nv_bfloat16 v = __float2bfloat16_rn(0.f);
        if (live) v = l > 0 ? h[((size_t)(l - 1) * n + s0 + t) * kW + i] : x[(size_t)(s0 + t) * kW + i];
        *reinterpret_cast<__nv_bfloat16 *>(hT + cm_off(i, t, kTile)) = v;
      }
      if (l > 0) stage(wt, P.WT[l], kW, N);   // W_l^T as [in][out] = B[K = out][N = in]
      fence_async_smem();
      fence_before_sync();
      __syncthreads();
      // weight gradient dW_l^T [in x out] = H_{l-1}^T [in x samples] * dZ_l [samples x out] -> cols 0..N
      if (threadIdx.x == 0) {
        fence_after_sync();
        const uint32_t idw = idesc_bf16(kTile, N);
        for (int k = 0; k < kTile; k += 16) {
          const uint64_t da = sdesc(smem_u32(hT) + (uint32_t)(k >> 3) * 128u, 128u, (uint32_t)kTile * 16u);
          const uint64_t db = sdesc(smem_u32(dzT) + (uint32_t)(k >> 3) * 128u, 128u, (uint32_t)kTile * 16u);
          mma_bf16(tmem, da, db, idw, k > 0);
        }
        if (l > 0) {
          // input gradient dH_{l-1} [samples x in] = dZ_l [samples x out] * W_l [out x in] -> cols 128..256
          const uint32_t idx = idesc_bf16(kTile, kW);
          for (int k = 0; k < N; k += 16) {
            const uint64_t da = sdesc(smem_u32(dz) + (uint32_t)(k >> 3) * 128u, 128u, (uint32_t)N * 16u);
            const uint64_t db = sdesc(smem_u32(wt) + (uint32_t)(k >> 3) * 128u, 128u, (uint32_t)N * 16u);
            mma_bf16(tmem + 128u, da, db, idx, k > 0);
          }
        }
        mma_commit(bar);
      }
      cx.wait();
      // thread t = input feature i = t: row t of dW_l^T -> grad W_l[:, t]
      for (int c = 0; c < N; c += 16) {
        float v[16];
        tmem_ld16(tmem + lane_base + (uint32_t)c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (v[j] != 0.f) atomicAdd(&grad[goff[l] + (size_t)(c + j) * kW + t], v[j]);
      }
      if (l > 0)
        for (int c = 0; c < kW; c += 32) tmem_ld32(tmem + lane_base + 128u + (uint32_t)c, g + c);
      fence_before_sync();
      __syncthreads();
    }
  }
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// Adam step on the FP32 master parameters; refreshes the BF16 copies W and WT.
__global__ void k_mlp_adam(float *theta, const float *grad, float *m, float *v, int count, float lr, float b1,
                           float b2, float eps, float c1, float c2, __nv_bfloat16 *wbf, __nv_bfloat16 *wtbf,
                           const int *woff, const int *wtoff) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float th = theta[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  theta[i] = th;
  // parameter i -> its BF16 copies (weights only; woff[i] < 0 for biases)
  const int o = woff[i];
  if (o >= 0) {
    wbf[o] = __float2bfloat16_rn(th);
    wtbf[wtoff[i]] = __float2bfloat16_rn(th);
  }
}

__global__ void k_to_bf16(const float *src, __nv_bfloat16 *dst, size_t count) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dst[i] = __float2bfloat16_rn(src[i]);
}

}  // namespace mlp
}  // namespace wg

// ------------------------------------------------------------------ host side
namespace {

using wg::mlp::kOut;
using wg::mlp::kTile;
using wg::mlp::kW;

constexpr int kLayerOut[4] = {kW, kW, kW, kOut};

struct Layout {
  size_t w[4], b[4], wb[4], total, wb_total;
  Layout() {
    size_t o = 0, q = 0;
    for (int l = 0; l < 4; ++l) {
      w[l] = o;
      o += (size_t)kLayerOut[l] * kW;
      b[l] = o;
      o += kLayerOut[l];
      wb[l] = q;
      q += (size_t)kLayerOut[l] * kW;
    }
    total = o;
    wb_total = q;
  }
};
const Layout kLay;

__global__ void k_gather_rows(const __nv_bfloat16 *x, const float *t, const int *perm, int out_dim, int n,
                              __nv_bfloat16 *xb, float *tb) {
  const int r = blockIdx.x, c = threadIdx.x;   // one block per row, 128 threads
  if (r >= n) return;
  const int src = perm[r];
  xb[(size_t)r * kW + c] = x[(size_t)src * kW + c];
  if (c < out_dim) tb[(size_t)r * out_dim + c] = t[(size_t)src * out_dim + c];
}

__global__ void k_refresh_bf16(const float *theta, const int *woff, const int *wtoff, int count, __nv_bfloat16 *wbf,
                               __nv_bfloat16 *wtbf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count || woff[i] < 0) return;
  wbf[woff[i]] = __float2bfloat16_rn(theta[i]);
  wtbf[wtoff[i]] = __float2bfloat16_rn(theta[i]);
}

}  // namespace

struct wg_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  float *theta = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
  __nv_bfloat16 *wbf = nullptr, *wtbf = nullptr;
  int *woff = nullptr, *wtoff = nullptr, *err = nullptr;
  // data buffers (grown on demand)
  __nv_bfloat16 *x = nullptr, *h = nullptr, *xb = nullptr;
  float *xf = nullptr, *y = nullptr, *t = nullptr, *tb = nullptr;
  int *perm = nullptr;
  size_t cap = 0, cap_batch = 0;
  int64_t steps = 0;
  std::vector<void *> allocs;
  int nsm = 1;

  template <class T>
  T *alloc(size_t count) {
    void *p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return (T *)p;
  }
  ~wg_mlp() {
    for (void *p : allocs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
  wg::mlp::Params params() const {
    wg::mlp::Params P;
    for (int l = 0; l < 4; ++l) {
      P.W[l] = wbf + kLay.wb[l];
      P.WT[l] = wtbf + kLay.wb[l];
      P.b[l] = theta + kLay.b[l];
    }
    return P;
  }
  // data buffers for n samples (x as FP32 staging and BF16, y, h, targets)
  bool reserve(size_t n) {
    if (n <= cap) return true;
    cap = n;
    xf = alloc<float>(n * kW);
    x = alloc<__nv_bfloat16>(n * kW);
    y = alloc<float>(n * kOut);
    t = alloc<float>(n * kOut);
    perm = alloc<int>(n);
    return xf && x && y && t && perm;
  }
  bool reserve_batch(size_t nb) {
    if (nb <= cap_batch) return true;
    cap_batch = nb;
    h = alloc<__nv_bfloat16>(3 * nb * kW);
    xb = alloc<__nv_bfloat16>(nb * kW);
    tb = alloc<float>(nb * kOut);
    return h && xb && tb;
  }
};

namespace {

wg_status check(wg_mlp *m, cudaError_t e) {
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? WG_ERR_NOMEM : WG_ERR_CUDA;
  int flag = 0;
  if (cudaMemcpy(&flag, m->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return WG_ERR_CUDA;
  return flag ? WG_ERR_TIMEOUT : WG_OK;
}

int grid_for(const wg_mlp *m, int n) { return std::max(1, std::min((n + kTile - 1) / kTile, m->nsm)); }

cudaError_t forward(wg_mlp *m, const __nv_bfloat16 *x, int n, float *y, __nv_bfloat16 *h) {
  wg::mlp::k_mlp_forward<<<grid_for(m, n), 128, wg::mlp::kSmemBytes, m->stream>>>(m->params(), x, n, y, h, m->err);
  return cudaGetLastError();
}

cudaError_t backward(wg_mlp *m, const __nv_bfloat16 *x, const __nv_bfloat16 *h, const float *t, int out_dim, int n,
                     float inv_n) {
  wg::mlp::k_mlp_backward<<<grid_for(m, n), 128, wg::mlp::kSmemBytes, m->stream>>>(
      m->params(), x, h, m->y, t, out_dim, n, inv_n, m->grad, m->loss, m->err);
  return cudaGetLastError();
}

cudaError_t upload_x(wg_mlp *m, const float *x, int n) {
  cudaError_t e = cudaMemcpyAsync(m->xf, x, (size_t)n * kW * sizeof(float), cudaMemcpyHostToDevice, m->stream);
  if (e != cudaSuccess) return e;
  const size_t cnt = (size_t)n * kW;
  wg::mlp::k_to_bf16<<<(unsigned)((cnt + 255) / 256), 256, 0, m->stream>>>(m->xf, m->x, cnt);
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int32_t wg_mlp_num_params(void) { return (int32_t)kLay.total; }

wg_status wg_mlp_create(int32_t device, uint64_t seed, wg_mlp **out) {
  if (!out) return WG_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return WG_ERR_DEVICE;
  cudaSetDevice(device);
  int major = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  if (major < 10) return WG_ERR_DEVICE;
  std::unique_ptr<wg_mlp> m(new wg_mlp());
  m->device = device;
  cudaDeviceGetAttribute(&m->nsm, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) return WG_ERR_CUDA;
  if (cudaFuncSetAttribute(wg::mlp::k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           wg::mlp::kSmemBytes) != cudaSuccess ||
      cudaFuncSetAttribute(wg::mlp::k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           wg::mlp::kSmemBytes) != cudaSuccess)
    return WG_ERR_CUDA;
  const size_t P = kLay.total;
  m->theta = m->alloc<float>(P);
  m->grad = m->alloc<float>(P);
  m->m = m->alloc<float>(P);
  m->v = m->alloc<float>(P);
  m->loss = m->alloc<float>(1);
  m->err = m->alloc<int>(1);
  m->wbf = m->alloc<__nv_bfloat16>(kLay.wb_total);
  m->wtbf = m->alloc<__nv_bfloat16>(kLay.wb_total);
  m->woff = m->alloc<int>(P);
  m->wtoff = m->alloc<int>(P);
  if (!m->theta || !m->grad || !m->m || !m->v || !m->loss || !m->err || !m->wbf || !m->wtbf || !m->woff ||
      !m->wtoff)
    return WG_ERR_NOMEM;
  std::vector<int> woff(P, -1), wtoff(P, -1);
  std::vector<float> theta(P, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < 4; ++l) {
    const int N = kLayerOut[l];
    const float a = std::sqrt(6.0f / kW) * (l == 3 ? 0.1f : 1.0f);
    std::uniform_real_distribution<float> U(-a, a);
    for (int o = 0; o < N; ++o)
      for (int i = 0; i < kW; ++i) {
        const size_t p = kLay.w[l] + (size_t)o * kW + i;
        theta[p] = U(rng);
        woff[p] = (int)(kLay.wb[l] + (size_t)o * kW + i);
        wtoff[p] = (int)(kLay.wb[l] + (size_t)i * N + o);
      }
  }
  cudaError_t e = cudaMemcpy(m->woff, woff.data(), P * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->wtoff, wtoff.data(), P * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->err, 0, sizeof(int));
  if (e != cudaSuccess) return WG_ERR_CUDA;
  *out = m.release();
  wg_status st = wg_mlp_set_params(*out, theta.data());
  if (st != WG_OK) {
    delete *out;
    *out = nullptr;
  }
  return st;
}

wg_status wg_mlp_destroy(wg_mlp *m) {
  if (!m) return WG_ERR_INVALID;
  cudaSetDevice(m->device);
  cudaStreamSynchronize(m->stream);
  delete m;
  return WG_OK;
}

wg_status wg_mlp_set_params(wg_mlp *m, const float *theta) {
  if (!m || !theta) return WG_ERR_INVALID;
  cudaSetDevice(m->device);
  const int P = (int)kLay.total;
  cudaError_t e = cudaMemcpyAsync(m->theta, theta, P * sizeof(float), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->m, 0, P * sizeof(float), m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->v, 0, P * sizeof(float), m->stream);
  if (e == cudaSuccess) {
    k_refresh_bf16<<<(P + 255) / 256, 256, 0, m->stream>>>(m->theta, m->woff, m->wtoff, P, m->wbf, m->wtbf);
    e = cudaGetLastError();
  }
  m->steps = 0;
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  return check(m, e);
}

wg_status wg_mlp_get_params(wg_mlp *m, float *theta) {
  if (!m || !theta) return WG_ERR_INVALID;
  cudaSetDevice(m->device);
  cudaError_t e = cudaStreamSynchronize(m->stream);
  if (e == cudaSuccess) e = cudaMemcpy(theta, m->theta, kLay.total * sizeof(float), cudaMemcpyDeviceToHost);
  return check(m, e);
}

wg_status wg_mlp_forward(wg_mlp *m, const float *x, int32_t n, float *y) {
  if (!m || !x || !y || n <= 0) return WG_ERR_INVALID;
  cudaSetDevice(m->device);
  if (!m->reserve(n)) return WG_ERR_NOMEM;
  cudaError_t e = upload_x(m, x, n);
  if (e == cudaSuccess) e = forward(m, m->x, n, m->y, nullptr);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(y, m->y, (size_t)n * kOut * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  return check(m, e);
}

wg_status wg_mlp_gradient(wg_mlp *m, const float *x, const float *target, int32_t out_dim, int32_t n, float *grad,
                          float *loss) {
  if (!m || !x || !target || !grad || !loss || n <= 0 || out_dim <= 0 || out_dim > kOut) return WG_ERR_INVALID;
  cudaSetDevice(m->device);
  if (!m->reserve(n) || !m->reserve_batch(n)) return WG_ERR_NOMEM;
  cudaError_t e = upload_x(m, x, n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m->t, target, (size_t)n * out_dim * sizeof(float), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->grad, 0, kLay.total * sizeof(float), m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream);
  if (e == cudaSuccess) e = forward(m, m->x, n, m->y, m->h);
  if (e == cudaSuccess) e = backward(m, m->x, m->h, m->t, out_dim, n, 1.0f / n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(grad, m->grad, kLay.total * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  return check(m, e);
}

wg_status wg_mlp_train(wg_mlp *m, const float *x, const float *target, int32_t out_dim, int32_t n, int32_t epochs,
                       int32_t batch, float lr, uint64_t seed, float *final_loss) {
  if (!m || !x || !target || n <= 0 || out_dim <= 0 || out_dim > kOut || epochs <= 0 || batch <= 0 ||
      batch % kTile || batch > n || !(lr > 0.f))
    return WG_ERR_INVALID;
  cudaSetDevice(m->device);
  if (!m->reserve(n) || !m->reserve_batch(batch)) return WG_ERR_NOMEM;
  cudaError_t e = upload_x(m, x, n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m->t, target, (size_t)n * out_dim * sizeof(float), cudaMemcpyHostToDevice, m->stream);
  const int P = (int)kLay.total;
  const int nbatch = n / batch;
  std::vector<int> perm(n);
  std::mt19937_64 rng(seed);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  float last = 0.f;
  for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
    for (int i = 0; i < n; ++i) perm[i] = i;
    std::shuffle(perm.begin(), perm.end(), rng);
    e = cudaMemcpyAsync(m->perm, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream);
    for (int bi = 0; bi < nbatch && e == cudaSuccess; ++bi) {
      k_gather_rows<<<batch, kW, 0, m->stream>>>(m->x, m->t, m->perm + (size_t)bi * batch, out_dim, batch, m->xb,
                                                 m->tb);
      e = cudaMemsetAsync(m->grad, 0, P * sizeof(float), m->stream);
      if (e == cudaSuccess) e = forward(m, m->xb, batch, m->y, m->h);
      if (e == cudaSuccess) e = backward(m, m->xb, m->h, m->tb, out_dim, batch, 1.0f / batch);
      if (e != cudaSuccess) break;
      m->steps++;
      const float c1 = 1.f / (1.f - std::pow(b1, (float)m->steps));
      const float c2 = 1.f / (1.f - std::pow(b2, (float)m->steps));
      wg::mlp::k_mlp_adam<<<(P + 255) / 256, 256, 0, m->stream>>>(m->theta, m->grad, m->m, m->v, P, lr, b1, b2, eps,
                                                                   c1, c2, m->wbf, m->wtbf, m->woff, m->wtoff);
      e = cudaGetLastError();
    }
    float lsum = 0.f;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&lsum, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    last = lsum / nbatch;
    wg_status st = check(m, e);
    if (st != WG_OK) return st;
  }
  if (final_loss) *final_loss = last;
  return check(m, e);
}

}  // extern "C"
