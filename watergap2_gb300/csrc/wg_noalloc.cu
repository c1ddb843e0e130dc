// wg_noalloc.cu -- wg_get_balance_noalloc: the water-balance sums of
// wg_get_balance for callers that cannot allocate device memory.
//
// Who needs it: a caller whose device memory is owned by someone else once the
// model is set up -- a host framework whose caching allocator holds the free
// device memory, or a driver that sizes every buffer at start and must not
// allocate afterwards.  wg_get_balance itself reduces into a per-block scratch
// buffer it allocates; this variant keeps that scratch in a fixed device array of
// this file, so the call allocates nothing.  The call still waits for the
// context's stream and copies the six sums to the caller's host array, so it is
// made outside CUDA stream capture.
//
// The array holds the partial sums of at most kNoallocMaxBlocks blocks of 256
// states, i.e. contexts of at most 16,777,216 states (cells x members); larger
// contexts are rejected with WG_ERR_INVALID.  Every GPU that loads the library
// holds the array (4 MiB) until the process exits.  All calls share it: calls
// that overlap on the GPU race on it, so run one at a time per device (the
// library's contexts are single-stream anyway).  Each call writes every entry it
// reads, so nothing needs clearing between calls.
//
// Host code must not use the array's name as a device address; the address is
// taken with cudaGetSymbolAddress on the device, with that device current, on the
// first call made on that device (a lookup that fails is not cached: the next
// call tries again).
#include <cuda_runtime.h>

#include <mutex>

#include "wg_device.h"
#include "wg_kernels.h"
#include "wg_volume.cuh"

namespace wg {

constexpr int kNoallocMaxBlocks = 65536;
constexpr int kNoallocThreads = 256;
constexpr size_t kNoallocScratchDoubles = (size_t)kNoallocMaxBlocks * 8 + 8;   // partials + result
static __device__ __align__(256) double g_noalloc_scratch[kNoallocScratchDoubles];

constexpr int kMaxDevices = 64;
static double *s_scratch[kMaxDevices];
static std::mutex s_scratch_mutex;

// Per-block partial sums, as k_balance_sum: 0 storage, 1 in, 2 evap, 3 outlet
// outflow, 4 clamp corrections (each Neumaier-compensated), 5 largest relative
// cell residual.
template <class R>
__global__ void __launch_bounds__(kNoallocThreads) k_balance_partials_static(DevCellsT<R> c, DevStateT<R> st, int M,
                                                                            DevBalance b, const double *vol0,
                                                                            double *scratch) {
  __shared__ double sh[6][kNoallocThreads];
  __shared__ double shc[5][kNoallocThreads];
  const size_t N = (size_t)c.n * M;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double val[6] = {0, 0, 0, 0, 0, 0};
  if (i < N) {
    const int s = (int)(i / M);
    const double vnow = cell_volume<R>(c, st, N, s, i);
    const double in = b.acc[0 * N + i] + b.acc[5 * N + i];
    const double ev = (b.acc[1 * N + i] + b.acc[6 * N + i]) + (b.acc[12 * N + i] + b.acc[13 * N + i]);
    const double out = b.acc[2 * N + i] + b.acc[7 * N + i];
    const double up = b.acc[3 * N + i] + b.acc[8 * N + i];
    const double lk = (b.acc[4 * N + i] + b.acc[9 * N + i]) + (b.acc[10 * N + i] + b.acc[11 * N + i]);
    val[0] = vnow;
    val[1] = in;
    val[2] = ev;
    val[3] = (c.flags[s] & F_OUTLET) ? out : 0.;
    val[4] = lk;
    const double resid = (vnow - vol0[i]) - (in - ev + up - out + lk);
    const double scale = fmax(fmax(fabs(vnow), fabs(vol0[i])), fmax(fmax(in, ev), fmax(up, out)));
    val[5] = scale > 0. ? fabs(resid) / scale : 0.;
  }
  for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] = val[k];
  for (int k = 0; k < 5; ++k) shc[k][threadIdx.x] = 0.;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      for (int k = 0; k < 5; ++k) {
        const double a = sh[k][threadIdx.x], x = sh[k][threadIdx.x + w];
        const double t = a + x;
        const double e = (fabs(a) >= fabs(x)) ? (a - t) + x : (x - t) + a;
        sh[k][threadIdx.x] = t;
        shc[k][threadIdx.x] += shc[k][threadIdx.x + w] + e;
      }
      sh[5][threadIdx.x] = fmax(sh[5][threadIdx.x], sh[5][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k) scratch[(size_t)blockIdx.x * 8 + k] = sh[k][0] + (k < 5 ? shc[k][0] : 0.);
}

// One block folds the nb partial rows in block order (Neumaier) into the result
// slot at the end of the scratch.
__global__ void __launch_bounds__(32) k_balance_final_static(double *scratch, int nb) {
  if (threadIdx.x != 0) return;
  double sum[5] = {0, 0, 0, 0, 0}, comp[5] = {0, 0, 0, 0, 0}, mx = 0.;
  for (int b = 0; b < nb; ++b) {
    for (int k = 0; k < 5; ++k) {
      const double x = scratch[(size_t)b * 8 + k], s = sum[k], t = s + x;
      comp[k] += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
      sum[k] = t;
    }
    mx = fmax(mx, scratch[(size_t)b * 8 + 5]);
  }
  double *res = scratch + (size_t)kNoallocMaxBlocks * 8;
  for (int k = 0; k < 5; ++k) res[k] = sum[k] + comp[k];
  res[5] = mx;
}

static cudaError_t noalloc_scratch(int device, double **out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(s_scratch_mutex);
  if (!s_scratch[device]) {
    // the caller has made `device` current; only a successful lookup is kept
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      *out = nullptr;
      return e;
    }
    s_scratch[device] = static_cast<double *>(p);
  }
  *out = s_scratch[device];
  return cudaSuccess;
}

int64_t noalloc_max_states() { return (int64_t)kNoallocMaxBlocks * kNoallocThreads; }

template <class R>
cudaError_t balance_noalloc(int device, const DevCellsT<R> &c, const DevStateT<R> &s, int M, const DevBalance &b,
                            const double *vol0, cudaStream_t st, double out[6]) {
  const size_t N = (size_t)c.n * M;
  if ((int64_t)N > noalloc_max_states()) return cudaErrorInvalidValue;
  if (N == 0) {   // no states: every sum is zero (a launch of zero blocks is an error)
    for (int k = 0; k < 6; ++k) out[k] = 0.;
    return cudaSuccess;
  }
  double *scratch = nullptr;
  cudaError_t e = noalloc_scratch(device, &scratch);
  if (e != cudaSuccess) return e;
  const int nb = (int)((N + kNoallocThreads - 1) / kNoallocThreads);
  k_balance_partials_static<R><<<nb, kNoallocThreads, 0, st>>>(c, s, M, b, vol0, scratch);
  k_balance_final_static<<<1, 32, 0, st>>>(scratch, nb);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(out, scratch + (size_t)kNoallocMaxBlocks * 8, 6 * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

template cudaError_t balance_noalloc<double>(int, const DevCellsT<double> &, const DevStateT<double> &, int,
                                             const DevBalance &, const double *, cudaStream_t, double[6]);
template cudaError_t balance_noalloc<float>(int, const DevCellsT<float> &, const DevStateT<float> &, int,
                                            const DevBalance &, const double *, cudaStream_t, double[6]);

}  // namespace wg
