// wg_kernels.h -- launchers of the kernels in wg_kernels.cu (host side).
#pragma once
#include <cuda_runtime.h>

#include "wg_device.h"

namespace wg {
// Largest block of the day-pipelined kernels (k_pipeline, k_vertical_ahead).
constexpr int kMaxBlockThreads = 512;

// Launch bounds of the day-pipelined kernels per arithmetic type: FP64 runs one
// block of up to 512 threads per SM (the single-member layout); FP32 blocks of at
// most 256 threads, three per SM, so that its registers leave room for the
// warps that hide its memory latency.
template <class R> struct Bounds;
template <> struct Bounds<double> { static constexpr int threads = 512, min_blocks = 1; };
template <> struct Bounds<float> { static constexpr int threads = 256, min_blocks = 3; };
// the ensemble's vertical-ahead kernel keeps a member's whole vertical state in
// registers: two blocks per SM, no spills
template <class R, bool ENS> struct VaBounds : Bounds<R> {};
template <> struct VaBounds<float, true> { static constexpr int threads = 256, min_blocks = 2; };
// the ensemble's wavefront kernel is bound by load latency: at most 128 threads
// per block and 64 registers, so that an SM holds 32 warps of it (no spills)
template <class R, bool ENS> struct PipeBounds : Bounds<R> {};
template <> struct PipeBounds<float, true> { static constexpr int threads = 128, min_blocks = 8; };
// the single-member FP64 wavefront with vertical-balance warps in the same block:
// up to 20 warps (5 per SM sub-partition, 96 registers each)
template <class R, bool ENS, bool VAW> struct WaveBounds : PipeBounds<R, ENS> {};
template <class R> struct WaveBounds<R, false, true> { static constexpr int threads = 640, min_blocks = 1; };

// Thread-to-slot layout of the single-member wavefront: each block runs
// cell_warps warps of 32 consecutive slots plus one idle warp at warp index
// idle_warp (idle_warp < 0: plain mapping, slot i on thread i mod the grid).
struct WarpLayout {
  int cell_warps = 0;
  int idle_warp = -1;
  int va_warps = 0;    // vertical-balance warps appended to each wavefront block (0: none)
  int blocks = 0;
  int threads = 0;
};
cudaError_t upload_fastmath_tables(const double exp2_tab[64], const double logF_tab[129], const double invF_tab[129]);
cudaError_t launch_math_eval(int fn, const double *x, const double *y, double *out, size_t n, cudaStream_t st);
cudaError_t launch_gather_forcing(const float *src, float *dst, const int32_t *cell_of_slot, int n, int ndays,
                                  cudaStream_t st);
cudaError_t launch_unf_forcing(const uint32_t *raw, float *dst, const int32_t *cell_of_slot, int n, int nd_file,
                               int d_first, int nd, cudaStream_t st, bool big_endian = true);
template <class R>
cudaError_t launch_vertical(const DevCellsT<R> &c, const DevStateT<R> &s, const DevVertT<R> &v, const DevForcing &f,
                            int doy, int fday, cudaStream_t st);
template <class R>
int pipeline_max_blocks(bool fused, bool ens, int threads, bool vaw = false, bool wt = false, bool wu = false);
// blocks of k_vertical_ahead resident on the whole device at once (its own occupancy)
template <class R>
int vertical_ahead_max_blocks(bool ens, int threads);
template <class R>
cudaError_t launch_pipeline(bool fused, const DevCellsT<R> &c, const DevStateT<R> &s, const DevVertT<R> &v,
                            const DevForcing &f, const DevMembers &mem, const DevBalance &b, const DevRingT<R> &ring,
                            const DevSync &sync, double *outq, double *qst, int doy0, int fday0, int oday0, int ndays,
                            int t_b, int t_e, int blocks, int threads, const WarpLayout &lay, const DevMonthly &mon,
                            const DevVaWork &vw, const DevWaterTemp &wtp, const DevWaterUse &wu, cudaStream_t st);
cudaError_t launch_fill(double *p, size_t n, double v, cudaStream_t st);
template <class R>
cudaError_t launch_vertical_ahead(const DevCellsT<R> &c, const DevStateT<R> &s, const DevForcing &f,
                                  const DevMembers &mem, const DevBalance &b, const DevRingT<R> &ring, int doy0,
                                  int fday0, int ndays, int t_b, int t_e, int blocks, int threads, cudaStream_t st,
                                  const DevMonthly &mon, int oday0);
template <class R>
cudaError_t launch_volume(const DevCellsT<R> &c, const DevStateT<R> &s, int M, double *vol, cudaStream_t st);
template <class R>
cudaError_t launch_balance_sum(const DevCellsT<R> &c, const DevStateT<R> &s, int M, const DevBalance &b,
                               const double *vol0, double *partial, int *nblocks, cudaStream_t st);
// wg_noalloc.cu: the balance sums with their scratch in a fixed device array
int64_t noalloc_max_states();
template <class R>
cudaError_t balance_noalloc(int device, const DevCellsT<R> &c, const DevStateT<R> &s, int M, const DevBalance &b,
                            const double *vol0, cudaStream_t st, double out[6]);
}  // namespace wg
