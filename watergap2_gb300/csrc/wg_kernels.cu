// wg_kernels.cu -- kernels of the GB300 WaterGAP2 daily step (sm_103a).
//
//  k_vertical      one thread per cell: calcNewDay for one day (daily.cpp:94-1257).
//  k_pipeline      persistent cooperative kernel: routing through the drainage
//                  tree as a wavefront over drainage levels; with FUSED it also
//                  runs the vertical balance and pipelines days, so that cell n
//                  computes day d at step d + offset(n) (offset = longest path -
//                  distance to the outlet).  Every upstream cell of n then has
//                  offset(n)-1 and delivers day d's outflow exactly one step
//                  earlier through a two-slot buffer; the only synchronisation
//                  is one grid barrier per step.
//  k_balance_sum   compensated (Neumaier) FP64 reduction of the balance terms.
//
// The grid barrier spins with an iteration limit: on timeout it raises the
// context's error word and every block returns (no trap, no endless wait).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "wg_device.h"
#include "wg_physics.cuh"
#include "wg_kernels.h"

namespace wg {

#define WG_BARRIER_SPIN_LIMIT (1u << 24)

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier for a cooperative launch (all blocks co-resident).  The
// counter only grows; round r completes when it reaches (r+1)*gridDim.x.
__device__ __forceinline__ bool grid_barrier(const DevSync &sync, unsigned round) {
  __syncthreads();
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    const unsigned target = (round + 1u) * gridDim.x;
    __threadfence();
    atomicAdd(sync.counter, 1u);
    unsigned it = 0;
    int ok = 1;
    while (ld_acquire(sync.counter) < target) {
      if (*(volatile int *)sync.error) { ok = 0; break; }
      if (++it > WG_BARRIER_SPIN_LIMIT) {
        atomicExch(sync.error, 1);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ void neumaier_add(double *acc, size_t k_sum, size_t k_comp, double x) {
  const double s = acc[k_sum];
  const double t = s + x;
  double c = acc[k_comp];
  if (fabs(s) >= fabs(x)) c += (s - t) + x;
  else c += (x - t) + s;
  acc[k_sum] = t;
  acc[k_comp] = c;
}

__device__ __forceinline__ void record_balance(const DevBalance &b, int n, int i, double in, double evap, double up,
                                               double out, double leak) {
  const size_t N = (size_t)n;
  neumaier_add(b.acc, 0 * N + i, 5 * N + i, in);
  neumaier_add(b.acc, 1 * N + i, 6 * N + i, evap);
  neumaier_add(b.acc, 2 * N + i, 7 * N + i, out);
  neumaier_add(b.acc, 3 * N + i, 8 * N + i, up);
  neumaier_add(b.acc, 4 * N + i, 9 * N + i, leak);
}

__global__ void __launch_bounds__(256) k_vertical(DevCells c, DevState s, DevVert v, DevForcing f, int doy, int fday) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const size_t fo = (size_t)fday * c.n + i;
  const double ext = c.ext_rad[(size_t)(doy - 1) * c.nrow + c.ext_row[i]];
  VOut o;
  vertical_cell(c, s, i, (double)f.prec[fo], (double)f.temp[fo], (double)f.swrad[fo], ext, o);
  v.rs[i] = o.rs; v.gwr[i] = o.gwr; v.transfer[i] = o.transfer; v.owp[i] = o.owp; v.owpet[i] = o.owpet;
  v.land_in[i] = o.land_in; v.land_evap[i] = o.land_evap; v.land_leak[i] = o.land_leak;
}

template <bool FUSED>
__global__ void __launch_bounds__(256) k_pipeline(DevCells c, DevState s, DevVert v, DevForcing f, DevBalance b,
                                                  DevSync sync, double *outq, double *qst, int doy0, int fday0,
                                                  int oday0, int ndays) {
  const int n = c.n;
  const int nsteps = ndays + c.nlevel - 1;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gstride = gridDim.x * blockDim.x;
  for (int t = 0; t < nsteps; ++t) {
    const int lo_off = max(0, t - ndays + 1), hi_off = min(c.nlevel - 1, t);
    if (lo_off <= hi_off) {
      const int lo = c.level_start[lo_off], hi = c.level_start[hi_off + 1];
      double *q_now = outq + (size_t)(t & 1) * n;
      const double *q_prev = outq + (size_t)((t + 1) & 1) * n;
      // slot i always belongs to thread i mod gstride, so a cell's state is read and
      // written by one thread; only upstream outflows cross threads (read via L2)
      int r0 = (gtid - lo) % gstride;
      if (r0 < 0) r0 += gstride;
      for (int i = lo + r0; i < hi; i += gstride) {
        const int d = t - c.offset[i];
        const int doy = (doy0 - 1 + d) % 365 + 1;
        const int month = month_of(doy);
        VOut o;
        if (FUSED) {
          const size_t fo = (size_t)(fday0 + d) * n + i;
          const double ext = c.ext_rad[(size_t)(doy - 1) * c.nrow + c.ext_row[i]];
          vertical_cell(c, s, i, (double)f.prec[fo], (double)f.temp[fo], (double)f.swrad[fo], ext, o);
        } else {
          o.rs = v.rs[i]; o.gwr = v.gwr[i]; o.transfer = v.transfer[i]; o.owp = v.owp[i]; o.owpet = v.owpet[i];
          o.land_in = v.land_in[i]; o.land_evap = v.land_evap[i]; o.land_leak = v.land_leak[i];
        }
        // upstream inflow: the reference sums pushes in routing order (routing.cpp:3955-3958)
        double up = 0.;
        const int u0 = c.up_ptr[i], u1 = c.up_ptr[i + 1];
        for (int k = u0; k < u1; ++k) up += __ldcg(q_prev + c.up_idx[k]);
        RTerms rt;
        const double land_f = c.area[i] * (s.laf[i] / 100.) / 1000000.;
        const double tv = routing_cell(c, s, i, doy, month, o, up, rt);
        q_now[i] = tv;
        if (b.enabled)
          record_balance(b, n, i, o.land_in * land_f + rt.p_ow, o.land_evap * land_f + rt.e_ow, up, tv,
                         o.land_leak * land_f + rt.leak);
        fraction_update(c, s, i);
        const int st = c.station[i];
        if (st >= 0) qst[(size_t)(oday0 + d) * c.nstation + st] = tv;
      }
    }
    if (t + 1 < nsteps) {
      if (!grid_barrier(sync, (unsigned)t)) return;
    }
  }
}

// Volume of the state of slot i [km3]: land storages (mm of the land fraction they
// were last rescaled to) plus groundwater and surface-water storages.
__device__ __forceinline__ double cell_volume(const DevCells &c, const DevState &s, int i) {
  double snow = 0.;
  for (int e = 0; e < c.nband; ++e) snow += s.snow_band[(size_t)e * c.n + i];
  snow /= (double)c.nband;
  const double laf = s.laf_started[i] ? s.laf_prev[i] : s.laf[i];
  const double f = c.area[i] * (laf / 100.) / 1000000.;
  return (s.canopy[i] + snow + s.soil[i]) * f + s.gw[i] + s.river[i] + s.loclake[i] + s.locwetl[i] + s.glolake[i] +
         s.glowetl[i] + s.res[i];
}

__global__ void k_volume(DevCells c, DevState s, double *vol) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < c.n) vol[i] = cell_volume(c, s, i);
}

// Block-level Neumaier reduction; out[blockIdx.x*8 + k] partial sums of
//   0 storage, 1 in, 2 evap, 3 outlet out, 4 leak, 5 max relative cell residual
__global__ void __launch_bounds__(256) k_balance_sum(DevCells c, DevState s, DevBalance b, const double *vol0,
                                                     double *partial) {
  __shared__ double sh[6][256];
  __shared__ double shc[6][256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double val[6] = {0, 0, 0, 0, 0, 0};
  if (i < c.n) {
    const size_t N = (size_t)c.n;
    const double vnow = cell_volume(c, s, i);
    const double in = b.acc[0 * N + i] + b.acc[5 * N + i];
    const double ev = b.acc[1 * N + i] + b.acc[6 * N + i];
    const double out = b.acc[2 * N + i] + b.acc[7 * N + i];
    const double up = b.acc[3 * N + i] + b.acc[8 * N + i];
    const double lk = b.acc[4 * N + i] + b.acc[9 * N + i];
    val[0] = vnow;
    val[1] = in;
    val[2] = ev;
    val[3] = (c.flags[i] & F_OUTLET) ? out : 0.;
    val[4] = lk;
    const double resid = (vnow - vol0[i]) - (in - ev + up - out + lk);
    const double scale = fmax(fmax(fabs(vnow), fabs(vol0[i])), fmax(fmax(in, ev), fmax(up, out)));
    val[5] = scale > 0. ? fabs(resid) / scale : 0.;
  }
  for (int k = 0; k < 6; ++k) {
    sh[k][threadIdx.x] = val[k];
    shc[k][threadIdx.x] = 0.;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      for (int k = 0; k < 5; ++k) {
        const double a = sh[k][threadIdx.x], x = sh[k][threadIdx.x + w];
        const double tsum = a + x;
        const double e = (fabs(a) >= fabs(x)) ? (a - tsum) + x : (x - tsum) + a;
        sh[k][threadIdx.x] = tsum;
        shc[k][threadIdx.x] += shc[k][threadIdx.x + w] + e;
      }
      sh[5][threadIdx.x] = fmax(sh[5][threadIdx.x], sh[5][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k) partial[blockIdx.x * 8 + k] = sh[k][0] + (k < 5 ? shc[k][0] : 0.);
}

// forcing arrives day-major in cell order; the device keeps it in slot order
__global__ void k_gather_forcing(const float *__restrict__ src, float *__restrict__ dst,
                                 const int32_t *__restrict__ cell_of_slot, int n, int ndays) {
  const size_t total = (size_t)n * ndays;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const size_t d = k / n;
    const int s = (int)(k - d * n);
    dst[k] = src[d * n + cell_of_slot[s]];
  }
}

// ---------------------------------------------------------------- launchers
cudaError_t launch_gather_forcing(const float *src, float *dst, const int32_t *cell_of_slot, int n, int ndays,
                                  cudaStream_t st) {
  const size_t total = (size_t)n * ndays;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, 152 * 16);
  k_gather_forcing<<<blocks, threads, 0, st>>>(src, dst, cell_of_slot, n, ndays);
  return cudaGetLastError();
}

cudaError_t launch_vertical(const DevCells &c, const DevState &s, const DevVert &v, const DevForcing &f, int doy,
                            int fday, cudaStream_t st) {
  const int threads = 256, blocks = (c.n + threads - 1) / threads;
  k_vertical<<<blocks, threads, 0, st>>>(c, s, v, f, doy, fday);
  return cudaGetLastError();
}

int pipeline_max_blocks(bool fused) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (fused) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pipeline<true>, 256, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pipeline<false>, 256, 0);
  return per * nsm;
}

cudaError_t launch_pipeline(bool fused, const DevCells &c, const DevState &s, const DevVert &v, const DevForcing &f,
                            const DevBalance &b, const DevSync &sync, double *outq, double *qst, int doy0, int fday0,
                            int oday0, int ndays, int blocks, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(sync.counter, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  void *args[] = {(void *)&c, (void *)&s, (void *)&v, (void *)&f, (void *)&b, (void *)&sync, (void *)&outq,
                  (void *)&qst, (void *)&doy0, (void *)&fday0, (void *)&oday0, (void *)&ndays};
  const void *fn = fused ? (const void *)k_pipeline<true> : (const void *)k_pipeline<false>;
  return cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(256), args, 0, st);
}

cudaError_t launch_volume(const DevCells &c, const DevState &s, double *vol, cudaStream_t st) {
  const int threads = 256, blocks = (c.n + threads - 1) / threads;
  k_volume<<<blocks, threads, 0, st>>>(c, s, vol);
  return cudaGetLastError();
}

cudaError_t launch_balance_sum(const DevCells &c, const DevState &s, const DevBalance &b, const double *vol0,
                               double *partial, int *nblocks, cudaStream_t st) {
  const int threads = 256, blocks = (c.n + threads - 1) / threads;
  *nblocks = blocks;
  k_balance_sum<<<blocks, threads, 0, st>>>(c, s, b, vol0, partial);
  return cudaGetLastError();
}

}  // namespace wg
