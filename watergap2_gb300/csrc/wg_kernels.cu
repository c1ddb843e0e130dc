// wg_kernels.cu -- kernels of the GB300 WaterGAP2 daily step (sm_103a).
//
//  k_vertical      one thread per cell: calcNewDay for one day (daily.cpp:94-1257),
//                  the reference's per-day call granularity.
//  k_pipeline      persistent cooperative kernel: routing through the drainage
//                  tree as a wavefront over drainage levels.  With FUSED it also
//                  runs the vertical balance and pipelines days: cell n computes
//                  day d at step d + offset(n), offset = longest flow path -
//                  distance of n to its outlet.  Every upstream cell of n then
//                  has offset(n) - 1 and delivers day d's outflow exactly one step
//                  earlier through a two-slot buffer, so one grid barrier per step
//                  (or, optionally, per-warp step flags) is the only
//                  synchronisation and every step keeps all cells busy.  Cells
//                  without a water body take their vertical balance from the ring
//                  that k_vertical_ahead filled; the monthly output aggregates are
//                  accumulated in its epilogue.  With ENS the cells carry
//                  `members` independent states (ensemble members), innermost in
//                  memory.  With VAW (one FP64 member) each block has five more
//                  warps that run k_vertical_ahead's work for the next chunk
//                  while the routing warps wait; with WT every cell also gets
//                  its water temperature (calcWTemp), the river temperature
//                  travelling downstream beside the outflow.
//  k_vertical_ahead  the vertical balance of the cells without a water body for
//                  a chunk of days, state in registers, into the ring.
//  k_math_eval     the FP64 path's exp/log/pow/reciprocal on arrays (tests).
//  k_unf_forcing / k_gather_forcing  forcing uploads into the slot layout.
//  k_volume / k_balance_sum   compensated (Neumaier) FP64 water-balance sums.
//
// Precision: R = double is the plain FP64 path; R = float keeps state and
// fluxes in FP32 while confluence sums, the outflow buffer and all balance
// sums stay FP64.  The grid barrier spins with an iteration limit: on timeout
// it raises the context's error word and every block returns (no trap).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>

#include "wg_device.h"
#include "wg_kernels.h"
#include "wg_physics.cuh"
#include "wg_volume.cuh"
#include "wg_wtemp.cuh"

namespace wg {

#define WG_BARRIER_SPIN_LIMIT (1u << 24)

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier for a cooperative launch (all blocks co-resident).  The
// counter only grows; round r completes when it reaches (r+1)*gridDim.x.
// Block-level part of the grid barrier: all threads of the block, or (nthr <
// blockDim.x) the first nthr threads only, on hardware barrier 1, while the
// block's other warps do independent work.
__device__ __forceinline__ void block_sync(int nthr) {
  if (nthr == (int)blockDim.x) __syncthreads();
  else asm volatile("bar.sync 1, %0;" ::"r"(nthr) : "memory");
}

__device__ __forceinline__ bool grid_barrier(const DevSync &sync, unsigned round, int nthr) {
  block_sync(nthr);
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    const unsigned target = (round + 1u) * gridDim.x + sync.extra_arrivals;
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
  block_sync(nthr);
  return s_ok != 0;
}

__device__ __forceinline__ int ld_acquire_int(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_int(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Step flags: wait until every warp this warp depends on has completed step
// `need` (relative).  The lanes share the dependency list; bounded like the grid
// barrier (a wait that runs out sets the error word; the caller then stops).
__device__ __forceinline__ bool wait_deps(const DevSync &sync, int w, int need) {
  bool ok = true;
  const int k0 = sync.dep_ptr[w], k1 = sync.dep_ptr[w + 1];
  for (int k = k0 + (int)(threadIdx.x & 31); k < k1; k += 32) {
    const int *flag = sync.wstep + sync.dep_idx[k];
    unsigned it = 0;
    while (ld_acquire_int(flag) < need) {
      if (*(volatile int *)sync.error || ++it > WG_BARRIER_SPIN_LIMIT) {
        atomicExch(sync.error, 1);
        ok = false;
        break;
      }
      __nanosleep(32);
    }
    if (!ok) break;
  }
  return __all_sync(0xffffffffu, ok);
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

__device__ __forceinline__ void record_routing_balance(const DevBalance &b, size_t N, size_t i, double up,
                                                       double out, double leak) {
  neumaier_add(b.acc, 2 * N + i, 7 * N + i, out);
  neumaier_add(b.acc, 3 * N + i, 8 * N + i, up);
  neumaier_add(b.acc, 4 * N + i, 9 * N + i, leak);
}

__device__ __forceinline__ void record_balance(const DevBalance &b, size_t N, size_t i, double in, double evap,
                                               double up, double out, double leak) {
  neumaier_add(b.acc, 0 * N + i, 5 * N + i, in);
  neumaier_add(b.acc, 1 * N + i, 6 * N + i, evap);
  neumaier_add(b.acc, 2 * N + i, 7 * N + i, out);
  neumaier_add(b.acc, 3 * N + i, 8 * N + i, up);
  neumaier_add(b.acc, 4 * N + i, 9 * N + i, leak);
}

template <class R>
__device__ __forceinline__ RState<R> load_rstate(const DevStateT<R> &s, size_t i, uint32_t fl) {
  RState<R> r;
  r.gw = s.gw[i];
  r.river = s.river[i];
  r.loclake = (fl & F_LOCLAKE) ? s.loclake[i] : R(0);
  r.rf_loclake = (fl & F_LOCLAKE) ? s.rf_loclake[i] : R(0);
  r.locwetl = (fl & F_LOCWETL) ? s.locwetl[i] : R(0);
  r.rf_locwetl = (fl & F_LOCWETL) ? s.rf_locwetl[i] : R(0);
  r.glolake = (fl & F_GLOLAKE) ? s.glolake[i] : R(0);
  r.rf_glolake = (fl & F_GLOLAKE) ? s.rf_glolake[i] : R(0);
  r.glowetl = (fl & F_GLOWETL) ? s.glowetl[i] : R(0);
  r.rf_glowetl = (fl & F_GLOWETL) ? s.rf_glowetl[i] : R(0);
  r.res = (fl & F_RES) ? s.res[i] : R(0);
  r.rf_res = (fl & F_RES) ? s.rf_res[i] : R(0);
  r.k_release = (fl & F_RES) ? s.k_release[i] : R(0);
  return r;
}

// Store only what the cell's water bodies can have changed.
template <class R>
__device__ __forceinline__ void store_rstate(const DevStateT<R> &s, size_t i, const RState<R> &r, uint32_t fl) {
  s.gw[i] = r.gw;
  s.river[i] = r.river;
  if (fl & F_LOCLAKE) { s.loclake[i] = r.loclake; s.rf_loclake[i] = r.rf_loclake; }
  if (fl & F_LOCWETL) { s.locwetl[i] = r.locwetl; s.rf_locwetl[i] = r.rf_locwetl; }
  if (fl & F_GLOLAKE) { s.glolake[i] = r.glolake; s.rf_glolake[i] = r.rf_glolake; }
  if (fl & F_GLOWETL) { s.glowetl[i] = r.glowetl; s.rf_glowetl[i] = r.rf_glowetl; }
  if (fl & F_RES) { s.res[i] = r.res; s.rf_res[i] = r.rf_res; s.k_release[i] = r.k_release; }
}

// One cell-day of the vertical balance on state index si (slot s).
template <class R>
__device__ __forceinline__ void vertical_at(const DevCellsT<R> &c, const DevStateT<R> &st, size_t N, int s,
                                            size_t si, int doy, R Pin, R gamma_soil, float Tf, float SWf, R laf,
                                            R prev, VOut<R> &o, const VSink *vs = nullptr) {
  if (c.flags[s] & F_NOCONT) {   // no vertical balance: the terms stay 0, the state as it is
    o.rs = R(0); o.gwr = R(0); o.transfer = R(0); o.owp = R(0); o.owpet = R(0);
    o.land_in = R(0); o.land_evap = R(0); o.land_leak = R(0);
    return;
  }
  const size_t ti = (size_t)(doy - 1) * c.nrow + c.ext_row[s];
  const R ext = c.ext_rad[ti], inv_s0 = c.inv_s0[ti];
  R canopy = st.canopy[si], soil = st.soil[si], gsnow = st.snow[si], psum = st.lai_precsum[si];
  int days = st.lai_days[si], status = st.lai_status[si];
  if (vs)   // the output grids (FP64 single member)
    vertical_cell<R, std::is_same<R, double>::value>(c, s, gamma_soil, canopy, soil, gsnow, st.snow_band + si, N,
                                                      days, status, psum, laf, prev, Pin, Tf, SWf, ext, inv_s0, o, vs);
  else
    vertical_cell<R>(c, s, gamma_soil, canopy, soil, gsnow, st.snow_band + si, N, days, status, psum, laf, prev, Pin,
                     Tf, SWf, ext, inv_s0, o);
  st.canopy[si] = canopy; st.soil[si] = soil; st.snow[si] = gsnow; st.lai_precsum[si] = psum;
  st.lai_days[si] = days; st.lai_status[si] = status;
}

template <class R>
__global__ void __launch_bounds__(256) k_vertical(DevCellsT<R> c, DevStateT<R> st, DevVertT<R> v, DevForcing f,
                                                  int doy, int fday) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.n || (c.active && !c.active[s])) return;
  const size_t fo = (size_t)fday * c.n + s;
  VOut<R> o;
  const R laf = st.laf[s];
  const R prev = (st.laf_started[s] == 1) ? st.laf_prev[s] : laf;   // daily.cpp:159-169
  vertical_at<R>(c, st, (size_t)c.n, s, (size_t)s, doy, R(f.prec[fo]), c.gamma[s], f.temp[fo], f.swrad[fo], laf, prev,
                 o);
  v.rs[s] = o.rs; v.gwr[s] = o.gwr; v.transfer[s] = o.transfer; v.owp[s] = o.owp; v.owpet[s] = o.owpet;
  v.land_in[s] = o.land_in; v.land_evap[s] = o.land_evap; v.land_leak[s] = o.land_leak;
}

// Vertical balance ahead of routing for the cells whose land fraction and open-water
// fluxes do not depend on routing (no water body): each thread takes one
// (cell, member) through the days the pipeline steps [t_b, t_e) will route, with
// the vertical state in registers, and leaves surface runoff and recharge in the
// ring buffer.  Results equal the in-wavefront computation: the vertical balance of
// such a cell reads nothing routing writes.
// One (cell, member) state index i of the vertical balance run ahead: the days
// the wavefront steps [t_b, t_e) will route, vertical state in registers, surface
// runoff and recharge into the ring; balance terms into arrays 0, 1 and 10.
// The output grids of state si for output day od: its entry in the vertical
// balance's monthly grids (the month of the output calendar, as the routing
// aggregates count it) and in the daily grids, each null when the grids are off
// or the day is outside them.  False: no grid takes the day.
__device__ __forceinline__ bool vert_sink(const DevMonthly &mon, int od, size_t si, size_t N, VSink &vs) {
  vs.mo = nullptr;
  vs.dd = nullptr;
  if (mon.vert) {
    const int yd = mon.doy_day0 - 1 + od;
    const int mi = (yd / 365) * 12 + month_of(yd % 365 + 1) - mon.month0;
    if (mi >= 0 && mi < mon.nmonths) vs.mo = mon.vert + (size_t)mi * N + si;
  }
  if (mon.dvert && od >= 0 && od < mon.dvert_days) vs.dd = mon.dvert + (size_t)od * N + si;
  vs.mos = (size_t)mon.nmonths * N;
  vs.dds = (size_t)mon.dvert_days * N;
  vs.vk = mon.vconst + si;
  vs.vks = N;
  return vs.mo || vs.dd;
}

template <class R, bool ENS>
__device__ __forceinline__ void va_cell(const DevCellsT<R> &c, const DevStateT<R> &st, const DevForcing &f,
                                        const DevMembers &mem, const DevBalance &b, const DevRingT<R> &ring,
                                        int doy0, int fday0, int ndays, int t_b, int t_e, size_t i, size_t N,
                                        const DevMonthly *mon = nullptr, int oday0 = 0) {
  const int n = c.n;
  const int M = ENS ? mem.members : 1;
  const int s = ENS ? (int)(i / M) : (int)i;
  const int mm = ENS ? (int)(i - (size_t)s * M) : 0;
  if ((c.flags[s] & F_VINLINE) || (c.active && !c.active[s])) return;
  const int off = c.offset[s];
  const int kd = ring.days_per_step;   // step t routes days kd*(t-off) .. kd*(t-off)+kd-1
  const int d0 = max(0, kd * (t_b - off)), d1 = min(ndays, kd * (t_e - off));
  if (d0 >= d1) return;
  R canopy = st.canopy[i], soil = st.soil[i], gsnow = st.snow[i], psum = st.lai_precsum[i];
  int days = st.lai_days[i], status = st.lai_status[i];
  const R laf = st.laf[i];   // constant for these cells (no water body)
  R pf = R(1), gam = c.gamma[s];
  if (ENS) {
    pf = R(mem.prec_factor[mm]);
    gam *= R(mem.gamma_factor[mm]);
  }
  double acc_in = 0., acc_ev = 0., acc_lk = 0.;
  const double land_f = (double)c.area_f[s] * (double)laf;
  for (int d = d0; d < d1; ++d) {
    const int doy = (doy0 - 1 + d) % 365 + 1;
    const size_t fo = (size_t)(fday0 + d) * n + s;
    const size_t ti = (size_t)(doy - 1) * c.nrow + c.ext_row[s];
    VOut<R> o;
    VSink vs;
    if (!ENS && mon && vert_sink(*mon, oday0 + d, i, N, vs))   // the output grids (FP64 single member)
      vertical_cell<R, std::is_same<R, double>::value>(c, s, gam, canopy, soil, gsnow, st.snow_band + i, N, days,
                                                        status, psum, laf, laf, R(f.prec[fo]) * pf, f.temp[fo],
                                                        f.swrad[fo], c.ext_rad[ti], c.inv_s0[ti], o, &vs);
    else
      vertical_cell<R>(c, s, gam, canopy, soil, gsnow, st.snow_band + i, N, days, status, psum, laf, laf,
                       R(f.prec[fo]) * pf, f.temp[fo], f.swrad[fo], c.ext_rad[ti], c.inv_s0[ti], o);
    const size_t ri = (size_t)(d % ring.ring_days) * N + i;
    ring.rs[ri] = o.rs;
    ring.gwr[ri] = o.gwr;
    if (ring.owp) {   // the water temperature's open-water terms of the river
      ring.owp[ri] = o.owp;
      ring.owpet[ri] = o.owpet;
    }
    if (b.enabled) {
      acc_in += (double)o.land_in * land_f;
      acc_ev += (double)o.land_evap * land_f;
      acc_lk += (double)o.land_leak * land_f;
    }
  }
  st.canopy[i] = canopy; st.soil[i] = soil; st.snow[i] = gsnow; st.lai_precsum[i] = psum;
  st.lai_days[i] = days; st.lai_status[i] = status;
  if (b.enabled) {
    neumaier_add(b.acc, 0 * N + i, 5 * N + i, acc_in);
    neumaier_add(b.acc, 1 * N + i, 6 * N + i, acc_ev);
    neumaier_add(b.acc, 10 * N + i, 11 * N + i, acc_lk);
  }
}

// Vertical balance ahead of routing for the cells whose land fraction and open-water
// fluxes do not depend on routing (no water body): each thread takes one
// (cell, member) through the days the pipeline steps [t_b, t_e) will route, with
// the vertical state in registers, and leaves surface runoff and recharge in the
// ring buffer.  Results equal the in-wavefront computation: the vertical balance of
// such a cell reads nothing routing writes.
// OUT: the vertical balance's monthly output grids too (DevMonthly::vert, FP64 single member).
template <class R, bool ENS, bool OUT = false>
__global__ void __launch_bounds__(VaBounds<R, ENS>::threads, VaBounds<R, ENS>::min_blocks) k_vertical_ahead(DevCellsT<R> c, DevStateT<R> st, DevForcing f,
                                                        DevMembers mem, DevBalance b, DevRingT<R> ring, int doy0,
                                                        int fday0, int ndays, int t_b, int t_e, DevMonthly mon,
                                                        int oday0) {
  const size_t N = (size_t)c.n * (ENS ? mem.members : 1);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
    va_cell<R, ENS>(c, st, f, mem, b, ring, doy0, fday0, ndays, t_b, t_e, i, N, OUT ? &mon : nullptr, oday0);
}

// X: what each cell computes after its routing, bit 0 the water temperature,
// bit 1 the water use, bit 2 (with bit 1) the water use of GLWD units' riparian
// cells met by their outflow cell, bit 3 the vertical balance's monthly output
// grids (FP64 single member, alone).
template <class R, bool FUSED, bool ENS, bool VAW, int X>
__global__ void __launch_bounds__(WaveBounds<R, ENS, VAW>::threads, WaveBounds<R, ENS, VAW>::min_blocks) k_pipeline(DevCellsT<R> c, DevStateT<R> st, DevVertT<R> v, DevForcing f,
                                                  DevMembers mem, DevBalance b, DevRingT<R> ring, DevSync sync,
                                                  double *outq, double *qst, int doy0, int fday0, int oday0,
                                                  int ndays, int t_b, int t_e, int cell_warps, int idle_warp,
                                                  DevMonthly mon, DevVaWork vw, DevWaterTemp wtp, DevWaterUse wu) {
  constexpr bool WT = (X & 1) != 0;
  constexpr bool WU = (X & 2) != 0;
  constexpr bool GL = (X & 4) != 0;   // water use with GLWD units (aggrNUsGloLakResOpt = 1)
  constexpr bool VO = (X & 8) != 0;   // the vertical balance's output grids
  constexpr bool RO = (X & 16) != 0;  // routing's further output grids (always with VO)
  const int n = c.n;
  const int M = ENS ? mem.members : 1;
  const size_t N = (size_t)n * M;
  if (VAW && (int)(threadIdx.x >> 5) >= (int)(blockDim.x >> 5) - vw.warps) {
    // the block's last vw.warps warps: vertical balance ahead for the next launch's
    // steps, 32 slots at a time from a shared counter, filling the FP64 pipe while
    // the routing warps wait on loads and step barriers
    const unsigned lane = threadIdx.x & 31;
    for (;;) {
      unsigned g = 0;
      if (lane == 0) g = atomicAdd(vw.next, 1u);
      g = __shfl_sync(0xffffffffu, g, 0);
      if (g >= (unsigned)vw.nitems) break;
      const size_t i = (size_t)g * 32 + lane;
      if (i < N) va_cell<R, ENS>(c, st, f, mem, b, ring, doy0, fday0, ndays, vw.t_b, vw.t_e, i, N, VO ? &mon : nullptr,
                                 oday0);
    }
    return;
  }
  const int route_threads = VAW ? (int)blockDim.x - 32 * vw.warps : (int)blockDim.x;

  const int kd = FUSED ? ring.days_per_step : 1;   // days per step (the per-day routing call: one)
  // thread -> first state index and stride: plain (i mod the grid), or the
  // single-member layout with one idle warp per block (cell_warps warps of cells)
  long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long gstride = (long long)gridDim.x * blockDim.x;
  int wpos = -1;   // this warp's position (flow mode): slots 32*wpos .. 32*wpos+31
  if (!ENS && idle_warp >= 0) {
    const int warp = threadIdx.x >> 5;
    const int weff = warp - (warp > idle_warp ? 1 : 0);
    gtid = warp == idle_warp ? (long long)N : ((long long)blockIdx.x * cell_warps + weff) * 32 + (threadIdx.x & 31);
    gstride = (long long)gridDim.x * cell_warps * 32;
    if (warp != idle_warp) wpos = blockIdx.x * cell_warps + weff;
  }
  // flow mode: every cell warp owns exactly its 32 slots (one cell per thread)
  const bool flow = !ENS && !VAW && !GL && sync.flow && idle_warp >= 0 && gstride >= (long long)N;
  if (flow && (wpos < 0 || wpos >= sync.nwarps)) return;   // no cells: nothing to wait for or publish
  // A cell's routing state and land fractions are read and written each day
  // (mostly L2 hits: the state of the grid is a few MB).  Holding them in
  // registers for the whole launch instead took ~32 registers per thread, which
  // the wavefront launch with vertical-balance warps (96 registers per thread)
  // paid in spills, and measured ~1 % slower on the global grid.
  for (int t = t_b; t < t_e; ++t) {
    if (flow && t > t_b) {
      if (!wait_deps(sync, wpos, t - t_b - 1)) return;
      __syncwarp();   // the lanes that acquired the flags order the others' loads
    }
    if (kd * (t - c.nlevel + 1) < ndays) {   // some cell still has a day to compute
      double *q_now0 = outq + (size_t)(t & 1) * kd * N;
      const double *q_prev0 = outq + (size_t)((t + 1) & 1) * kd * N;
      double *t_now0 = WT ? wtp.outt + (size_t)(t & 1) * kd * N : nullptr;   // river temperature, same slots
      const double *t_prev0 = WT ? wtp.outt + (size_t)((t + 1) & 1) * kd * N : nullptr;
      // state index i always belongs to thread i mod gstride, so a cell's state is read
      // and written by one thread; only upstream outflows cross threads (read via L2)
      for (long long i = gtid; i < (long long)N; i += gstride) {
        const int s0 = ENS ? (int)(i / M) : (int)i;
        const int mm = ENS ? (int)(i - (long long)s0 * M) : 0;
        const int dbase = kd * (t - c.offset[s0]);
        if (dbase < 0 || dbase >= ndays) continue;   // this cell's wavefront has not reached it yet / is done
        // a GLWD unit whose riparian cells' use its outflow cell meets (GL) is routed
        // by the thread of its first cell in routing order, cell by cell in that
        // order each day (its cells share one wavefront offset): a riparian cell
        // after the outflow cell sees the unmet share of the same day, one before
        // it that of the day before, as in the reference's sweep
        int unit = -1, m_b = 0, m_e = 1;
        if constexpr (GL) {
          const int u = wu.unit_of[s0];
          if (u >= 0) {
            if (wu.unit_mem[wu.unit_ptr[u]] != s0) continue;   // routed by the unit's first cell
            unit = u;
            m_b = wu.unit_ptr[u];
            m_e = wu.unit_ptr[u + 1];
          }
        }
        if (unit < 0 && c.active && !c.active[s0]) continue;
        // the step's kd days of this cell, in order; the upstream cells routed the
        // same days one step earlier (their offset is one less)
        for (int kk = 0; kk < kd && dbase + kk < ndays; ++kk) {
         for (int m = m_b; m < m_e; ++m) {
          const int s = unit >= 0 ? wu.unit_mem[m] : s0;
          const size_t si = unit >= 0 ? (size_t)s : (size_t)i;
          if (unit >= 0 && c.active && !c.active[s]) continue;
          const int d = dbase + kk;
          double *q_now = q_now0 + (size_t)kk * N;
          const double *q_prev = q_prev0 + (size_t)kk * N;
          const int doy = (doy0 - 1 + d) % 365 + 1;
          const int month = month_of(doy);
          const uint32_t fl = c.flags[s];
          VOut<R> o;
          const R laf = st.laf[si];
          const R laf_prev = st.laf_prev[si];
          if (FUSED && !(fl & F_VINLINE)) {
            const size_t ri = (size_t)(d % ring.ring_days) * N + si;
            o.rs = ring.rs[ri];
            o.gwr = ring.gwr[ri];
            o.transfer = R(0); o.owp = R(0); o.owpet = R(0);
            o.land_in = R(0); o.land_evap = R(0); o.land_leak = R(0);   // accounted ahead
            if constexpr (WT) {
              o.owp = ring.owp[ri];
              o.owpet = ring.owpet[ri];
            }
          } else if (FUSED) {
            const size_t fo = (size_t)(fday0 + d) * n + s;
            R Pin = R(f.prec[fo]);
            R gam = c.gamma[s];
            if (ENS) {
              Pin *= R(mem.prec_factor[mm]);
              gam *= R(mem.gamma_factor[mm]);
            }
            const int started = st.laf_started[si];
            VSink vs;
            const bool vo = VO && vert_sink(mon, oday0 + d, si, N, vs);
            if (VO && doy == 1 && started == 1 && (fl & F_LOCLAKE) && mon.vconst) {
              // total PET's freshwater share after the first year: the local lakes'
              // share at the year's start (routing.cpp:1249-1259, 5045-5048)
              double *vk = mon.vconst + si;
              const double rf = (double)st.rf_loclake[si], ll = (double)c.ll100[s];   // G_loc_lake / 100
              const double fll = (ll > 0. && rf > 0.) ? rf * ll : 0.;              // G_fLocLake
              vk[3 * N] = vk[4 * N] + fll * 100. + vk[5 * N];
            }
            vertical_at<R>(c, st, N, s, si, doy, Pin, gam, f.temp[fo], f.swrad[fo], laf,
                           started == 1 ? laf_prev : laf, o, vo ? &vs : nullptr);   // daily.cpp:159-169
          } else {
            o.rs = v.rs[s]; o.gwr = v.gwr[s]; o.transfer = v.transfer[s]; o.owp = v.owp[s]; o.owpet = v.owpet[s];
            o.land_in = v.land_in[s]; o.land_evap = v.land_evap[s]; o.land_leak = v.land_leak[s];
          }
          // upstream inflow, summed in FP64 in the reference's push order (routing.cpp:3955-3958)
          double up = 0., e_up = 0.;
          const int u0 = c.up_ptr[s], u1 = c.up_ptr[s + 1];
          for (int k = u0; k < u1; ++k) {
            const size_t ui = (size_t)c.up_idx[k] * M + mm;
            // an upstream cell of the same unit was routed this step, earlier in this loop
            const double qu = (GL && unit >= 0 && wu.unit_of[c.up_idx[k]] == unit) ? q_now[ui] : __ldcg(q_prev + ui);
            up += qu;
            if constexpr (WT)   // the energy the inflow carries (calcWaterTemp.cpp:76-83)
              e_up += qu * WT_RC * (__ldcg(t_prev0 + (size_t)kk * N + ui) + WT_CONV_K);
          }
          RState<R> rs = load_rstate(st, si, fl);
          RTerms<R> rt;
          // the water temperature (routing.cpp:4241-4513) body by body inside
          // routing_cell, the river after it
          wt::WtDay wtd;
          if constexpr (WT) {
            const size_t fo = (size_t)(fday0 + d) * n + s;
            const float g = wtp.gwt[s];
            wtd.begin(&wtp, s, si, N, fl, (double)f.temp[fo], (double)f.swrad[fo], (double)wtp.lw[fo], (double)o.owp,
                      (double)c.area[s], g < 0.f ? 0. : (double)g, up, e_up);
            if (mon.wtemp) {   // the monthly mean temperatures of the day's month
              const int yd = mon.doy_day0 - 1 + oday0 + d;
              const int mi = (yd / 365) * 12 + month_of(yd % 365 + 1) - mon.month0;
              if (mi >= 0 && mi < mon.nmonths) {
                wtd.msum = mon.wtemp + (size_t)mi * N + si;
                wtd.ms = (size_t)mon.nmonths * N;
              }
            }
          }
          const size_t wrow = WU ? (size_t)wu.row_of_fday[fday0 + d] * WU_FIELDS * (size_t)n : 0;
          R tv;
          [[maybe_unused]] RoutOut ro;   // the output grids' routing terms (RO)
          const bool nocont = (fl & F_NOCONT) != 0;
          if (nocont) {
            // the reference routes only continental cells (routing.cpp:1878-4518): the
            // storages stay, nothing flows on, and the inflow stays behind in
            // G_riverInflow, i.e. leaves the system (a negative leak: the leak
            // counts water the model adds)
            tv = R(0);
            rt.p_ow = R(0); rt.e_ow = R(0); rt.leak = R(-up); rt.velocity = R(0);
          } else {
            tv = routing_cell<R, WT, WU, GL, RO>(c, s, rs, doy, month, laf, laf_prev, o, up, rt, &wtd, &wu, wrow, si,
                                                 N, &ro);
            store_rstate(st, si, rs, fl);
          }
          q_now[si] = (double)tv;
          if constexpr (WT) {
            // a cell without continental area keeps the reference's initial 15 degrees (routing.cpp:174)
            const double tr = nocont ? 15. : wtd.river((double)rs.river, (double)c.bw[s], (double)c.rlen[s],
                                                       (double)c.cfa[s], (double)o.owpet);
            t_now0[(size_t)kk * N + si] = tr;
            const int stw = c.station[s];
            if (stw >= 0) wtp.qst_t[(size_t)(oday0 + d) * c.nstation + stw] = tr;
          }
          if (b.enabled) {
            const double land_f = (double)c.area_f[s] * (double)laf;
            if (!FUSED || (fl & F_VINLINE))
              record_balance(b, N, si, (double)o.land_in * land_f + (double)rt.p_ow,
                             (double)o.land_evap * land_f + (double)rt.e_ow, up, (double)tv,
                             (double)o.land_leak * land_f + (double)rt.leak);
            else {   // vertical ran ahead: its land terms are in arrays 0, 1 and 10
              record_routing_balance(b, N, si, up, (double)tv, (double)rt.leak);
              if constexpr (WU) neumaier_add(b.acc, 12 * N + si, 13 * N + si, (double)rt.e_ow);
            }
          }
          // land-area fraction for the next day (routing.cpp:5034-5188, 5343-5352)
          if (fl & (F_LOCLAKE | F_LOCWETL | F_GLOWETL)) {
            R fswb = st.fswb_next[si];
            st.laf[si] = fraction_next<R>(fl, rs, c.ll100[s], c.lw100[s], c.gw100[s], laf, fswb);
            st.fswb_next[si] = fswb;
          }
          st.laf_prev[si] = laf;
          st.laf_started[si] = 1;
          const int stn = c.station[s];
          if (stn >= 0) qst[((size_t)(oday0 + d) * c.nstation + stn) * M + mm] = (double)tv;
          if (mon.daily_storage && oday0 + d < mon.daily_days) {   // the state file's daily storages
            double *ds = mon.daily_storage + (size_t)(oday0 + d) * 7 * N + si;
            ds[0] = (double)rs.loclake;
            ds[N] = (double)rs.locwetl;
            ds[2 * N] = (double)rs.glolake;
            ds[3 * N] = (double)rs.glowetl;
            ds[4 * N] = (double)rs.res;
            ds[5 * N] = (double)rs.river;
            ds[6 * N] = (double)rs.gw;
          }
          if (mon.enabled) {
            // monthly epilogue: this thread owns the cell, so no atomics
            const int od = oday0 + d;
            const int yd = mon.doy_day0 - 1 + od;
            const int mi = (yd / 365) * 12 + month_of(yd % 365 + 1) - mon.month0;
            if (mi >= 0 && mi < mon.nmonths) {
              const size_t k = (size_t)mi * N + si;
              const double q = (double)tv;
              // the flux grids of continental cells (routing.cpp:1878-4518), river
              // availability outside inland sinks (routing.cpp:4010-4037)
              if (!(fl & (F_SINK | F_NOCONT))) {
                mon.river_avail[k] += q;
                mon.min_avail[k] = fmin(mon.min_avail[k], q);
                mon.max_avail[k] = fmax(mon.max_avail[k], q);
              }
              mon.storage[k] += (double)rs.gw + (double)rs.river + (double)rs.loclake + (double)rs.locwetl +
                                (double)rs.glolake + (double)rs.glowetl + (double)rs.res;
              if (!(fl & F_NOCONT)) {
                // CellRunoff (routing.cpp:3933-3939): in inland sinks the transported
                // volume leaves the cell as evaporation
                mon.cell_runoff[k] += ((fl & F_SINK) ? 0. : q) - up;
                mon.velocity[k] += (double)rt.velocity / 86.4;   // km/d -> m/s
              }
            }
          }
          if constexpr (RO) {
            // routing's further output grids (routing.cpp:3964-4238, 4525-4737,
            // 5183-5186); the flux terms of continental cells only (routing.cpp:1878-4518)
            const int od = oday0 + d;
            const double q = (double)tv;
            const double cr = ((fl & F_SINK) ? 0. : q) - up;   // CellRunoff [km3]
            double owe = 0., csr = 0., crmm = 0., cp = 0.;
            if (!nocont && (mon.rext || mon.drout)) {
              const double cf = (double)c.contfreq[s], area = (double)c.area[s];
              const double rc = 1e8 * fm::rcp_pos(area * cf);   // km3 -> mm over the continental area
              // open-water evaporation, with an inland sink's transported volume (routing.cpp:4549-4560)
              owe = (ro.owe + ((fl & F_SINK) ? q : 0.)) * rc;
              csr = (cr - ro.gw_runoff) * rc;                  // routing.cpp:3998-4001
              crmm = cr * rc;
              const double *vk = mon.vconst + si;
              double lwe = cf - vk[4 * N] - vk[5 * N];          // G_landWaterExclGloLakAreaFrac (routing.cpp:1187-1196)
              if (lwe < 0.) lwe = 0.;
              const double owp = (double)(c.mprec[s] * R(f.prec[(size_t)(fday0 + d) * n + s]));
              cp = owp * lwe * area * 1e-8 + ro.p_lake;       // consistent precipitation (routing.cpp:3973-3977)
            }
            if (mon.rext) {
              const int yd = mon.doy_day0 - 1 + od;
              const int mi = (yd / 365) * 12 + month_of(yd % 365 + 1) - mon.month0;
              if (mi >= 0 && mi < mon.nmonths) {
                double *r = mon.rext + (size_t)mi * N + si;
                const size_t k = (size_t)mon.nmonths * N;
                if (!nocont) {
                  r[0] += owe;
                  r[k] += csr;
                  r[2 * k] += ro.gw_runoff;
                  r[4 * k] += ro.lw_ext;
                  r[5 * k] += ro.gw_ext;
                  // the reference adds the reservoir's flows twice a day, in the cell
                  // loop and after it (routing.cpp:4049-4050, 4653-4655)
                  r[6 * k] += 2. * ro.res_in;
                  r[7 * k] += 2. * ro.res_out;
                  r[8 * k] += cp;
                }
                r[3 * k] += (double)laf;
                r[9 * k] = (double)rs.loclake + (double)rs.locwetl + (double)rs.glolake + (double)rs.glowetl +
                           (double)rs.river + (double)rs.res;
                if constexpr (WU) {
                  if (!nocont) {   // routing.cpp:3744-3747
                    r[10 * k] += ro.actual_use;
                    r[11 * k] += ro.nug;
                  }
                }
              }
            }
            if (mon.drout && !nocont && od < mon.drout_days) {
              double *r = mon.drout + (size_t)od * N + si;
              const size_t k = (size_t)mon.drout_days * N;
              r[0] = (fl & F_SINK) ? 0. : q;
              r[k] = (double)rt.velocity / 86.4;
              r[2 * k] = cr;
              r[3 * k] = crmm;
              r[4 * k] = csr;
              r[5 * k] = ro.gw_runoff;
              r[6 * k] = (double)laf;
              r[7 * k] = cp;
              r[8 * k] = owe;
            }
          }
         }   // cells of the unit
        }   // days of the step
      }
    }
    if (flow) {
      // publish step t: every lane's writes of this step (fence, one instruction for
      // the warp), then the flag (release)
      __threadfence();
      __syncwarp();
      if ((threadIdx.x & 31) == 0) st_release_int(sync.wstep + wpos, t - t_b);
    } else if (t + 1 < t_e) {
      if (!grid_barrier(sync, (unsigned)(t - t_b), route_threads)) return;
    }
  }
}

template <class R>
__global__ void k_volume(DevCellsT<R> c, DevStateT<R> st, int M, double *vol) {
  const size_t N = (size_t)c.n * M;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) vol[i] = cell_volume<R>(c, st, N, (int)(i / M), i);
}

// Block-level Neumaier reduction; partial[blockIdx.x*8 + k] sums of
//   0 storage, 1 in, 2 evap, 3 outflow at outlets and sinks, 4 leak,
//   5 largest closure residual of a cell relative to its throughput.
template <class R>
__global__ void __launch_bounds__(256) k_balance_sum(DevCellsT<R> c, DevStateT<R> st, int M, DevBalance b,
                                                     const double *vol0, double *partial) {
  __shared__ double sh[6][256];
  __shared__ double shc[5][256];
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

// Forcing as the reference's yearly files hold it (`.365.UNF0`: big-endian float,
// cell-major [cell][nd_file], climateYear.cpp:38-79, grid_io_adapters.h:91-129):
// days [d_first, d_first + nd) of the file into dst [day][slot].  32 x 32 tiles
// through shared memory: a warp reads 32 days of one cell (contiguous) and writes
// 32 slots of one day (contiguous); the byte swap is one byte permute.
__global__ void __launch_bounds__(256) k_unf_forcing(const uint32_t *__restrict__ raw, float *__restrict__ dst,
                                                     const int32_t *__restrict__ cell_of_slot, int n, int nd_file,
                                                     int d_first, int nd, unsigned swap) {
  __shared__ float tile[32][33];
  const int s0 = blockIdx.x * 32, d0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < 32; r += 8) {
    const int s = s0 + r, d = d0 + tx;
    if (s < n && d < nd) {
      const uint32_t v = raw[(size_t)cell_of_slot[s] * nd_file + d_first + d];
      tile[r][tx] = __uint_as_float(__byte_perm(v, 0u, swap));   // 0x0123: big-endian file bytes
    }
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int d = d0 + r, s = s0 + tx;
    if (s < n && d < nd) dst[(size_t)d * n + s] = tile[tx][r];
  }
}

cudaError_t launch_unf_forcing(const uint32_t *raw, float *dst, const int32_t *cell_of_slot, int n, int nd_file,
                               int d_first, int nd, cudaStream_t st, bool big_endian) {
  const dim3 grid((unsigned)((n + 31) / 32), (unsigned)((nd + 31) / 32));
  k_unf_forcing<<<grid, 256, 0, st>>>(raw, dst, cell_of_slot, n, nd_file, d_first, nd,
                                      big_endian ? 0x0123u : 0x3210u);
  return cudaGetLastError();
}

__global__ void k_fill(double *p, size_t n, double v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

cudaError_t launch_fill(double *p, size_t n, double v, cudaStream_t st) {
  k_fill<<<(unsigned)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, st>>>(p, n, v);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- launchers
// The day step's FP64 math functions on arrays (numerics tests): 0 exp, 1 log,
// 2 pow, 3 the refined reciprocal, 4 the hardware's approximate reciprocal alone.
__global__ void k_math_eval(int fn, const double *x, const double *y, double *out, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = x[i];
  double r = 0.;
  switch (fn) {
    case 0: r = fm::exp(a); break;
    case 1: r = fm::log(a); break;
    case 2: r = fm::pow(a, y[i]); break;
    case 3: r = fm::rcp_pos(a); break;
    default: asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(a)); break;
  }
  out[i] = r;
}

cudaError_t launch_math_eval(int fn, const double *x, const double *y, double *out, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_math_eval<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(fn, x, y, out, n);
  return cudaGetLastError();
}

cudaError_t upload_fastmath_tables(const double exp2_tab[64], const double logF_tab[129], const double invF_tab[129]) {
  cudaError_t e = cudaMemcpyToSymbol(fm::g_exp2_tab, exp2_tab, 64 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(fm::g_logF_tab, logF_tab, 129 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(fm::g_invF_tab, invF_tab, 129 * sizeof(double));
  return e;
}

cudaError_t launch_gather_forcing(const float *src, float *dst, const int32_t *cell_of_slot, int n, int ndays,
                                  cudaStream_t st) {
  const size_t total = (size_t)n * ndays;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((total + threads - 1) / threads, 152 * 16);
  k_gather_forcing<<<blocks, threads, 0, st>>>(src, dst, cell_of_slot, n, ndays);
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_vertical(const DevCellsT<R> &c, const DevStateT<R> &s, const DevVertT<R> &v, const DevForcing &f,
                            int doy, int fday, cudaStream_t st) {
  const int threads = 256, blocks = (c.n + threads - 1) / threads;
  k_vertical<R><<<blocks, threads, 0, st>>>(c, s, v, f, doy, fday);
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_vertical_ahead(const DevCellsT<R> &c, const DevStateT<R> &s, const DevForcing &f,
                                  const DevMembers &mem, const DevBalance &b, const DevRingT<R> &ring, int doy0,
                                  int fday0, int ndays, int t_b, int t_e, int blocks, int threads, cudaStream_t st,
                                  const DevMonthly &mon, int oday0) {
  if (mem.members > 1)
    k_vertical_ahead<R, true><<<blocks, threads, 0, st>>>(c, s, f, mem, b, ring, doy0, fday0, ndays, t_b, t_e, mon,
                                                          oday0);
  else if ((mon.vert || mon.dvert) && std::is_same<R, double>::value)
    k_vertical_ahead<R, false, true><<<blocks, threads, 0, st>>>(c, s, f, mem, b, ring, doy0, fday0, ndays, t_b, t_e,
                                                                 mon, oday0);
  else
    k_vertical_ahead<R, false><<<blocks, threads, 0, st>>>(c, s, f, mem, b, ring, doy0, fday0, ndays, t_b, t_e, mon,
                                                           oday0);
  return cudaGetLastError();
}

template <class R, int X>
static const void *pipeline_fn_x(bool fused, bool vaw) {
  return vaw ? (fused ? (const void *)k_pipeline<R, true, false, true, X> : nullptr)
             : (fused ? (const void *)k_pipeline<R, true, false, false, X>
                      : (const void *)k_pipeline<R, false, false, false, X>);
}

template <class R>
static const void *pipeline_fn(bool fused, bool ens, bool vaw, bool wt = false, bool wu = false, bool gl = false,
                               bool vo = false, bool ro = false) {
  if (gl && (ens || wt || !wu || !std::is_same<R, double>::value)) return nullptr;   // GLWD units: FP64, one member
  if (vo || ro) {   // the output grids: FP64, one member
    if (ens || !std::is_same<R, double>::value) return nullptr;
    if (wt) return (wu || ro) ? nullptr : pipeline_fn_x<R, 9>(fused, vaw);   // the vertical balance's with the water temperature
    if (gl) return pipeline_fn_x<R, 30>(fused, vaw);   // water use over GLWD units: all outputs in one variant
    if (wu) return pipeline_fn_x<R, 26>(fused, vaw);   // with water use: all outputs in one variant
    return ro ? pipeline_fn_x<R, 24>(fused, vaw) : pipeline_fn_x<R, 8>(fused, vaw);
  }
  if (ens) return wt ? nullptr
                     : (wu ? (const void *)k_pipeline<R, true, true, false, 2> : (const void *)k_pipeline<R, true, true, false, 0>);
  if constexpr (std::is_same<R, double>::value) {   // FP64 single member only
    if (gl) return pipeline_fn_x<R, 6>(fused, vaw);
    if (wt && wu) return pipeline_fn_x<R, 3>(fused, vaw);
    if (wt) return pipeline_fn_x<R, 1>(fused, vaw);
    if (wu) return pipeline_fn_x<R, 2>(fused, vaw);
    if (vaw) return (const void *)k_pipeline<R, true, false, true, 0>;
  } else {   // FP32: no vertical-balance warps, no water temperature
    if (vaw || wt) return nullptr;
    if (wu) return fused ? (const void *)k_pipeline<R, true, false, false, 2> : (const void *)k_pipeline<R, false, false, false, 2>;
  }
  return fused ? (const void *)k_pipeline<R, true, false, false, 0>
               : (const void *)k_pipeline<R, false, false, false, 0>;
}

template <class R>
int pipeline_max_blocks(bool fused, bool ens, int threads, bool vaw, bool wt, bool wu) {
  int dev = 0, nsm = 0, per = 0;
  const void *fn = pipeline_fn<R>(fused, ens, vaw, wt, wu);
  if (!fn) return 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0) != cudaSuccess) return 0;
  return per * nsm;
}

template <class R>
int vertical_ahead_max_blocks(bool ens, int threads) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const void *fn = ens ? (const void *)k_vertical_ahead<R, true> : (const void *)k_vertical_ahead<R, false>;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0) != cudaSuccess) return 0;
  return per * nsm;
}

template <class R>
cudaError_t launch_pipeline(bool fused, const DevCellsT<R> &c, const DevStateT<R> &s, const DevVertT<R> &v,
                            const DevForcing &f, const DevMembers &mem, const DevBalance &b, const DevRingT<R> &ring,
                            const DevSync &sync, double *outq, double *qst, int doy0, int fday0, int oday0, int ndays,
                            int t_b, int t_e, int blocks, int threads, const WarpLayout &lay, const DevMonthly &mon,
                            const DevVaWork &vw, const DevWaterTemp &wtp, const DevWaterUse &wu, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(sync.counter, 0, sizeof(unsigned), st);
  if (e == cudaSuccess && sync.flow && sync.wstep)
    e = cudaMemsetAsync(sync.wstep, 0xff, (size_t)sync.nwarps * sizeof(int), st);   // -1: no step done yet
  const bool vaw = fused && vw.warps > 0;
  if (e == cudaSuccess && vaw) e = cudaMemsetAsync(vw.next, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  int cell_warps = lay.cell_warps, idle_warp = mem.members > 1 ? -1 : lay.idle_warp;
  if (idle_warp >= 0 && (threads != lay.threads || (long long)blocks * cell_warps * 32 < (long long)c.n))
    idle_warp = -1;   // the layout does not describe this launch: plain mapping
  // vertical-balance warps only on the single-member layout they were sized for
  if (vaw && (idle_warp < 0 || mem.members > 1 || vw.warps != lay.va_warps)) return cudaErrorInvalidConfiguration;
  DevVaWork vwk = vw;
  if (!vaw) vwk.warps = 0;
  void *args[] = {(void *)&c,    (void *)&s,    (void *)&v,     (void *)&f,     (void *)&mem,   (void *)&b,
                  (void *)&ring, (void *)&sync, (void *)&outq,  (void *)&qst,   (void *)&doy0,  (void *)&fday0,
                  (void *)&oday0, (void *)&ndays, (void *)&t_b, (void *)&t_e, (void *)&cell_warps,
                  (void *)&idle_warp, (void *)&mon, (void *)&vwk, (void *)&wtp, (void *)&wu};
  const bool ens = mem.members > 1;
  const void *fn = pipeline_fn<R>(fused, ens, vaw, wtp.enabled != 0, wu.enabled != 0, wu.enabled && wu.glwd,
                                  mon.vert != nullptr || mon.dvert != nullptr,
                                  mon.rext != nullptr || mon.drout != nullptr);
  if (!fn) return cudaErrorInvalidConfiguration;
  if (vaw) threads += 32 * vw.warps;
  // cooperative (all blocks resident, or the launch fails) through the launch
  // attribute, which stream capture records into a graph kernel node
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, fn, args);
}

template <class R>
cudaError_t launch_volume(const DevCellsT<R> &c, const DevStateT<R> &s, int M, double *vol, cudaStream_t st) {
  const size_t N = (size_t)c.n * M;
  const int threads = 256, blocks = (int)((N + threads - 1) / threads);
  k_volume<R><<<blocks, threads, 0, st>>>(c, s, M, vol);
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_balance_sum(const DevCellsT<R> &c, const DevStateT<R> &s, int M, const DevBalance &b,
                               const double *vol0, double *partial, int *nblocks, cudaStream_t st) {
  const size_t N = (size_t)c.n * M;
  const int threads = 256, blocks = (int)((N + threads - 1) / threads);
  *nblocks = blocks;
  k_balance_sum<R><<<blocks, threads, 0, st>>>(c, s, M, b, vol0, partial);
  return cudaGetLastError();
}

#define WG_INSTANTIATE(R)                                                                                          \
  template cudaError_t launch_vertical<R>(const DevCellsT<R> &, const DevStateT<R> &, const DevVertT<R> &,        \
                                          const DevForcing &, int, int, cudaStream_t);                             \
  template int pipeline_max_blocks<R>(bool, bool, int, bool, bool, bool);                                        \
  template int vertical_ahead_max_blocks<R>(bool, int);                                                           \
  template cudaError_t launch_pipeline<R>(bool, const DevCellsT<R> &, const DevStateT<R> &, const DevVertT<R> &,  \
                                          const DevForcing &, const DevMembers &, const DevBalance &,             \
                                          const DevRingT<R> &, const DevSync &, double *, double *, int, int,     \
                                          int, int, int, int, int, int, const WarpLayout &, const DevMonthly &,    \
                                          const DevVaWork &, const DevWaterTemp &, const DevWaterUse &,           \
                                          cudaStream_t);                                                          \
  template cudaError_t launch_vertical_ahead<R>(const DevCellsT<R> &, const DevStateT<R> &, const DevForcing &,   \
                                                const DevMembers &, const DevBalance &, const DevRingT<R> &, int,  \
                                                int, int, int, int, int, int, cudaStream_t, const DevMonthly &,   \
                                                int);                                                              \
  template cudaError_t launch_volume<R>(const DevCellsT<R> &, const DevStateT<R> &, int, double *, cudaStream_t); \
  template cudaError_t launch_balance_sum<R>(const DevCellsT<R> &, const DevStateT<R> &, int, const DevBalance &,  \
                                             const double *, double *, int *, cudaStream_t);
WG_INSTANTIATE(double)
WG_INSTANTIATE(float)

}  // namespace wg
