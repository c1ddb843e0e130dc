// wg_ctx.h -- the library's context (struct wg_ctx of include/wg_gpu.h) and the
// host-side topology; shared by the C ABI (wg_capi.cpp) and the run-time tools
// (wg_tune.cpp: snapshot, autotuner, CUDA graphs).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/wg_gpu.h"
#include "wg_device.h"
#include "wg_kernels.h"

using wg::DevBalance;
using wg::DevCellsT;
using wg::DevForcing;
using wg::DevMembers;
using wg::DevMonthly;
using wg::DevWaterTemp;
using wg::DevWaterUse;
using wg::DevRingT;
using wg::DevStateT;
using wg::DevSync;
using wg::DevVertT;
using wg::WarpLayout;

// Drainage topology and slot order of one region (built once by wg_create).
struct Topology {
  std::vector<int32_t> rout_pos;      // position of each cell in the reference routing order
  std::vector<int32_t> offset;        // per cell: pipeline step offset
  std::vector<int32_t> cell_of_slot;  // slot -> cell
  std::vector<int32_t> slot_of_cell;  // cell -> slot
  std::vector<int32_t> up_ptr, up_idx;// slot space
  int32_t nlevel = 0;
};

// The mutable per-state arrays of DevStateT (besides snow_band).
#define WG_STATE_R(X)                                                                                               \
  X(canopy) X(soil) X(snow) X(lai_precsum) X(gw) X(river) X(loclake) X(locwetl) X(glolake) X(glowetl) X(res)      \
  X(rf_loclake) X(rf_locwetl) X(rf_glolake) X(rf_glowetl) X(rf_res) X(k_release) X(laf) X(laf_prev) X(fswb_next)
#define WG_STATE_I(X) X(lai_days) X(lai_status) X(laf_started)

struct Snapshot;   // wg_tune.cpp

// One context: all device buffers of one region in one precision.
struct wg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t copy_stream = nullptr;      // wg_upload_forcing_async
  cudaEvent_t upload_done = nullptr;
  bool upload_pending = false;
  int n = 0, nband = 0, max_days = 0, nstation = 0, members = 1, precision = 0;
  int threads = 256, blocks_fused = 0, blocks_route = 0;
  WarpLayout layout;                       // single-member wavefront layout (idle_warp < 0: none)
  Topology topo;
  DevCellsT<double> cd{};
  DevStateT<double> sd{};
  DevVertT<double> vd{};
  DevCellsT<float> cf{};
  DevStateT<float> sf{};
  DevVertT<float> vf{};
  DevRingT<double> rd{};
  DevRingT<float> rf{};
  DevForcing forcing{};
  DevBalance balance{};
  DevMembers mem{};
  DevSync sync{};
  DevMonthly mon{};                        // wg_monthly_outputs
  double *mon_buf = nullptr;
  double *mon_vbuf = nullptr;              // the vertical balance's monthly grids (wg_monthly_outputs_vertical)
  bool mon_vert_on = false;
  double *mon_dbuf = nullptr;              // its daily grids (wg_daily_outputs_vertical)
  double *mon_rbuf = nullptr;              // routing's further monthly grids (wg_monthly_outputs_routing)
  double *mon_tbuf = nullptr;              // the monthly mean water temperatures (with the water temperature)
  bool mon_rout_on = false;
  double *mon_drbuf = nullptr;             // routing's daily grids (wg_daily_outputs_routing)
  double *mon_vconst = nullptr;            // their constants (DevMonthly::vconst)
  // [7][n] cell order, from wg_create: the grids' constants (DevMonthly::vconst,
  // the first year's freshwater share) and G_loc_lake / 100
  std::vector<double> vstatic;
  bool has_kc = false;                     // the region gave the LCT crop coefficients
  std::vector<double> cell_area, cell_cont;   // cell order: area [km2], continental share [%] as raised
  double *daily_storage_buf = nullptr;     // wg_record_daily_storages (context allocation)
  double *outq = nullptr, *qst = nullptr, *vol0 = nullptr, *partial = nullptr;
  float *staging = nullptr;
  float *staging_async = nullptr;          // staging of wg_upload_forcing_async
  uint32_t *unf_raw[2] = {nullptr, nullptr};   // raw file bytes (context stream, copy stream)
  size_t unf_cap[2] = {0, 0};
  int32_t *d_cell_of_slot = nullptr;
  uint8_t *d_active = nullptr;             // wg_set_active_cells (slot order)
  int staging_days = 0;
  int64_t launches = 0;
  std::vector<void *> allocs;
  std::string err;
  int chunk_steps = 0;                     // steps per (vertical-ahead, wavefront) launch pair
  int days_per_step = 1;                   // days every cell advances per wavefront step
  int frac_routing = 0;                    // options.fractionalRoutingOpt
  DevWaterTemp wt{};                       // water temperature (wt.enabled = 0: off)
  DevWaterUse wu{};                        // water use (wu.enabled = 0: off)
  int wu_blocks = 0, wu_next = 0;          // 12-row table blocks (block 0: no use), next to fill
  std::vector<double> wu_prov0;            // [n] slot order: provisional release without use
  struct WuRes { int slot, cell, type; double mean_outflow, mean_demand; };
  std::vector<WuRes> wu_res;               // the reservoirs, for the monthly provisional release
  // GLWD units (aggrNUsGloLakResOpt = 1): per cell its unit (G_glwdUnit) and
  // whether it is a global lake's or reservoir's outflow cell; per cell the index
  // of its unit among the units with an outflow cell (-1 no unit, -2 a unit
  // without one), and the cells of each such unit in cell order
  struct Glwd {
    bool on = false;
    std::vector<int32_t> unit, unit_of, ptr, cells;
    std::vector<uint8_t> outflow;
  } glwd;
  int last_vertical_fday = 0;              // forcing slot of the last wg_step_vertical
  struct Deferred {                        // wg_set_deferred: the per-day calls queued
    bool on = false;
    int doy0 = 0, fday0 = 0, oday0 = 0, ndays = 0;   // consecutive days with both calls made
    bool vpending = false;                 // a vertical call waiting for its routing call
    int vdoy = 0, vfday = 0;
  } defer;
  int va_warps_default = 0;                // vertical-balance warps the layout was sized for
  unsigned int *va_next = nullptr;         // their work counter
  Snapshot *snap = nullptr;                // device copy of the mutable state (autotuner)
  cudaGraph_t graph = nullptr;             // wg_graph_capture
  cudaGraphExec_t graph_exec = nullptr;
  int graph_launches = 0;                  // kernels in the captured graph
  // ensembles (FP32, members > 1): the next chunk's vertical balance runs on a
  // second stream while this chunk's wavefront launch runs (ens_overlap), the
  // wavefront launch leaving room on the SMs for its blocks; the ring then holds
  // two chunks' days.  The fork event starts the second stream after the
  // context's stream, the others order the launches (wg_capi.cpp run_steps_impl)
  bool ens_overlap = false;
  cudaStream_t va_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_va = nullptr, ev_pipe[2] = {nullptr, nullptr};
  int blocks_va = 0;                       // grid of the vertical-ahead launches on va_stream
  bool timing = false;                     // CUDA events around each launch pair of wg_run_steps
  std::vector<cudaEvent_t> tev;            // 3 per recorded launch pair
  size_t tev_used = 0;
  cudaEvent_t *timing_events() {           // the next three events of the pool
    if (tev_used + 3 > tev.size())
      for (int k = 0; k < 3; ++k) {
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        tev.push_back(e);
      }
    cudaEvent_t *p = tev.data() + tev_used;
    tev_used += 3;
    return p;
  }

  ~wg_ctx() {
    release_tools();
    if (mon_buf) cudaFree(mon_buf);
    if (mon_vbuf) cudaFree(mon_vbuf);
    if (mon_dbuf) cudaFree(mon_dbuf);
    if (mon_rbuf) cudaFree(mon_rbuf);
    if (mon_tbuf) cudaFree(mon_tbuf);
    if (mon_drbuf) cudaFree(mon_drbuf);
    if (mon_vconst) cudaFree(mon_vconst);
    for (void *p : allocs) cudaFree(p);
    if (own_stream && stream) cudaStreamDestroy(stream);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    if (upload_done) cudaEventDestroy(upload_done);
    if (va_stream) cudaStreamDestroy(va_stream);
    for (cudaEvent_t e : {ev_fork, ev_va, ev_pipe[0], ev_pipe[1]})
      if (e) cudaEventDestroy(e);
  }
  template <class T>
  T *alloc(size_t count) {
    void *p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return (T *)p;
  }
  size_t nstate() const { return (size_t)n * members; }
  int ring_days() const { return precision == 0 ? rd.ring_days : rf.ring_days; }
  // longest chunk of wavefront steps one launch pair may run: its days fit the ring
  int max_chunk() const { return ring_days() / days_per_step; }
  // the wavefront launches carry vertical-balance warps for the next chunk
  bool overlap() const { return layout.va_warps > 0 && layout.idle_warp >= 0 && threads == layout.threads; }
  // longest chunk: with the overlap the ring holds this chunk's and the next one's days
  int chunk_cap() const { return (overlap() || ens_overlap) ? max_chunk() / 2 : max_chunk(); }
  // steps per launch: the set chunk length if it fits, else about 16 days with
  // the overlap (the first chunk of each call runs its vertical balance alone)
  // or the ring
  int eff_chunk() const {
    if (chunk_steps > 0 && chunk_steps <= chunk_cap()) return chunk_steps;
    return overlap() ? std::min((16 + days_per_step - 1) / days_per_step, chunk_cap()) : chunk_cap();
    // (with ens_overlap the longest chunk that fits the ring: the launches of a
    // chunk pair run side by side, so fewer, longer chunks lose less at their ends)
  }
  // wavefront steps of a run of ndays days
  int total_steps(int ndays) const { return (ndays + days_per_step - 1) / days_per_step + topo.nlevel - 1; }
  void release_tools();   // snapshot and graph (wg_tune.cpp)
};

// Runs the per-day calls that wg_set_deferred has queued (wg_capi.cpp); every
// entry point that reads or changes the model, its inputs or its run shape
// calls it first.
wg_status flush_deferred(wg_ctx *ctx);
#define WG_FLUSH(ctx)                                    \
  do {                                                   \
    if ((ctx)->defer.on) {                               \
      const wg_status wg_flush_st_ = flush_deferred(ctx); \
      if (wg_flush_st_ != WG_OK) return wg_flush_st_;    \
    }                                                    \
  } while (0)
