// wg_tune.cpp -- run-time tools of a context: a device snapshot of the mutable
// state, the launch-shape autotuner, and CUDA-graph capture of a run.
//
// The reference has no counterpart (its day loop is OpenMP over cells); these
// exist for the batched paths: an ensemble of hundreds of members in one
// persistent wavefront, whose best block size (members of one cell per block)
// and chunk length (wavefront steps per vertical-ahead/wavefront launch pair)
// depend on the member count and the device, is tuned once and then replayed
// as one graph launch per run.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "wg_ctx.h"
#include "wg_kernels.h"

using namespace wg;

// Device copy of everything a run mutates: the state arrays, the snow bands,
// the two-slot outflow buffer of the wavefront and the balance accumulators.
// (The ring of vertical outputs holds nothing between calls: each chunk's
// vertical-ahead launch fills exactly the days its wavefront launch reads.)
struct Snapshot {
  std::vector<std::pair<void *, size_t>> fields;   // (device array, bytes)
  char *buf = nullptr;
  size_t bytes = 0;
};

namespace {

wg_status fail(wg_ctx *ctx, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return WG_OK;
  ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? WG_ERR_NOMEM : WG_ERR_CUDA;
}

template <class R>
void list_fields(wg_ctx *ctx, const DevStateT<R> &s, Snapshot &sn) {
  const size_t N = ctx->nstate();
#define X(f) sn.fields.push_back({(void *)s.f, N * sizeof(R)});
  WG_STATE_R(X)
#undef X
#define X(f) sn.fields.push_back({(void *)s.f, N * sizeof(int32_t)});
  WG_STATE_I(X)
#undef X
  sn.fields.push_back({(void *)s.snow_band, N * ctx->nband * sizeof(R)});
  sn.fields.push_back({(void *)ctx->outq, 2 * (size_t)ctx->days_per_step * N * sizeof(double)});
  if (ctx->balance.enabled) sn.fields.push_back({(void *)ctx->balance.acc, WG_BALANCE_ARRAYS * N * sizeof(double)});
  if (ctx->wu.enabled) sn.fields.push_back({(void *)ctx->wu.st, (size_t)wg::WU_NSTATE * N * sizeof(double)});
  if (ctx->wt.enabled) {
    sn.fields.push_back({(void *)ctx->wt.temp, 6 * N * sizeof(double)});
    sn.fields.push_back({(void *)ctx->wt.ice, 6 * N * sizeof(double)});
    sn.fields.push_back({(void *)ctx->wt.outt, 2 * (size_t)ctx->days_per_step * N * sizeof(double)});
  }
}

wg_status snapshot_save(wg_ctx *ctx) {
  if (!ctx->snap) {
    Snapshot *sn = new Snapshot();
    if (ctx->precision == 0) list_fields(ctx, ctx->sd, *sn);
    else list_fields(ctx, ctx->sf, *sn);
    for (auto &f : sn->fields) sn->bytes += (f.second + 255) / 256 * 256;
    cudaError_t e = cudaMalloc((void **)&sn->buf, sn->bytes);
    if (e != cudaSuccess) {
      delete sn;
      return fail(ctx, e, "snapshot");
    }
    ctx->snap = sn;
  }
  size_t off = 0;
  for (auto &f : ctx->snap->fields) {
    cudaError_t e = cudaMemcpyAsync(ctx->snap->buf + off, f.first, f.second, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return fail(ctx, e, "snapshot");
    off += (f.second + 255) / 256 * 256;
  }
  return WG_OK;
}

wg_status snapshot_restore(wg_ctx *ctx) {
  if (!ctx->snap) return WG_ERR_INVALID;
  size_t off = 0;
  for (auto &f : ctx->snap->fields) {
    cudaError_t e = cudaMemcpyAsync(f.first, ctx->snap->buf + off, f.second, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return fail(ctx, e, "restore");
    off += (f.second + 255) / 256 * 256;
  }
  return WG_OK;
}

}  // namespace

void wg_ctx::release_tools() {
  for (cudaEvent_t e : tev) cudaEventDestroy(e);
  tev.clear();
  tev_used = 0;
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
  graph_exec = nullptr;
  graph = nullptr;
  if (snap) {
    cudaFree(snap->buf);
    delete snap;
    snap = nullptr;
  }
}

extern "C" {

wg_status wg_save_snapshot(wg_ctx *ctx) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  cudaSetDevice(ctx->device);
  wg_status st = snapshot_save(ctx);
  return st != WG_OK ? st : wg_synchronize(ctx);
}

wg_status wg_restore_snapshot(wg_ctx *ctx) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  cudaSetDevice(ctx->device);
  wg_status st = snapshot_restore(ctx);
  return st != WG_OK ? st : wg_synchronize(ctx);
}

wg_status wg_kernel_timing(wg_ctx *ctx, int32_t enable) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  ctx->timing = enable != 0;
  ctx->tev_used = 0;
  return WG_OK;
}

wg_status wg_get_kernel_times(wg_ctx *ctx, double *vertical_ahead_ms, double *wavefront_ms, int32_t *launch_pairs) {
  if (!ctx || !vertical_ahead_ms || !wavefront_ms || !launch_pairs) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  double va = 0., wf = 0.;
  for (size_t k = 0; k + 3 <= ctx->tev_used; k += 3) {
    float a = 0.f, b = 0.f;
    if (cudaEventElapsedTime(&a, ctx->tev[k], ctx->tev[k + 1]) != cudaSuccess ||
        cudaEventElapsedTime(&b, ctx->tev[k + 1], ctx->tev[k + 2]) != cudaSuccess)
      return fail(ctx, cudaGetLastError(), "kernel times");
    va += a;
    wf += b;
  }
  *vertical_ahead_ms = va;
  *wavefront_ms = wf;
  *launch_pairs = (int32_t)(ctx->tev_used / 3);
  ctx->tev_used = 0;
  return WG_OK;
}

wg_status wg_set_chunk_steps(wg_ctx *ctx, int32_t steps) {
  if (!ctx || steps < 0 || steps > ctx->chunk_cap()) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  ctx->chunk_steps = steps;
  return WG_OK;
}

wg_status wg_set_vertical_overlap(wg_ctx *ctx, int32_t enable) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (ctx->members > 1) {   // ensembles: the next chunk's vertical balance on the second stream
    if (!ctx->va_stream) return WG_ERR_UNSUPPORTED;
    ctx->ens_overlap = enable != 0;
    return WG_OK;
  }
  if (!enable) {
    ctx->layout.va_warps = 0;
    return WG_OK;
  }
  if (ctx->va_warps_default <= 0 || ctx->layout.idle_warp < 0 || ctx->threads != ctx->layout.threads)
    return WG_ERR_UNSUPPORTED;
  ctx->layout.va_warps = ctx->va_warps_default;
  return WG_OK;
}

int32_t wg_get_vertical_overlap(const wg_ctx *ctx) {
  if (ctx && ctx->members > 1) return ctx->ens_overlap ? 1 : 0;
  return ctx && ctx->overlap() ? ctx->layout.va_warps : 0;
}

int32_t wg_get_chunk_steps(const wg_ctx *ctx) {
  if (!ctx) return 0;
  return ctx->eff_chunk();
}

wg_status wg_autotune(wg_ctx *ctx, int32_t doy0, int32_t fday0, int32_t ndays, int32_t t_begin,
                      int32_t trial_steps, wg_tune_result *out) {
  if (!ctx || !out || trial_steps <= 0) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  const int total = ctx->total_steps(ndays);
  if (t_begin < 0 || t_begin + trial_steps > total) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  const int th0 = ctx->threads, ch0 = ctx->chunk_steps;
  const int bf0 = ctx->blocks_fused, br0 = ctx->blocks_route, bv0 = ctx->blocks_va;
  const bool eo0 = ctx->ens_overlap;
  const WarpLayout lay0 = ctx->layout;
  int32_t tmp = 0;
  wg_status st = snapshot_save(ctx);
  if (st != WG_OK) return st;
  // the trials must not add to the monthly sums (their days run again after the
  // state is restored); the day's grids they write are written again the same
  const DevMonthly mon0 = ctx->mon;
  ctx->mon.enabled = 0;
  ctx->mon.vert = nullptr;
  ctx->mon.rext = nullptr;
  ctx->mon.wtemp = nullptr;
  // candidates: block sizes 64..512 (for ensembles: members of one cell per block,
  // or whole cells per block when a cell has fewer members), chunk lengths 8..ring
  std::vector<int> ths = {64, 128, 256, 512};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 1e300;
  int best_th = -1, best_ch = ch0, trials = 0;   // best_th < 0: the shape the context had
  auto restore_shape0 = [&]() {
    ctx->threads = th0;
    ctx->blocks_fused = bf0;
    ctx->blocks_route = br0;
    ctx->blocks_va = bv0;
    ctx->layout = lay0;
  };
  // ensembles: without and with the stream overlap, the wavefront launch on all
  // its blocks or on 3/4 or 1/2 of them (leaving the SMs room for the vertical
  // balance beside it)
  struct Ov { bool on; int num; };
  std::vector<Ov> ovs = {{false, 4}};
  if (ctx->members > 1 && ctx->va_stream) ovs = {{false, 4}, {true, 4}, {true, 3}, {true, 2}};
  bool best_eo = eo0;
  int best_blocks = bf0;
  // first the context's own shape and layout; with vertical-balance warps, also
  // the same layout without them
  ths.insert(ths.begin(), -1);
  if (lay0.va_warps > 0) ths.insert(ths.begin() + 1, -2);
  int best_va = lay0.va_warps;
  for (int th : ths) {
    if (th < 0) {
      restore_shape0();
      if (th == -2) ctx->layout.va_warps = 0;
    } else if (wg_launch_shape(ctx, th, 0) != WG_OK) {
      continue;   // does not fit the device
    }
    const int full_blocks = ctx->blocks_fused;
    for (const Ov &ov : ovs) {
      ctx->ens_overlap = ov.on;
      ctx->blocks_fused = std::max(1, full_blocks * ov.num / 4);
      std::vector<int> chs;   // chunk lengths 8 .. the longest this shape allows
      for (int c = 8; c <= ctx->chunk_cap(); c *= 2) chs.push_back(c);
      if (chs.empty() || chs.back() != ctx->chunk_cap()) chs.push_back(ctx->chunk_cap());
      for (int ch : chs) {
        if (ch > trial_steps && ch != chs.front()) continue;   // a chunk longer than the trial says nothing
        ctx->chunk_steps = ch;
        st = snapshot_restore(ctx);
        if (st != WG_OK) break;
        cudaEventRecord(e0, ctx->stream);
        st = wg_run_steps(ctx, doy0, fday0, ndays, t_begin, t_begin + trial_steps);
        cudaEventRecord(e1, ctx->stream);
        if (st != WG_OK) break;
        st = wg_synchronize(ctx);
        if (st != WG_OK) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ++trials;
        if (ms < best) {
          best = ms;
          best_th = th;
          best_ch = ch;
          best_va = ctx->layout.va_warps;
          best_eo = ov.on;
          best_blocks = ctx->blocks_fused;
        }
      }
      if (st != WG_OK) break;
    }
    ctx->blocks_fused = full_blocks;
    if (st != WG_OK) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->mon = mon0;
  wg_status st2 = snapshot_restore(ctx);
  if (st == WG_OK) st = st2;
  if (st == WG_OK) st = wg_synchronize(ctx);
  if (st != WG_OK || trials == 0) {
    restore_shape0();
    ctx->ens_overlap = eo0;
    ctx->chunk_steps = ch0;
    return st != WG_OK ? st : WG_ERR_UNSUPPORTED;
  }
  if (best_th < 0) {
    restore_shape0();
    ctx->layout.va_warps = best_va;
  } else {
    wg_launch_shape(ctx, best_th, 0);
  }
  ctx->ens_overlap = best_eo;
  if (ctx->members > 1) ctx->blocks_fused = best_blocks;
  ctx->chunk_steps = best_ch;
  out->threads = ctx->threads;
  int32_t mb = 0;
  wg_get_launch_shape(ctx, &tmp, &out->blocks, &mb);
  out->chunk_steps = best_ch;
  out->ms_per_step = best / trial_steps;
  out->trials = trials;
  return WG_OK;
}

wg_status wg_graph_capture(wg_ctx *ctx, int32_t doy0, int32_t fday0, int32_t ndays, int32_t t_begin, int32_t t_end) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  const int total = ctx->total_steps(ndays);
  if (doy0 < 1 || doy0 > 365 || fday0 < 0 || ndays <= 0 || fday0 + ndays > ctx->max_days || t_begin < 0 ||
      t_end > total || t_begin >= t_end)
    return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  ctx->upload_pending = false;   // synchronised: nothing for the graph to wait on
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  ctx->graph_exec = nullptr;
  ctx->graph = nullptr;
  const int64_t l0 = ctx->launches;
  const bool timing = ctx->timing;
  ctx->timing = false;   // no timing events inside the graph
  cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    ctx->timing = timing;
    return fail(ctx, e, "graph capture");
  }
  st = wg_run_steps(ctx, doy0, fday0, ndays, t_begin, t_end);
  ctx->timing = timing;
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &g);
  ctx->graph_launches = (int)(ctx->launches - l0);
  ctx->launches = l0;   // captured, not run
  if (st != WG_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return fail(ctx, e, "graph capture");
  e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(ctx, e, "graph instantiate");
  }
  ctx->graph = g;
  return WG_OK;
}

wg_status wg_graph_launch(wg_ctx *ctx) {
  if (!ctx || !ctx->graph_exec) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  cudaSetDevice(ctx->device);
  ctx->launches += ctx->graph_launches;
  return fail(ctx, cudaGraphLaunch(ctx->graph_exec, ctx->stream), "graph launch");
}

}  // extern "C"
