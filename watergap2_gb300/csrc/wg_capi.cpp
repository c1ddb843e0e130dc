// wg_capi.cpp -- host side of libwg_gpu.so: the C ABI declared in include/wg_gpu.h.
//
// wg_create replaces the set-up the reference performs before its day loop:
//   routingClass::init        (source/routing.cpp:131-742)  river geometry, reservoirs
//   rout_order                (source/rout_prepare.cpp:834-886) routing order, here
//                             extended by drainage depth and the slot layout
//   initLakeDepthActive / initWetlDepthActive (routing.cpp:5621-5643)
//   setStoragesToZero / setLakeWetlToMaximum  (daily.cpp:1882-1894, routing.cpp:790-848, 5647-5716)
//   initFractionStatus / annualInit (routing.cpp:748-765, 979-1205)
// Constants the reference recomputes each day from per-cell inputs are
// evaluated here once, with the reference's expressions, in the precision of
// the context (FP64, or FP32 for the mixed-precision and ensemble paths).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/wg_gpu.h"
#include "wg_ctx.h"
#include "wg_device.h"
#include "wg_kernels.h"

using namespace wg;

namespace {

const double kPi = 3.141592653589793;   // daily.cpp:73
const short kFirstDayInMonth[12] = {1, 32, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335};

// dailyWaterBalanceClass::calc_ext_rad (daily.cpp:2398-2449) for a latitude in degrees.
double calc_ext_rad(short day, double lat_deg) {
  double declination_angle = asin(0.39795 * cos(0.2163108 + 2. * atan(0.9671396 * tan(0.00860 * (day - 186)))));
  const double pi_180 = kPi / 180.0;
  double theta = lat_deg * pi_180;
  double omega_s = (sin(theta) * sin(declination_angle)) / (cos(theta) * cos(declination_angle));
  if ((omega_s) < -1.) omega_s = -1;
  if ((omega_s) > 1.) omega_s = 1;
  omega_s = kPi - acos(omega_s);
  const double pi2_365 = 2. * kPi / 365.0;
  double dist_es = 1. + 0.033 * cos(pi2_365 * day);
  return (15.392 * dist_es * (omega_s * sin(theta) * sin(declination_angle) +
                              cos(theta) * cos(declination_angle) * sin(omega_s)));
}


// Routing order of the reference (rout_prepare.cpp:834-886): Kahn passes, each pass
// numbering the cells without pending inflow in index order.
wg_status reference_rout_order(int n, const int32_t *down, std::vector<int32_t> &order) {
  std::vector<int32_t> cnt(n, 0);
  for (int i = 0; i < n; ++i)
    if (down[i] >= 0) cnt[down[i]]++;
  order.clear();
  order.reserve(n);
  std::vector<int32_t> frontier, next;
  for (int i = 0; i < n; ++i)
    if (cnt[i] == 0) frontier.push_back(i);
  while (!frontier.empty()) {
    std::sort(frontier.begin(), frontier.end());
    next.clear();
    for (int c : frontier) order.push_back(c);
    for (int c : frontier) {
      const int d = down[c];
      if (d >= 0 && --cnt[d] == 0) next.push_back(d);
    }
    frontier.swap(next);
  }
  return (int)order.size() == n ? WG_OK : WG_ERR_TOPOLOGY;
}

// Slot order.  The day-pipelined kernel maps slot i to thread i (mod the grid),
// so a warp runs the 32 cells of 32 consecutive slots in lock step, and every cell
// is busy in every step of the steady state.  Cells are therefore grouped by work
// class (cls: cells of one class run the same branches -- above all, cells with a
// water body also run the vertical balance inside the wavefront), within a class
// by offset and then routing order (so that a warp's cells mostly compute the same
// day and read forcing and ring rows contiguously).  The warps of each class are
// then spread evenly over the slot range, so that each block -- one per SM by
// default -- holds its share of every class and no SM waits on the others at the
// step barrier.  The order of slots changes nothing in the results: each cell's
// inputs are addressed through its slot, and inflows are summed in the upstream
// lists' routing order.
// Warp placement for the single-member wavefront layout: blocks of
// cell_warps warps of cells plus one idle warp (warps_per_block in all).  Warp
// w of a block issues on SM sub-partition w % 4, and the FP64 work between two
// step barriers is the sum over a sub-partition's warps, so the one idle warp
// leaves one sub-partition per block with fewer warps; a water-body warp
// (about three times the FP64 work of a plain one) goes there, and plain warps
// fill the rest.  Greedy: each water-body warp to the sub-partition whose
// predicted load (its water-body warps plus one per remaining position) is
// lowest; plain warps keep their class-sorted order.  The partial last warp
// stays at the last position so that slots stay dense.
void place_warps(const std::vector<int32_t> &seq, const uint32_t *cls, int n, const WarpLayout &lay,
                 std::vector<int32_t> &worder) {
  const int W = (n + 31) / 32, wfull = n / 32, cw = lay.cell_warps;
  // positions p = block * cw + weff, p < W; sub-partition of each
  std::vector<int> smsp(W);
  for (int p = 0; p < W; ++p) {
    const int weff = p % cw;
    const int w = weff < lay.idle_warp ? weff : weff + 1;
    smsp[p] = w & 3;
  }
  const int nbucket = ((W + cw - 1) / cw) * 4;
  std::vector<std::vector<int>> free_pos(nbucket);
  for (int p = wfull - 1; p >= 0; --p) free_pos[(p / cw) * 4 + smsp[p]].push_back(p);   // ascending when popped
  std::vector<int> heavy_cost(nbucket, 0);
  std::vector<int> heavy, light;
  for (int w = 0; w < wfull; ++w) {
    bool h = false;
    for (int j = w * 32; j < w * 32 + 32 && !h; ++j) h = cls && cls[seq[j]] != 0u;
    (h ? heavy : light).push_back(w);
  }
  const int kHeavy = 3;
  std::vector<int> placed(wfull, -1);
  std::vector<uint8_t> used(W, 0);
  for (int w : heavy) {
    int best = -1;
    long long best_load = 0;
    for (int b = 0; b < nbucket; ++b) {
      if (free_pos[b].empty()) continue;
      const long long load = heavy_cost[b] + kHeavy + (long long)(free_pos[b].size() - 1);
      if (best < 0 || load < best_load) {
        best = b;
        best_load = load;
      }
    }
    const int p = free_pos[best].back();
    free_pos[best].pop_back();
    heavy_cost[best] += kHeavy;
    placed[w] = p;
    used[p] = 1;
  }
  size_t li = 0;
  for (int p = 0; p < wfull; ++p)
    if (!used[p]) placed[light[li++]] = p;
  for (int w = 0; w < wfull; ++w) worder[placed[w]] = w;
  if (W > wfull) worder[W - 1] = W - 1;
}

wg_status build_topology(int n, const int32_t *down, const int32_t *rout_order, const uint32_t *cls,
                         const WarpLayout *lay, Topology &t, const int32_t *node_of) {
  for (int i = 0; i < n; ++i)
    if (down[i] < -1 || down[i] >= n || down[i] == i) return WG_ERR_TOPOLOGY;
  std::vector<int32_t> order;
  if (rout_order) {
    order.assign(rout_order, rout_order + n);
  } else {
    wg_status st = reference_rout_order(n, down, order);
    if (st != WG_OK) return st;
  }
  t.rout_pos.assign(n, -1);
  for (int k = 0; k < n; ++k) {
    const int c = order[k];
    if (c < 0 || c >= n || t.rout_pos[c] >= 0) return WG_ERR_TOPOLOGY;
    t.rout_pos[c] = k;
  }
  for (int i = 0; i < n; ++i)
    if (down[i] >= 0 && t.rout_pos[down[i]] <= t.rout_pos[i]) return WG_ERR_TOPOLOGY;
  // distance to the outlet, downstream first
  std::vector<int32_t> depth(n, 0);
  int32_t dmax = 0;
  if (!node_of) {
    for (int k = n - 1; k >= 0; --k) {
      const int c = order[k];
      depth[c] = down[c] < 0 ? 0 : depth[down[c]] + 1;
      dmax = std::max(dmax, depth[c]);
    }
  } else {
    // cells that one thread routes together (node_of: the same node) share one
    // offset: the longest path to an outlet over the graph of nodes, which must
    // stay acyclic (a node's cells may not drain out of it and back in)
    std::vector<std::vector<int32_t>> succ(n);
    std::vector<int32_t> indeg(n, 0);
    for (int c = 0; c < n; ++c) {
      if (node_of[c] < 0 || node_of[c] >= n || node_of[node_of[c]] != node_of[c]) return WG_ERR_TOPOLOGY;
      if (down[c] < 0) continue;
      const int a = node_of[c], b = node_of[down[c]];
      if (a != b) {
        succ[a].push_back(b);
        indeg[b]++;
      }
    }
    std::vector<int32_t> topo_nodes, frontier;
    for (int c = 0; c < n; ++c)
      if (node_of[c] == c && indeg[c] == 0) frontier.push_back(c);
    while (!frontier.empty()) {
      const int a = frontier.back();
      frontier.pop_back();
      topo_nodes.push_back(a);
      for (int b : succ[a])
        if (--indeg[b] == 0) frontier.push_back(b);
    }
    int nodes = 0;
    for (int c = 0; c < n; ++c) nodes += node_of[c] == c;
    if ((int)topo_nodes.size() != nodes) return WG_ERR_TOPOLOGY;
    std::vector<int32_t> ndepth(n, 0);
    for (int k = (int)topo_nodes.size() - 1; k >= 0; --k) {
      const int a = topo_nodes[k];
      for (int b : succ[a]) ndepth[a] = std::max(ndepth[a], ndepth[b] + 1);
      dmax = std::max(dmax, ndepth[a]);
    }
    for (int c = 0; c < n; ++c) depth[c] = ndepth[node_of[c]];
  }
  t.nlevel = dmax + 1;
  t.offset.resize(n);
  for (int i = 0; i < n; ++i) t.offset[i] = dmax - depth[i];
  std::vector<int32_t> seq(order);
  std::stable_sort(seq.begin(), seq.end(), [&](int a, int b) {
    const uint32_t ca = cls ? cls[a] : 0u, cb = cls ? cls[b] : 0u;
    if (ca != cb) return ca < cb;
    return t.offset[a] < t.offset[b];
  });
  const int W = (n + 31) / 32;
  const int wfull = n / 32;   // a partial last warp stays last, so that every full warp stays aligned
  std::vector<uint32_t> wcls(W);
  std::map<uint32_t, int> count;
  for (int w = 0; w < W; ++w) {
    wcls[w] = cls ? cls[seq[(size_t)w * 32]] : 0u;
    if (w < wfull) count[wcls[w]]++;
  }
  std::vector<int32_t> worder(W);
  if (lay && lay->idle_warp >= 0) {
    place_warps(seq, cls, n, *lay, worder);
  } else {
    std::map<uint32_t, int> seen;
    std::vector<std::pair<double, int>> key(wfull);
    for (int w = 0; w < wfull; ++w) key[w] = {(seen[wcls[w]]++ + 0.5) / count[wcls[w]], w};
    std::stable_sort(key.begin(), key.end());
    for (int k = 0; k < wfull; ++k) worder[k] = key[k].second;
    if (W > wfull) worder[W - 1] = W - 1;
  }
  t.cell_of_slot.resize(n);
  t.slot_of_cell.resize(n);
  int slot = 0;
  for (int k = 0; k < W; ++k)
    for (int j = worder[k] * 32; j < std::min(n, worder[k] * 32 + 32); ++j) {
      t.cell_of_slot[slot] = seq[j];
      t.slot_of_cell[seq[j]] = slot++;
    }
  // upstream lists in slot space, each in routing order (the order of the reference's pushes)
  t.up_ptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i)
    if (down[i] >= 0) t.up_ptr[t.slot_of_cell[down[i]] + 1]++;
  for (int s = 0; s < n; ++s) t.up_ptr[s + 1] += t.up_ptr[s];
  t.up_idx.resize(t.up_ptr[n]);
  std::vector<int32_t> pos(t.up_ptr.begin(), t.up_ptr.end() - 1);
  for (int k = 0; k < n; ++k) {
    const int c = order[k];
    if (down[c] >= 0) t.up_idx[pos[t.slot_of_cell[down[c]]]++] = t.slot_of_cell[c];
  }
  return WG_OK;
}

// The continental share of cell i as geo.init leaves it (geo.cpp:25-45): at least
// the cell's share of local lakes, global lakes, local reservoirs (none) and
// reservoirs, summed in that order.
double cont_share(const wg_region *r, int i) {
  double fw = 0.;
  fw += r->loc_lake[i];
  fw += r->glo_lake[i];
  fw += 0.;
  fw += r->glo_res[i];
  return fw > r->contfreq[i] ? fw : r->contfreq[i];
}

// Water-body flags of cell i and F_VINLINE (the vertical balance runs inside the
// wavefront: a water body, or no land left outside the water bodies).
uint32_t water_flags(const wg_region *r, int i) {
  uint32_t f = 0;
  if (r->loc_lake[i] > 0.) f |= F_LOCLAKE;
  if (r->loc_wetl[i] > 0.) f |= F_LOCWETL;
  if (r->lake_area[i] > 0.) f |= F_GLOLAKE;
  if (r->res_area[i] > 0.) f |= F_RES;
  if (r->glo_wetl[i] > 0) f |= F_GLOWETL;
  const double cf = cont_share(r, i);
  const double l0 = (cf - (r->glo_lake[i] + r->glo_wetl[i] + r->loc_lake[i] + r->loc_wetl[i] + r->glo_res[i]));
  if (f || !(l0 > 0.)) f |= F_VINLINE;
  if (cf < 0.000001) f |= F_NOCONT | F_VINLINE;   // limit_contcell_pct (geo.h:32)
  return f;
}

// Work class for the slot order: the branches a cell takes in the wavefront.
uint32_t work_class(const wg_region *r, int i) {
  const uint32_t f = water_flags(r, i);
  return (f & F_VINLINE) ? (f | (r->res_type[i] == 1 ? F_RES_IRRIG : 0u)) : 0u;
}

// Per-cell constants in cell order, double precision (converted to the context's
// precision on upload).
struct HostConsts {
  std::vector<uint32_t> flags;
  std::vector<int32_t> ext_row, station;
  std::vector<int16_t> init_days, band_el;
  std::vector<int8_t> start_month;
  // one vector per DevCellsT field of type R
#define WG_RFIELDS(X)                                                                                            \
  X(cfa) X(inv_cfa) X(mprec) X(alpha) X(pet_mxdy) X(mnetrad) X(mcwh) X(t_snowfz) X(t_snowmt) X(pcritgwa) X(gamma) \
  X(albedo) X(albedo_snow) X(ddf_m) X(lai_min) X(lai_max) X(smax) X(inv_smax) X(fg) X(rgmax) X(built_up)         \
  X(t_gradnt) X(elev0) X(contfreq) X(area) X(area_f) X(gw_e) X(gw_ik) X(gw_ome) X(sw_k) X(sw_e) X(sw_ik)        \
  X(sw_ome) X(evx)                                                                                               \
  X(a6) X(ll100) X(maxs_ll) X(inv_maxs_ll) X(lw100) X(maxs_lw) X(inv_maxs_lw) X(la6) X(maxs_gl) X(inv_maxs_gl)  \
  X(ra6) X(rcap) X(rcap01) X(c_ratio) X(c4) X(one_m_c4) X(prov_rel) X(gw100)                                   \
  X(maxs_gw) X(inv_maxs_gw) X(bw) X(inv_mr) X(sqrt_slope) X(inv_len) X(rlen) X(fcatch)
#define X(f) std::vector<double> f;
  WG_RFIELDS(X)
#undef X
  std::vector<double> band_dt;   // [ncell][nband]
  std::vector<double> ext, inv_s0;
  std::vector<double> statcorr;  // G_statCorrFact (P_CFS) with statcorrOpt = 1, else empty
  std::vector<float> snow_thr;   // [ncell][nband] FP32 paths' snowfall thresholds (snowfall_threshold)
  std::vector<double> t_gradnt64, t_snowfz64;
  int nrow = 0;
};

// The largest float temperature t at which a band gets snowfall as the FP64 path
// decides it: ((double)t - band_dt) <= t_snowfz (daily.cpp:982), band_dt =
// (elev_b - elev_0) * P_T_GRADNT in FP64.  The test is monotone in t, so the FP32
// paths compare their float temperature with this value and take the same
// decision for every input.
float snowfall_threshold(double band_dt, double t_snowfz) {
  auto snow = [&](float t) { return ((double)t - band_dt) <= t_snowfz; };
  float t = (float)(t_snowfz + band_dt);
  for (int k = 0; k < 64 && snow(t) && t < FLT_MAX; ++k) t = std::nextafter(t, FLT_MAX);
  for (int k = 0; k < 64 && !snow(t); ++k) t = std::nextafter(t, -FLT_MAX);
  return t;
}

inline double safe_inv(double x) { return x != 0. ? 1. / x : 0.; }

}  // namespace


namespace {

wg_status cuda_fail(wg_ctx *ctx, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return WG_OK;
  if (ctx) ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? WG_ERR_NOMEM : WG_ERR_CUDA;
}

// Runs on the context's stream wait for the overlapped forcing uploads.
void join_uploads(wg_ctx *ctx) {
  if (ctx->upload_pending) {
    cudaStreamWaitEvent(ctx->stream, ctx->upload_done, 0);
    ctx->upload_pending = false;
  }
}

bool valid_block_threads(int threads, int precision, int members) {
  const int mx = members > 1 ? PipeBounds<float, true>::threads
                             : (precision == 0 ? Bounds<double>::threads : Bounds<float>::threads);
  return threads >= 32 && threads <= mx && threads % 32 == 0;
}

// Single-member contexts: one block per SM with an equal share of the cells in
// whole warps plus one idle warp (see place_warps), so that every SM and every
// SM sub-partition carries about the same FP64 work between step barriers.
// No layout (idle_warp < 0) when the cells do not fit one block per SM or the
// block does not fit an SM.
WarpLayout default_layout(wg_ctx *ctx) {
  WarpLayout lay;
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
  if (nsm <= 0) return lay;
  const long long W = ((long long)ctx->nstate() + 31) / 32;
  const int cw = (int)std::max<long long>(2, (W + nsm - 1) / nsm);
  const int wpb = cw + 1;
  if (ctx->precision != 0 || wpb * 32 > Bounds<double>::threads) return lay;   // FP64 only
  const int blocks = (int)((W + cw - 1) / cw);
  const int fits = ctx->precision == 0 ? pipeline_max_blocks<double>(true, false, wpb * 32)
                                       : pipeline_max_blocks<float>(true, false, wpb * 32);
  const int fits_r = ctx->precision == 0 ? pipeline_max_blocks<double>(false, false, wpb * 32)
                                         : pipeline_max_blocks<float>(false, false, wpb * 32);
  if (fits < blocks || fits_r < blocks) return lay;
  // vertical-balance warps: fill the block to 20 warps (five per sub-partition at
  // the 96 registers that kernel is built for), if at least two fit
  const int va = 20 - wpb;
  if (va >= 2 && pipeline_max_blocks<double>(true, false, (wpb + va) * 32, true) >= blocks) lay.va_warps = va;
  // the idle warp: the last warp of the sub-partition that has the fewest warps
  // (of those that have any: a block of fewer than four warps leaves some empty)
  int cnt[4] = {0, 0, 0, 0};
  for (int w = 0; w < wpb; ++w) cnt[w & 3]++;
  int sp = 0;
  for (int k = 1; k < 4; ++k)
    if (cnt[k] > 0 && cnt[k] < cnt[sp]) sp = k;
  int idle = -1;
  for (int w = 0; w < wpb; ++w)
    if ((w & 3) == sp) idle = w;
  lay.cell_warps = cw;
  lay.idle_warp = idle;
  lay.blocks = blocks;
  lay.threads = wpb * 32;
  return lay;
}

// upload a per-cell host array (cell order) into slot order, converting to T
template <class T, class S>
const T *upload_slots(wg_ctx *ctx, const std::vector<S> &by_cell, wg_status &st) {
  std::vector<T> by_slot(by_cell.size());
  for (size_t s = 0; s < by_slot.size(); ++s) by_slot[s] = (T)by_cell[ctx->topo.cell_of_slot[s]];
  T *d = ctx->alloc<T>(by_slot.size());
  if (!d) { st = WG_ERR_NOMEM; return nullptr; }
  cudaError_t e = cudaMemcpy(d, by_slot.data(), by_slot.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) st = cuda_fail(ctx, e, "upload");
  return d;
}

template <class T, class S>
const T *upload_raw(wg_ctx *ctx, const std::vector<S> &v, wg_status &st) {
  std::vector<T> c(v.begin(), v.end());
  T *d = ctx->alloc<T>(c.size());
  if (!d) { st = WG_ERR_NOMEM; return nullptr; }
  cudaError_t e = cudaMemcpy(d, c.data(), c.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) st = cuda_fail(ctx, e, "upload");
  return d;
}

// Step flags of the single-member layout: for every warp of cells (slots
// 32w..32w+31) the warps holding its cells' upstream and downstream cells.
wg_status setup_step_flags(wg_ctx *ctx) {
  const int n = ctx->n, W = (n + 31) / 32;
  std::vector<std::vector<int32_t>> deps(W);
  for (int sl = 0; sl < n; ++sl) {
    const int w = sl / 32;
    for (int k = ctx->topo.up_ptr[sl]; k < ctx->topo.up_ptr[sl + 1]; ++k) {
      const int u = ctx->topo.up_idx[k] / 32;
      if (u != w) {
        deps[w].push_back(u);
        deps[u].push_back(w);   // w is downstream of u
      }
    }
  }
  std::vector<int32_t> ptr(W + 1, 0), idx;
  for (int w = 0; w < W; ++w) {
    auto &d = deps[w];
    std::sort(d.begin(), d.end());
    d.erase(std::unique(d.begin(), d.end()), d.end());
    ptr[w + 1] = ptr[w] + (int32_t)d.size();
    idx.insert(idx.end(), d.begin(), d.end());
  }
  wg_status st = WG_OK;
  ctx->sync.dep_ptr = upload_raw<int32_t>(ctx, ptr, st);
  ctx->sync.dep_idx = upload_raw<int32_t>(ctx, idx, st);
  ctx->sync.wstep = ctx->alloc<int>(W);
  if (st != WG_OK) return st;
  if (!ctx->sync.wstep) return WG_ERR_NOMEM;
  ctx->sync.nwarps = W;
  ctx->sync.flow = 0;   // measured on GB300: the grid barrier is 3.6 % faster (flags: wg_set_step_sync)
  return WG_OK;
}

// band-major slot layout of a cell-major [ncell][nb] array
template <class T, class S>
std::vector<T> bands_to_slots(const wg_ctx *ctx, const S *cellmajor, int nb) {
  const int n = ctx->n;
  std::vector<T> out((size_t)n * nb);
  for (int s = 0; s < n; ++s) {
    const int c = ctx->topo.cell_of_slot[s];
    for (int b = 0; b < nb; ++b) out[(size_t)b * n + s] = (T)cellmajor[(size_t)c * nb + b];
  }
  return out;
}

template <class R>
wg_status upload_cells(wg_ctx *ctx, const HostConsts &h, DevCellsT<R> &c, double default_velocity, int velo_opt) {
  wg_status st = WG_OK;
  c.n = ctx->n;
  c.nband = ctx->nband;
  c.velo_opt = velo_opt;
  c.frac_routing = ctx->frac_routing;
  c.nrow = h.nrow;
  c.default_velocity = (R)default_velocity;
  c.invB = (R)(1.0 / ctx->nband);
  c.nlevel = ctx->topo.nlevel;
  c.nstation = ctx->nstation;
  c.flags = upload_slots<uint32_t>(ctx, h.flags, st);
  c.ext_row = upload_slots<int32_t>(ctx, h.ext_row, st);
  c.station = upload_slots<int32_t>(ctx, h.station, st);
  c.init_days = upload_slots<int16_t>(ctx, h.init_days, st);
  c.start_month = upload_slots<int8_t>(ctx, h.start_month, st);
#define X(f) c.f = upload_slots<R>(ctx, h.f, st);
  WG_RFIELDS(X)
#undef X
  c.band_dt = upload_raw<R>(ctx, bands_to_slots<double>(ctx, h.band_dt.data(), ctx->nband), st);
  c.snow_thr = nullptr;
  c.thr64 = nullptr;
  if (sizeof(R) == 4) {   // the FP32 paths' snowfall decisions (vertical_cell)
    c.snow_thr = upload_raw<float>(ctx, bands_to_slots<float>(ctx, h.snow_thr.data(), ctx->nband), st);
    // the arid recharge rule dailyPrec <= P_PCRITGWA (daily.cpp:1172) on a float
    // precipitation: against the largest float not above the FP64 threshold it
    // takes the FP64 path's decision for every input
    std::vector<float> pc(ctx->n);
    for (int i = 0; i < ctx->n; ++i) {
      float f = (float)h.pcritgwa[i];
      if ((double)f > h.pcritgwa[i]) f = std::nextafter(f, -FLT_MAX);
      pc[i] = f;
    }
    c.pcritgwa = (const R *)upload_slots<float>(ctx, pc, st);
    std::vector<double> t64(2 * (size_t)ctx->n);
    for (int sl = 0; sl < ctx->n; ++sl) {
      const int cell = ctx->topo.cell_of_slot[sl];
      t64[sl] = h.t_gradnt64[cell];
      t64[(size_t)ctx->n + sl] = h.t_snowfz64[cell];
    }
    c.thr64 = upload_raw<double>(ctx, t64, st);
  }
  c.band_el = upload_raw<int16_t>(ctx, bands_to_slots<int16_t>(ctx, h.band_el.data(), ctx->nband), st);
  c.ext_rad = upload_raw<R>(ctx, h.ext, st);
  c.inv_s0 = upload_raw<R>(ctx, h.inv_s0, st);
  std::vector<int32_t> off_slot(ctx->n);
  for (int s = 0; s < ctx->n; ++s) off_slot[s] = ctx->topo.offset[ctx->topo.cell_of_slot[s]];
  c.offset = upload_raw<int32_t>(ctx, off_slot, st);
  c.up_ptr = upload_raw<int32_t>(ctx, ctx->topo.up_ptr, st);
  c.up_idx = upload_raw<int32_t>(ctx, ctx->topo.up_idx, st);
  c.statcorr = h.statcorr.empty() ? nullptr : upload_slots<R>(ctx, h.statcorr, st);
  return st;
}


template <class R>
wg_status alloc_state(wg_ctx *ctx, DevStateT<R> &s, DevVertT<R> &v) {
  const size_t N = ctx->nstate();
#define X(f) s.f = ctx->alloc<R>(N); if (!s.f) return WG_ERR_NOMEM;
  WG_STATE_R(X)
#undef X
#define X(f) s.f = ctx->alloc<int32_t>(N); if (!s.f) return WG_ERR_NOMEM;
  WG_STATE_I(X)
#undef X
  s.snow_band = ctx->alloc<R>(N * ctx->nband);
  if (!s.snow_band) return WG_ERR_NOMEM;
  const int n = ctx->n;
  v.rs = ctx->alloc<R>(n); v.gwr = ctx->alloc<R>(n); v.transfer = ctx->alloc<R>(n); v.owp = ctx->alloc<R>(n);
  v.owpet = ctx->alloc<R>(n); v.land_in = ctx->alloc<R>(n); v.land_evap = ctx->alloc<R>(n);
  v.land_leak = ctx->alloc<R>(n);
  return v.land_leak ? WG_OK : WG_ERR_NOMEM;
}

// Copy one member's state between host arrays (cell order, double) and the device.
template <class R>
wg_status copy_state(wg_ctx *ctx, const DevStateT<R> &s, const wg_state_view *v, int member, bool to_device) {
  const int n = ctx->n, B = ctx->nband, M = ctx->members;
  const size_t N = ctx->nstate();
  const auto &c2s = ctx->topo.cell_of_slot;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  // gather/scatter the member's values with a strided 2D copy (member innermost)
  std::vector<R> tmp(n);
  std::vector<int32_t> itmp(n);
  auto xfer = [&](void *host_slots, void *dev, size_t elem) {
    if (e != cudaSuccess) return;
    char *base = (char *)dev + (size_t)member * elem;
    if (to_device)
      e = cudaMemcpy2D(base, elem * M, host_slots, elem, elem, n, cudaMemcpyHostToDevice);
    else
      e = cudaMemcpy2D(host_slots, elem, base, elem * M, elem, n, cudaMemcpyDeviceToHost);
  };
  auto dbl = [&](double *host, R *dev) {
    if (!host) return;
    if (to_device) {
      for (int q = 0; q < n; ++q) tmp[q] = (R)host[c2s[q]];
      xfer(tmp.data(), dev, sizeof(R));
    } else {
      xfer(tmp.data(), dev, sizeof(R));
      for (int q = 0; q < n; ++q) host[c2s[q]] = (double)tmp[q];
    }
  };
  auto i32 = [&](int32_t *host, int32_t *dev) {
    if (!host) return;
    if (to_device) {
      for (int q = 0; q < n; ++q) itmp[q] = host[c2s[q]];
      xfer(itmp.data(), dev, sizeof(int32_t));
    } else {
      xfer(itmp.data(), dev, sizeof(int32_t));
      for (int q = 0; q < n; ++q) host[c2s[q]] = itmp[q];
    }
  };
#define X(f) dbl(v->f, s.f);
  WG_STATE_R(X)
#undef X
#define X(f) i32(v->f, s.f);
  WG_STATE_I(X)
#undef X
  if (v->snow_band) {
    for (int b = 0; b < B; ++b) {
      R *dev = s.snow_band + (size_t)b * N;
      if (to_device) {
        for (int q = 0; q < n; ++q) tmp[q] = (R)v->snow_band[(size_t)c2s[q] * B + b];
        xfer(tmp.data(), dev, sizeof(R));
      } else {
        xfer(tmp.data(), dev, sizeof(R));
        for (int q = 0; q < n; ++q) v->snow_band[(size_t)c2s[q] * B + b] = (double)tmp[q];
      }
    }
  }
  return cuda_fail(ctx, e, to_device ? "set_state" : "get_state");
}

// The same host state (cell order) into every member, one copy per field.
template <class R>
wg_status broadcast_state(wg_ctx *ctx, const DevStateT<R> &s, const wg_state_view *v) {
  const int n = ctx->n, B = ctx->nband, M = ctx->members;
  const size_t N = ctx->nstate();
  const auto &c2s = ctx->topo.cell_of_slot;
  cudaError_t e = cudaSuccess;
  std::vector<R> tmp(N);
  std::vector<int32_t> itmp(N);
  auto dbl = [&](const double *host, R *dev) {
    if (e != cudaSuccess) return;
    for (int q = 0; q < n; ++q)
      for (int m = 0; m < M; ++m) tmp[(size_t)q * M + m] = (R)host[c2s[q]];
    e = cudaMemcpy(dev, tmp.data(), N * sizeof(R), cudaMemcpyHostToDevice);
  };
  auto i32 = [&](const int32_t *host, int32_t *dev) {
    if (e != cudaSuccess) return;
    for (int q = 0; q < n; ++q)
      for (int m = 0; m < M; ++m) itmp[(size_t)q * M + m] = host[c2s[q]];
    e = cudaMemcpy(dev, itmp.data(), N * sizeof(int32_t), cudaMemcpyHostToDevice);
  };
#define X(f) dbl(v->f, s.f);
  WG_STATE_R(X)
#undef X
#define X(f) i32(v->f, s.f);
  WG_STATE_I(X)
#undef X
  for (int b = 0; b < B && e == cudaSuccess; ++b) {
    for (int q = 0; q < n; ++q)
      for (int m = 0; m < M; ++m) tmp[(size_t)q * M + m] = (R)v->snow_band[(size_t)c2s[q] * B + b];
    e = cudaMemcpy(s.snow_band + (size_t)b * N, tmp.data(), N * sizeof(R), cudaMemcpyHostToDevice);
  }
  return cuda_fail(ctx, e, "initial state");
}

wg_status state_io(wg_ctx *ctx, const wg_state_view *v, int member, bool to_device) {
  if (member < 0 || member >= ctx->members) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  return ctx->precision == 0 ? copy_state(ctx, ctx->sd, v, member, to_device)
                             : copy_state(ctx, ctx->sf, v, member, to_device);
}

void fill_fastmath_tables(double e2[64], double lf[129], double inv[129]) {
  for (int j = 0; j < 64; ++j) e2[j] = exp2((double)j / 64.0);
  for (int j = 0; j <= 128; ++j) {
    const double F = 1.0 + j / 128.0;
    lf[j] = log(F);
    inv[j] = 1.0 / F;
  }
}

}  // namespace

namespace {
template <class R>
wg_status set_calib_param(wg_ctx *ctx, const DevCellsT<R> &c, int32_t k, const double *values) {
  const int n = ctx->n;
  std::vector<R> a(n), b(n);
  for (int s = 0; s < n; ++s) {
    const double v = values[ctx->topo.cell_of_slot[s]];
    a[s] = (R)v;
    b[s] = (R)safe_inv(v);
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (k == 0) {
    if (e == cudaSuccess) e = cudaMemcpy((R *)c.gamma, a.data(), n * sizeof(R), cudaMemcpyHostToDevice);
  } else {
    if (e == cudaSuccess) e = cudaMemcpy((R *)c.cfa, a.data(), n * sizeof(R), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy((R *)c.inv_cfa, b.data(), n * sizeof(R), cudaMemcpyHostToDevice);
  }
  return cuda_fail(ctx, e, "set_calib_param");
}
}  // namespace

// cell-order host array -> slot-order device array (n values)
template <class T>
static wg_status to_slots(wg_ctx *ctx, const T *host, T *dev) {
  std::vector<T> v(ctx->n);
  for (int s = 0; s < ctx->n; ++s) v[s] = host[ctx->topo.cell_of_slot[s]];
  return cuda_fail(ctx, cudaMemcpy(dev, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "water temperature");
}

static wg_status vertical_now(wg_ctx *ctx, int doy, int fday);
static wg_status routing_now(wg_ctx *ctx, int doy, int oday);

extern "C" {

const char *wg_status_string(wg_status s) {
  switch (s) {
    case WG_OK: return "ok";
    case WG_ERR_INVALID: return "invalid argument";
    case WG_ERR_UNSUPPORTED: return "unsupported option";
    case WG_ERR_CUDA: return "CUDA error";
    case WG_ERR_NOMEM: return "out of device memory";
    case WG_ERR_TOPOLOGY: return "invalid drainage topology";
    case WG_ERR_TIMEOUT: return "device wait exceeded its limit";
    case WG_ERR_DEVICE: return "no usable device";
  }
  return "unknown";
}

// why the calling thread's last wg_create failed (wg_last_error(NULL))
thread_local std::string t_create_err;

const char *wg_last_error(const wg_ctx *ctx) { return ctx ? ctx->err.c_str() : t_create_err.c_str(); }

void wg_model_options_default(wg_model_options *o) {
  if (!o) return;
  *o = wg_model_options{};
  o->time_series = 1;
  o->cloud = 2;
  o->intercept = 1;
  o->res_opt = 1;
}
int32_t wg_num_levels(const wg_ctx *ctx) { return ctx ? ctx->topo.nlevel : 0; }
int64_t wg_launch_count(const wg_ctx *ctx) { return ctx ? ctx->launches : 0; }

// Provisional release of a reservoir [m3/s] for the month's use of the cell
// [m3/s] (routing.cpp:2970-2994): irrigation reservoirs (type 1) follow the
// demand, others release their mean outflow.
static double provisional_release(int type, double mean_outflow, double mean_demand, double monthlyUse) {
  if (type != 1) return mean_outflow;
  if (mean_demand >= 0.5 * mean_outflow) return mean_outflow / 2. * (1. + monthlyUse / mean_demand);
  return mean_outflow + monthlyUse - mean_demand;
}

// Water-use tables and state: blocks of 12 monthly rows, block 0 without use
// (the provisional release of every reservoir as without water use), one block
// per year uploaded, enough for a run of max_days; state at zero.
static wg_status setup_water_use(wg_ctx *ctx, const wg_region *r) {
  const int n = ctx->n;
  const size_t N = ctx->nstate();   // state per member, tables per cell
  DevWaterUse &w = ctx->wu;
  ctx->wu_blocks = 1 + ((ctx->max_days + 364) / 365 + 1);
  const size_t block = (size_t)12 * wg::WU_FIELDS * n;
  w.tab = ctx->alloc<double>((size_t)ctx->wu_blocks * block);
  w.row_of_fday = ctx->alloc<int32_t>((size_t)ctx->max_days);
  w.frgi = ctx->alloc<double>((size_t)n);
  w.st = ctx->alloc<double>((size_t)wg::WU_NSTATE * N);
  if (!w.tab || !w.row_of_fday || !w.frgi || !w.st) return WG_ERR_NOMEM;
  ctx->wu_prov0.assign(n, 0.);
  ctx->wu_res.clear();
  for (int s = 0; s < n; ++s) {
    const int i = ctx->topo.cell_of_slot[s];
    if (r->res_area[i] > 0.) {
      ctx->wu_prov0[s] = provisional_release(r->res_type[i], r->mean_outflow[i], r->mean_demand[i], 0.0);
      ctx->wu_res.push_back({s, i, (int)r->res_type[i], r->mean_outflow[i], r->mean_demand[i]});
    }
  }
  std::vector<double> zero(block, 0.);
  for (int m = 0; m < 12; ++m)
    std::copy(ctx->wu_prov0.begin(), ctx->wu_prov0.end(), zero.begin() + ((size_t)m * wg::WU_FIELDS + 4) * n);
  cudaError_t e = cudaMemcpy((void *)w.tab, zero.data(), block * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset((void *)w.row_of_fday, 0, (size_t)ctx->max_days * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMemset((void *)w.frgi, 0, (size_t)n * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(w.st, 0, (size_t)wg::WU_NSTATE * N * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "water use");
  if (ctx->glwd.on) {   // the units in slot space: per unit its slots in routing order and in cell order
    const auto &g = ctx->glwd;
    const size_t nu = g.ptr.size() - 1;
    std::vector<int32_t> unit_of(n), mem(g.cells.size()), idx(g.cells.size());
    for (int s = 0; s < n; ++s) unit_of[s] = g.unit_of[ctx->topo.cell_of_slot[s]];
    for (size_t u = 0; u < nu; ++u) {
      std::vector<int32_t> by_rout(g.cells.begin() + g.ptr[u], g.cells.begin() + g.ptr[u + 1]);
      std::sort(by_rout.begin(), by_rout.end(),
                [&](int a, int b) { return ctx->topo.rout_pos[a] < ctx->topo.rout_pos[b]; });
      for (int k = g.ptr[u]; k < g.ptr[u + 1]; ++k) {
        mem[k] = ctx->topo.slot_of_cell[by_rout[k - g.ptr[u]]];
        idx[k] = ctx->topo.slot_of_cell[g.cells[k]];
      }
    }
    wg_status us = WG_OK;
    w.unit_of = upload_raw<int32_t>(ctx, unit_of, us);
    w.unit_ptr = upload_raw<int32_t>(ctx, g.ptr, us);
    w.unit_mem = upload_raw<int32_t>(ctx, mem, us);
    w.unit_idx = upload_raw<int32_t>(ctx, idx, us);
    if (us != WG_OK) return us;
    w.glwd = 1;
  }
  w.enabled = 1;
  return WG_OK;
}

// GLWD units of a region (aggrNUsGloLakResOpt = 1): every outflow cell of a
// global lake or reservoir needs a unit > 0 and a unit at most one outflow cell
// (the reference's loops would otherwise aggregate over every cell without a
// unit, or twice: routing.cpp:935-962, 3094-3095).
static wg_status glwd_setup(const wg_region *r, wg_ctx::Glwd &g) {
  const int n = r->ncell;
  g.unit.assign(r->glwd_unit, r->glwd_unit + n);
  g.outflow.assign(n, 0);
  g.unit_of.assign(n, -1);
  std::map<int32_t, std::vector<int32_t>> cells;   // unit -> cells in cell order
  for (int i = 0; i < n; ++i) {
    g.outflow[i] = (r->lake_area[i] > 0. || r->res_area[i] > 0.) ? 1 : 0;
    if (g.outflow[i] && g.unit[i] <= 0) {
      t_create_err = "GLWD units: outflow cell " + std::to_string(i) + " of a global lake or reservoir has no unit";
      return WG_ERR_INVALID;
    }
    if (g.unit[i] > 0) cells[g.unit[i]].push_back(i);
  }
  g.ptr.assign(1, 0);
  g.cells.clear();
  for (const auto &kv : cells) {
    int outflows = 0;
    for (int c : kv.second) outflows += g.outflow[c];
    if (outflows > 1) {
      t_create_err = "GLWD units: unit " + std::to_string(kv.first) + " has " + std::to_string(outflows) +
                     " outflow cells of global lakes or reservoirs";
      return WG_ERR_INVALID;
    }
    const int u = outflows ? (int)g.ptr.size() - 1 : -2;
    for (int c : kv.second) g.unit_of[c] = u;
    if (outflows) {
      g.cells.insert(g.cells.end(), kv.second.begin(), kv.second.end());
      g.ptr.push_back((int32_t)g.cells.size());
    }
  }
  g.on = true;
  return WG_OK;
}

// dailyNUInit's aggregation of one month's NUs [m3, cell order] over the GLWD
// units (routing.cpp:926-965): each outflow cell, in cell order, takes the
// aggregated value of every other cell of its unit whose own NUs is positive,
// which drops to zero.
static void glwd_aggregate(const wg_ctx::Glwd &g, const double *nus, double *out, int n) {
  std::copy(nus, nus + n, out);
  for (size_t u = 0; u + 1 < g.ptr.size(); ++u) {
    int o = -1;
    for (int k = g.ptr[u]; k < g.ptr[u + 1]; ++k)
      if (g.outflow[g.cells[k]]) o = g.cells[k];
    for (int k = g.ptr[u]; k < g.ptr[u + 1]; ++k) {
      const int i = g.cells[k];
      if (i == o) continue;
      if (nus[i] > 0.) {
        out[o] += out[i];
        out[i] = 0.;
      }
    }
  }
}

// Water temperature buffers: state at the reference's start values (15 degC, no
// ice: routing.cpp:172-197), the per-cell inputs in slot order.
static wg_status setup_water_temp(wg_ctx *ctx, const wg_region *r) {
  const int n = ctx->n;
  const size_t N = ctx->nstate();
  DevWaterTemp &w = ctx->wt;
  w.temp = ctx->alloc<double>(6 * N);
  w.ice = ctx->alloc<double>(6 * N);
  w.outt = ctx->alloc<double>((size_t)2 * ctx->days_per_step * N);
  w.lw = ctx->alloc<float>((size_t)ctx->max_days * n);
  w.qst_t = ctx->alloc<double>((size_t)ctx->max_days * std::max(1, ctx->nstation));
  if (!w.temp || !w.ice || !w.outt || !w.lw || !w.qst_t) return WG_ERR_NOMEM;
  wg_status st = WG_OK;
  std::vector<float> gwt(n, 10.f);
  std::vector<double> lake(r->lake_area, r->lake_area + n), res(r->res_area, r->res_area + n);
  std::vector<double> ll(r->loc_lake, r->loc_lake + n), lw(r->loc_wetl, r->loc_wetl + n);
  std::vector<double> gw(r->glo_wetl, r->glo_wetl + n), len(r->river_length, r->river_length + n);
  w.gwt = upload_slots<float>(ctx, gwt, st);
  w.len_check = upload_slots<double>(ctx, len, st);
  w.lake_km2 = upload_slots<double>(ctx, lake, st);
  w.res_km2 = upload_slots<double>(ctx, res, st);
  w.ll_pct = upload_slots<double>(ctx, ll, st);
  w.lw_pct = upload_slots<double>(ctx, lw, st);
  w.gw_pct = upload_slots<double>(ctx, gw, st);
  if (st != WG_OK) return st;
  std::vector<double> t15(6 * N, 15.), zero(6 * N, 0.);
  cudaError_t e = cudaMemcpy(w.temp, t15.data(), 6 * N * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(w.ice, zero.data(), 6 * N * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(w.outt, 0, (size_t)2 * ctx->days_per_step * N * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset((void *)w.lw, 0, (size_t)ctx->max_days * n * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(w.qst_t, 0, (size_t)ctx->max_days * std::max(1, ctx->nstation) * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "water temperature");
  w.enabled = 1;
  return WG_OK;
}

namespace {

// The reference's options outside the built set: refused with their name.
wg_status check_model_options(const wg_region *r, const wg_options *opt) {
  wg_model_options m;
  wg_model_options_default(&m);
  if (opt->model) m = *opt->model;
  struct {
    const char *name;
    int32_t value, want;
  } fixed[] = {{"time_series", m.time_series, 1}, {"cloud", m.cloud, 2}, {"intercept", m.intercept, 1},
               {"calc_albedo", m.calc_albedo, 0}, {"use_kc", m.use_kc, 0}, {"petOpt", m.pet_opt, 0},
               {"clclOpt", m.clcl_opt, 0}, {"permaOpt", m.perma_opt, 0}, {"glacierOpt", m.glacier_opt, 0},
               {"landCoverOpt", m.land_cover_opt, 0}, {"aridareaOpt", m.arid_area_opt, 0},
               {"riverEvapoOpt", m.river_evapo_opt, 0}, {"use_alloc", m.use_alloc, 0},
               {"antNatOpt", m.ant_nat_opt, 0},
               {"resYearOpt", m.res_year_opt, 0}, {"climate_spatial_resolution", m.climate_spatial_resolution, 0}};
  for (const auto &f : fixed)
    if (f.value != f.want) {
      t_create_err = std::string("options.") + f.name + " = " + std::to_string(f.value) +
                     " is not built (built: " + std::to_string(f.want) + ")";
      return WG_ERR_UNSUPPORTED;
    }
  if (m.aggr_nus_glo_lak_res_opt != 0 && m.aggr_nus_glo_lak_res_opt != 1) {
    t_create_err = "options.aggrNUsGloLakResOpt = " + std::to_string(m.aggr_nus_glo_lak_res_opt) +
                   " is not built (built: 0, 1)";
    return WG_ERR_UNSUPPORTED;
  }
  if (m.aggr_nus_glo_lak_res_opt == 1) {
    if (!opt->water_use || !r->glwd_unit) {
      t_create_err = "options.aggrNUsGloLakResOpt = 1 needs water use and the GLWD units (wg_region.glwd_unit)";
      return WG_ERR_INVALID;
    }
    if (opt->precision != 0 || opt->members != 1 || opt->water_temp) {
      t_create_err = "options.aggrNUsGloLakResOpt = 1 is built for FP64, one member, without the water temperature";
      return WG_ERR_UNSUPPORTED;
    }
  }
  if (m.statcorr_opt != 0 && m.statcorr_opt != 1) {
    t_create_err = "options.statcorrOpt = " + std::to_string(m.statcorr_opt) + " is not built (built: 0, 1)";
    return WG_ERR_UNSUPPORTED;
  }
  if (m.statcorr_opt == 1 && opt->water_temp) {
    t_create_err = "options.statcorrOpt = 1 together with calc_wtemp = 1 is not built";
    return WG_ERR_UNSUPPORTED;
  }
  if (m.res_opt != 1) {
    bool any_res = false;
    for (int i = 0; i < r->ncell && !any_res; ++i) any_res = r->res_area[i] > 0.;
    if (m.res_opt != 0 || any_res) {
      t_create_err = "options.resOpt = " + std::to_string(m.res_opt) +
                     " is not built (built: 1; 0 for a region without reservoirs)";
      return WG_ERR_UNSUPPORTED;
    }
  }
  if (r->river_velo_opt < 0 || r->river_velo_opt > 2) {
    t_create_err = "options.riverveloOpt = " + std::to_string(r->river_velo_opt) + " is not built (built: 0, 1, 2)";
    return WG_ERR_UNSUPPORTED;
  }
  return WG_OK;
}

}  // namespace

wg_status wg_create(const wg_region *r, const wg_options *opt, wg_ctx **out) {
  t_create_err.clear();
  if (!r || !opt || !out) return WG_ERR_INVALID;
  *out = nullptr;
  if (wg_status ms = check_model_options(r, opt); ms != WG_OK) return ms;
  if (r->ncell <= 0 || r->nband <= 0 || r->nband > 256 || opt->max_days <= 0) return WG_ERR_INVALID;
  if (r->river_velo_opt < 0 || r->river_velo_opt > 2) return WG_ERR_UNSUPPORTED;
  if (r->frac_routing < 0 || r->frac_routing > 1) return WG_ERR_INVALID;
  if (opt->precision < 0 || opt->precision > 1) return WG_ERR_UNSUPPORTED;
  if (opt->members < 1 || (opt->members > 1 && opt->precision != 1)) return WG_ERR_UNSUPPORTED;
  if (opt->nstation < 0 || (opt->nstation > 0 && !opt->stations)) return WG_ERR_INVALID;
  if (opt->block_threads != 0 && !valid_block_threads(opt->block_threads, opt->precision, opt->members))
    return WG_ERR_INVALID;
  if (opt->days_per_step < 0 || opt->days_per_step > 31) return WG_ERR_INVALID;
  if (opt->water_temp < 0 || opt->water_temp > 1) return WG_ERR_INVALID;
  if (opt->water_temp && (opt->precision != 0 || opt->members != 1)) return WG_ERR_UNSUPPORTED;
  if (opt->water_use < 0 || opt->water_use > 2) return WG_ERR_INVALID;
  if (opt->water_use && opt->water_temp && (opt->precision != 0 || opt->members != 1)) return WG_ERR_UNSUPPORTED;
  const bool aggr = opt->model && opt->model->aggr_nus_glo_lak_res_opt == 1;
  const int n = r->ncell, B = r->nband;
  for (int i = 0; i < n; ++i) {
    if (r->lct[i] < 1 || r->lct[i] > WG_NLCT) return WG_ERR_INVALID;
    if (r->res_area[i] > 0.) {
      if (r->res_type[i] != 1 && r->res_type[i] != 2) return WG_ERR_INVALID;
      if (!(r->mean_outflow[i] > 0.) || r->start_month[i] < 1 || r->start_month[i] > 12) return WG_ERR_INVALID;
    }
    // a river needs a length; cells without continental area are not routed, and
    // their length (scaled by the share) may be 0
    if (!(r->river_length[i] > 0.) && !(cont_share(r, i) < 0.000001)) return WG_ERR_INVALID;
  }
  wg_ctx::Glwd glwd;   // GLWD units, checked before any device is touched
  if (aggr) {
    wg_status gs = glwd_setup(r, glwd);
    if (gs != WG_OK) return gs;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= opt->device) return WG_ERR_DEVICE;
  std::unique_ptr<wg_ctx> ctx(new wg_ctx());
  ctx->glwd = std::move(glwd);
  ctx->device = opt->device;
  ctx->n = n;
  ctx->nband = B;
  ctx->max_days = opt->max_days;
  ctx->nstation = opt->nstation;
  ctx->members = opt->members;
  ctx->precision = opt->precision;
  ctx->threads = opt->block_threads ? opt->block_threads : (opt->members > 1 ? 64 : 256);
  ctx->days_per_step = opt->days_per_step ? opt->days_per_step : 1;
  ctx->frac_routing = r->frac_routing;
  if (cudaSetDevice(opt->device) != cudaSuccess) return WG_ERR_DEVICE;
  if (opt->stream) {
    ctx->stream = (cudaStream_t)opt->stream;
  } else {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return WG_ERR_CUDA;
    ctx->own_stream = true;
  }
  if (cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->upload_done, cudaEventDisableTiming) != cudaSuccess)
    return WG_ERR_CUDA;
  std::vector<uint32_t> cls(n);
  for (int i = 0; i < n; ++i) cls[i] = work_class(r, i);
  if (!opt->block_threads && ctx->members == 1) ctx->layout = default_layout(ctx.get());
  ctx->va_warps_default = ctx->layout.va_warps;
  std::vector<int32_t> node_of;   // GLWD units: a unit's cells are one node of the wavefront
  if (aggr) {
    std::vector<int32_t> order;
    if (r->rout_order) order.assign(r->rout_order, r->rout_order + n);
    else if (reference_rout_order(n, r->downstream, order) != WG_OK) return WG_ERR_TOPOLOGY;
    node_of.resize(n);
    for (int i = 0; i < n; ++i) node_of[i] = i;
    std::vector<int32_t> first(ctx->glwd.ptr.size(), -1);   // per unit its first cell in routing order
    for (int k = 0; k < n; ++k) {
      const int c = order[k];
      if (c < 0 || c >= n) return WG_ERR_TOPOLOGY;
      const int u = ctx->glwd.unit_of[c];
      if (u >= 0 && first[u] < 0) first[u] = c;
    }
    for (int i = 0; i < n; ++i)
      if (ctx->glwd.unit_of[i] >= 0) node_of[i] = first[ctx->glwd.unit_of[i]];
  }
  wg_status st = build_topology(n, r->downstream, r->rout_order, cls.data(), &ctx->layout, ctx->topo,
                                aggr ? node_of.data() : nullptr);
  if (st != WG_OK) {
    if (aggr && st == WG_ERR_TOPOLOGY)
      t_create_err = "GLWD units: the cells of a unit drain out of it and back in (no wavefront order)";
    return st;
  }
  {
    double e2[64], lf[129], inv[129];
    fill_fastmath_tables(e2, lf, inv);
    st = cuda_fail(ctx.get(), upload_fastmath_tables(e2, lf, inv), "fastmath tables");
    if (st != WG_OK) return st;
  }

  // ----- per-cell constants in cell order, with the reference's expressions
  auto P = [&](int k, int i) { return r->param[(size_t)k * n + i]; };
  enum { GAMRUN = 0, CFA = 1, CFS = 2, RIVRGH = 4, LAK_D = 5, WET_D = 6, SWOUTF = 7, EVAREDEX = 8, NETRAD = 9, PTC_HUM = 10,
         PTC_ARI = 11, PET_MXDY = 12, MCWH = 13, T_SNOWFZ = 15, T_SNOWMT = 16, DEGDAY = 17, T_GRADNT = 18,
         PCRITGWA = 21, GWOUTF = 22, PREC = 25 };
  HostConsts h;
  ctx->has_kc = r->lct_kc_min && r->lct_kc_max;
  ctx->cell_area.assign(r->area_km2, r->area_km2 + n);
  ctx->cell_cont.resize(n);
  for (int i = 0; i < n; ++i) ctx->cell_cont[i] = cont_share(r, i);
  ctx->vstatic.assign((size_t)(wg::VCONST_FIELDS + 1) * n, 0.);
  h.flags.resize(n); h.ext_row.resize(n); h.station.assign(n, -1); h.init_days.resize(n); h.start_month.resize(n);
#define X(f) h.f.assign(n, 0.);
  WG_RFIELDS(X)
#undef X
  h.band_dt.resize((size_t)n * B);
  h.band_el.resize((size_t)n * B);
  h.snow_thr.resize((size_t)n * B);
  h.t_gradnt64.resize(n);
  h.t_snowfz64.resize(n);
  std::vector<double> lats;
  for (int i = 0; i < n; ++i) {
    const int lct = r->lct[i];
    uint32_t f = 0;
    if (r->aindex[i] == 1) f |= F_ARID;
    if (r->aindex[i] == 1 && r->texture[i] < 21) f |= F_ARID_GW;
    if (r->ldd[i] < 0) f |= F_SINK;
    if (lct <= 2) f |= F_EVERGREEN;
    f |= water_flags(r, i);
    if (r->res_type[i] == 1) f |= F_RES_IRRIG;
    if (r->downstream[i] < 0) f |= F_OUTLET;
    h.flags[i] = f;
    const double ar = r->area_km2[i];
    h.area[i] = ar;
    h.contfreq[i] = cont_share(r, i);
    h.area_f[i] = ar * 1e-8;
    h.a6[i] = ar / 1000000.;
    h.albedo[i] = r->lct_albedo[lct - 1];
    h.albedo_snow[i] = r->lct_albedo_snow[lct - 1];
    h.ddf_m[i] = P(DEGDAY, i) * r->lct_ddf[lct - 1];
    const float lmin = r->lct_lai_a[lct - 1] + r->lct_lai_b[lct - 1] * r->lai_max[i];   // lai.cpp:154 (float)
    h.lai_min[i] = lmin;
    h.lai_max[i] = r->lai_max[i];
    {   // the output grids' constants: Kc (lai.cpp:295-306, LAImin in float as there),
        // the first year's freshwater share (routing.cpp:1213), the global-lake and
        // reservoir shares, G_loc_lake / 100
      double *v = ctx->vstatic.data();
      if (ctx->has_kc) {
        const double kmin = r->lct_kc_min[lct - 1], kmax = r->lct_kc_max[lct - 1];
        const double den = (double)r->lai_max[i] - (double)lmin;
        v[i] = kmin;
        v[(size_t)n + i] = den == 0. ? 0. : (kmax - kmin) / den;
      }
      v[2 * (size_t)n + i] = lmin;
      v[3 * (size_t)n + i] = r->glo_lake[i] + r->loc_lake[i] + r->glo_res[i];
      v[4 * (size_t)n + i] = r->glo_lake[i];
      v[5 * (size_t)n + i] = r->glo_res[i];
      v[6 * (size_t)n + i] = r->loc_lake[i] / 100.;
    }
    h.init_days[i] = r->lct_initial_days[lct - 1];
    h.mprec[i] = P(PREC, i);
    h.alpha[i] = (r->aindex[i] == 1) ? P(PTC_ARI, i) : P(PTC_HUM, i);
    h.pet_mxdy[i] = P(PET_MXDY, i);
    h.mnetrad[i] = P(NETRAD, i);
    h.mcwh[i] = P(MCWH, i);
    h.t_snowfz[i] = P(T_SNOWFZ, i);
    h.t_snowmt[i] = P(T_SNOWMT, i);
    h.pcritgwa[i] = P(PCRITGWA, i);
    h.gamma[i] = P(GAMRUN, i);
    h.cfa[i] = P(CFA, i);
    h.inv_cfa[i] = safe_inv(P(CFA, i));
    h.smax[i] = r->smax[i];
    h.inv_smax[i] = safe_inv((double)r->smax[i]);
    h.fg[i] = r->gw_factor[i];
    h.rgmax[i] = r->rg_max[i] / 100.;
    h.built_up[i] = r->built_up[i];
    h.t_gradnt[i] = P(T_GRADNT, i);
    const int16_t *el = r->elev + (size_t)i * (B + 1);
    h.elev0[i] = el[0];
    for (int b = 0; b < B; ++b) {
      h.band_dt[(size_t)i * B + b] = (el[b + 1] - el[0]) * P(T_GRADNT, i);
      h.band_el[(size_t)i * B + b] = el[b + 1];
      h.snow_thr[(size_t)i * B + b] = snowfall_threshold(h.band_dt[(size_t)i * B + b], P(T_SNOWFZ, i));
    }
    h.t_gradnt64[i] = P(T_GRADNT, i);
    h.t_snowfz64[i] = P(T_SNOWFZ, i);
    const double kg = P(GWOUTF, i);
    h.gw_e[i] = exp(-1. * kg);
    h.gw_ik[i] = 1. / kg;
    h.gw_ome[i] = 1. - exp(-1. * kg);
    const double ks = P(SWOUTF, i);
    h.sw_k[i] = ks;
    h.sw_e[i] = exp(-1. * ks);
    h.sw_ik[i] = 1. / ks;
    h.sw_ome[i] = 1. - exp(-1. * ks);
    h.evx[i] = P(EVAREDEX, i) * 3.32193;
    const double lakeDepth = P(LAK_D, i) * 0.001, wetlDepth = P(WET_D, i) * 0.001;
    h.ll100[i] = r->loc_lake[i] / 100.;
    h.maxs_ll[i] = ((r->loc_lake[i]) / 100.) * ar * lakeDepth;
    h.inv_maxs_ll[i] = safe_inv(h.maxs_ll[i]);
    h.lw100[i] = r->loc_wetl[i] / 100.;
    h.maxs_lw[i] = ((r->loc_wetl[i]) / 100.) * ar * wetlDepth;
    h.inv_maxs_lw[i] = safe_inv(h.maxs_lw[i]);
    h.la6[i] = r->lake_area[i] / 1000000.;
    h.maxs_gl[i] = (r->lake_area[i]) * lakeDepth;
    h.inv_maxs_gl[i] = safe_inv(h.maxs_gl[i]);
    h.ra6[i] = r->res_area[i] / 1000000.;
    h.rcap[i] = r->stor_cap[i];
    h.rcap01[i] = r->stor_cap[i] * 0.1;
    if (r->res_area[i] > 0.) {
      h.c_ratio[i] = r->stor_cap[i] / (r->mean_outflow[i] * 31536000. / 1000000000.);
      h.c4[i] = (4. * h.c_ratio[i] * h.c_ratio[i]);
      h.one_m_c4[i] = (1.0 - ((4. * h.c_ratio[i] * h.c_ratio[i])));
      // without water use the month's demand is 0 (routing.cpp:2970-2994)
      h.prov_rel[i] = provisional_release(r->res_type[i], r->mean_outflow[i], r->mean_demand[i], 0.0);
    }
    h.start_month[i] = r->start_month[i];
    h.gw100[i] = r->glo_wetl[i] / 100.;
    h.maxs_gw[i] = ((r->glo_wetl[i]) / 100.) * ar * wetlDepth;
    h.inv_maxs_gw[i] = safe_inv(h.maxs_gw[i]);
    double bf = r->bankfull[i];                       // routing.cpp:488-495
    if (bf < 0.05) bf = 0.05;
    h.bw[i] = 2.71 * pow(bf, 0.557) - 2.0 * 2.0 * (0.349 * pow(bf, 0.341));
    h.inv_mr[i] = 1. / (P(RIVRGH, i) * r->roughness[i]);
    h.sqrt_slope[i] = pow(r->river_slope[i], 0.5);
    h.rlen[i] = r->river_length[i];
    {   // fractional routing: catchment of the water bodies, 20 x their initial area (routing.cpp:759, 1899-1903)
      double fc = (r->loc_lake[i] / 100. + r->loc_wetl[i] / 100. + r->glo_wetl[i] / 100.) * 20.;
      h.fcatch[i] = fc > 1. ? 1. : fc;
    }
    h.inv_len[i] = 1. / r->river_length[i];
    auto it = std::find(lats.begin(), lats.end(), r->lat_deg[i]);
    if (it == lats.end()) { lats.push_back(r->lat_deg[i]); h.ext_row[i] = (int32_t)lats.size() - 1; }
    else h.ext_row[i] = (int32_t)(it - lats.begin());
  }
  for (int k = 0; k < opt->nstation; ++k) {
    const int cidx = opt->stations[k];
    if (cidx < 0 || cidx >= n) return WG_ERR_INVALID;
    h.station[cidx] = k;
  }
  if (opt->model && opt->model->statcorr_opt == 1) {   // G_statCorrFact = P_CFS (integrateWGHM.cpp:364)
    h.statcorr.resize(n);
    for (int i = 0; i < n; ++i) h.statcorr[i] = P(CFS, i);
  }
  h.nrow = (int)lats.size();
  h.ext.resize((size_t)365 * h.nrow);
  h.inv_s0.resize((size_t)365 * h.nrow);
  for (int d = 1; d <= 365; ++d)
    for (int k = 0; k < h.nrow; ++k) {
      const double e = calc_ext_rad((short)d, lats[k]);
      h.ext[(size_t)(d - 1) * h.nrow + k] = e;
      h.inv_s0[(size_t)(d - 1) * h.nrow + k] = safe_inv((0.25 + 0.5) * e);
    }
  st = ctx->precision == 0 ? upload_cells(ctx.get(), h, ctx->cd, r->default_velocity, r->river_velo_opt)
                           : upload_cells(ctx.get(), h, ctx->cf, r->default_velocity, r->river_velo_opt);
  ctx->d_cell_of_slot = (int32_t *)upload_raw<int32_t>(ctx.get(), ctx->topo.cell_of_slot, st);
  if (st != WG_OK) return st;

  // ----- dynamic buffers
  st = ctx->precision == 0 ? alloc_state(ctx.get(), ctx->sd, ctx->vd) : alloc_state(ctx.get(), ctx->sf, ctx->vf);
  if (st != WG_OK) return st;
  const size_t N = ctx->nstate();
  {
    // ring of vertical outputs: as many days as fit in 8 GB or an eighth of the free
    // device memory, whichever is less; at least 8, at most max_days
    const size_t elem = ctx->precision == 0 ? sizeof(double) : sizeof(float);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = (size_t)16 << 30;
    // (ensembles: 24 GB, so that the ring holds two chunks of the stream overlap)
    const size_t ring_bytes = std::min<size_t>((size_t)(ctx->members > 1 ? 24 : 8) << 30, free_b / 8);
    const size_t budget = opt->ring_days > 0 ? (size_t)opt->ring_days : ring_bytes / (2 * elem * N);
    const int ring = (int)std::max<size_t>(std::max(8, 2 * ctx->days_per_step),
                                           std::min<size_t>(budget, (size_t)ctx->max_days));
    ctx->rd.days_per_step = ctx->rf.days_per_step = ctx->days_per_step;
    if (ctx->precision == 0) {
      ctx->rd.ring_days = ring;
      ctx->rd.rs = ctx->alloc<double>((size_t)ring * N);
      ctx->rd.gwr = ctx->alloc<double>((size_t)ring * N);
      if (!ctx->rd.gwr) return WG_ERR_NOMEM;
      if (opt->water_temp) {   // the river's open-water terms of the cells run ahead
        ctx->rd.owp = ctx->alloc<double>((size_t)ring * N);
        ctx->rd.owpet = ctx->alloc<double>((size_t)ring * N);
        if (!ctx->rd.owpet) return WG_ERR_NOMEM;
      }
    } else {
      ctx->rf.ring_days = ring;
      ctx->rf.rs = ctx->alloc<float>((size_t)ring * N);
      ctx->rf.gwr = ctx->alloc<float>((size_t)ring * N);
      if (!ctx->rf.gwr) return WG_ERR_NOMEM;
    }
  }
  float *fb = ctx->alloc<float>((size_t)3 * ctx->max_days * n);
  ctx->forcing.prec = fb;
  ctx->forcing.temp = fb ? fb + (size_t)ctx->max_days * n : nullptr;
  ctx->forcing.swrad = fb ? fb + (size_t)2 * ctx->max_days * n : nullptr;
  ctx->forcing.max_days = ctx->max_days;
  ctx->staging_days = std::min(ctx->max_days, 32);
  ctx->staging = ctx->alloc<float>((size_t)ctx->staging_days * n);
  ctx->outq = ctx->alloc<double>((size_t)2 * ctx->days_per_step * N);   // two steps of days
  ctx->qst = ctx->alloc<double>((size_t)ctx->max_days * std::max(1, ctx->nstation) * ctx->members);
  ctx->balance.enabled = opt->record_balance ? 1 : 0;
  ctx->balance.acc = ctx->alloc<double>(ctx->balance.enabled ? (size_t)WG_BALANCE_ARRAYS * N : 1);
  ctx->vol0 = ctx->alloc<double>(N);
  ctx->partial = ctx->alloc<double>((size_t)8 * ((N + 255) / 256));
  ctx->sync.counter = ctx->alloc<unsigned int>(1);
  ctx->sync.error = ctx->alloc<int>(1);
  ctx->va_next = ctx->alloc<unsigned int>(1);
  float *mf = ctx->alloc<float>((size_t)2 * ctx->members);
  if (!fb || !ctx->staging || !ctx->outq || !ctx->qst || !ctx->balance.acc || !ctx->vol0 || !ctx->partial ||
      !ctx->sync.counter || !ctx->sync.error || !ctx->va_next || !mf)
    return WG_ERR_NOMEM;
  {
    std::vector<float> fac(2 * ctx->members, 1.0f);
    for (int k = 0; k < ctx->members; ++k) {
      if (opt->member_prec_factor) fac[k] = opt->member_prec_factor[k];
      if (opt->member_gamma_factor) fac[ctx->members + k] = opt->member_gamma_factor[k];
    }
    cudaMemcpy(mf, fac.data(), fac.size() * sizeof(float), cudaMemcpyHostToDevice);
    ctx->mem.members = ctx->members;
    ctx->mem.prec_factor = mf;
    ctx->mem.gamma_factor = mf + ctx->members;
  }
  cudaMemset(ctx->sync.error, 0, sizeof(int));
  cudaMemset(ctx->outq, 0, (size_t)2 * ctx->days_per_step * N * sizeof(double));
  cudaMemset(ctx->qst, 0, (size_t)ctx->max_days * std::max(1, ctx->nstation) * ctx->members * sizeof(double));

  // ----- start-of-run state, cell order (the reference's set-up sequence; see file header)
  std::vector<double> zeros(n, 0.), ones(n, 1.), kr(n, 0.1), loclake(n), locwetl(n), glolake(n), glowetl(n),
      resv(n), laf(n), fswb(n), bands((size_t)n * B, 0.), river(n, 0.), rfres(n, 0.);
  std::vector<int32_t> izero(n, 0);
  for (int i = 0; i < n; ++i) {
    const double ar = r->area_km2[i];
    const double lakeDepth = P(LAK_D, i) * 0.001, wetlDepth = P(WET_D, i) * 0.001;
    loclake[i] = (r->loc_lake[i] / 100.) * ar * lakeDepth;
    locwetl[i] = (r->loc_wetl[i] / 100.) * ar * wetlDepth;
    glolake[i] = r->lake_area[i] * lakeDepth;
    glowetl[i] = (r->glo_wetl[i] / 100.) * ar * wetlDepth;
    resv[i] = (r->res_area[i] > 0.) ? r->stor_cap[i] : 0.;
    fswb[i] = r->loc_lake[i] / 100. + r->loc_wetl[i] / 100. + r->glo_wetl[i] / 100.;
    double l = (cont_share(r, i) - (r->glo_lake[i] + r->glo_wetl[i] + r->loc_lake[i] + r->loc_wetl[i] + r->glo_res[i]));
    laf[i] = l < 0. ? 0. : l;
    if (r->river_velo_opt == 2) {   // setStoragesToZero starts from G_riverStorageMax (routing.cpp:807-812)
      double bf = r->bankfull[i] < 0.05 ? 0.05 : r->bankfull[i];
      double wbf = 2.71 * pow(bf, 0.557), dbf = 0.349 * pow(bf, 0.341);
      double bwi = wbf - 2.0 * 2.0 * dbf;
      river[i] = r->river_length[i] * 0.5 * dbf / 1000. * (bwi / 1000. + wbf / 1000.);
    }
  }
  wg_state_view init{};
  init.canopy = zeros.data(); init.soil = zeros.data(); init.snow = zeros.data(); init.snow_band = bands.data();
  init.lai_days = izero.data(); init.lai_status = izero.data(); init.lai_precsum = zeros.data();
  init.gw = zeros.data(); init.river = river.data(); init.loclake = loclake.data(); init.locwetl = locwetl.data();
  init.glolake = glolake.data(); init.glowetl = glowetl.data(); init.res = resv.data();
  init.rf_loclake = ones.data(); init.rf_locwetl = ones.data(); init.rf_glolake = ones.data();
  init.rf_glowetl = ones.data(); init.rf_res = rfres.data(); init.k_release = kr.data();
  init.laf = laf.data(); init.laf_prev = zeros.data(); init.fswb_next = fswb.data(); init.laf_started = izero.data();
  st = ctx->precision == 0 ? broadcast_state(ctx.get(), ctx->sd, &init) : broadcast_state(ctx.get(), ctx->sf, &init);
  if (st != WG_OK) return st;
  if (opt->water_temp) {
    st = setup_water_temp(ctx.get(), r);
    if (st != WG_OK) return st;
  }
  if (opt->water_use) {
    st = setup_water_use(ctx.get(), r);
    if (st != WG_OK) return st;
    ctx->wu.delayed = opt->water_use == 2;
  }
  const bool ens = ctx->members > 1;
  if (ctx->layout.idle_warp >= 0) ctx->threads = ctx->layout.threads;
  const int th = ctx->threads;
  const int need = ctx->layout.idle_warp >= 0 ? ctx->layout.blocks
                                              : (int)std::min<size_t>((N + th - 1) / th, (size_t)1 << 30);
  if (ctx->precision == 0) {
    ctx->blocks_fused = std::min(pipeline_max_blocks<double>(true, ens, th), need);
    ctx->blocks_route = std::min(pipeline_max_blocks<double>(false, ens, th), need);
  } else {
    ctx->blocks_fused = std::min(pipeline_max_blocks<float>(true, ens, th), need);
    ctx->blocks_route = std::min(pipeline_max_blocks<float>(false, ens, th), need);
  }
  if (ctx->blocks_fused <= 0 || ctx->blocks_route <= 0) {
    ctx->err = "cooperative launch not possible";
    return WG_ERR_DEVICE;
  }
  if (ens) {   // the second stream of the ensemble's stream overlap (off until switched on or tuned)
    if (cudaStreamCreateWithFlags(&ctx->va_stream, cudaStreamNonBlocking) != cudaSuccess) return WG_ERR_CUDA;
    for (cudaEvent_t *e : {&ctx->ev_fork, &ctx->ev_va, &ctx->ev_pipe[0], &ctx->ev_pipe[1]})
      if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return WG_ERR_CUDA;
    ctx->blocks_va = std::min(vertical_ahead_max_blocks<float>(true, th), need);
  }
  if (ctx->layout.idle_warp >= 0) {
    st = setup_step_flags(ctx.get());
    if (st != WG_OK) return st;
  }
  st = wg_reset_balance(ctx.get());
  if (st != WG_OK) return st;
  *out = ctx.release();
  return WG_OK;
}

wg_status wg_destroy(wg_ctx *ctx) {
  if (!ctx) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  delete ctx;
  return WG_OK;
}

wg_status wg_set_state(wg_ctx *ctx, const wg_state_view *v) {
  if (!ctx || !v) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  return state_io(ctx, v, 0, true);
}

wg_status wg_get_state(wg_ctx *ctx, wg_state_view *v) {
  if (!ctx || !v) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  return state_io(ctx, v, 0, false);
}

wg_status wg_set_member_state(wg_ctx *ctx, int32_t member, const wg_state_view *v) {
  if (!ctx || !v) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  return state_io(ctx, v, member, true);
}

wg_status wg_get_member_state(wg_ctx *ctx, int32_t member, wg_state_view *v) {
  if (!ctx || !v) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  return state_io(ctx, v, member, false);
}

static wg_status upload_forcing_on(wg_ctx *ctx, cudaStream_t st, float *staging, int32_t day0, int32_t ndays,
                                   const float *prec, const float *temp, const float *swrad) {
  if (!ctx || (!prec && !temp && !swrad) || day0 < 0 || ndays < 0 || day0 + ndays > ctx->max_days)
    return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  const int n = ctx->n;
  const float *src[3] = {prec, temp, swrad};
  float *dst[3] = {(float *)ctx->forcing.prec, (float *)ctx->forcing.temp, (float *)ctx->forcing.swrad};
  for (int d = 0; d < ndays; d += ctx->staging_days) {
    const int nd = std::min(ctx->staging_days, ndays - d);
    for (int k = 0; k < 3; ++k) {
      if (!src[k]) continue;   // the slots keep this variable's values
      cudaError_t e = cudaMemcpyAsync(staging, src[k] + (size_t)d * n, (size_t)nd * n * sizeof(float),
                                      cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess)
        e = launch_gather_forcing(staging, dst[k] + (size_t)(day0 + d) * n, ctx->d_cell_of_slot, n, nd, st);
      ctx->launches++;
      if (e != cudaSuccess) return cuda_fail(ctx, e, "upload_forcing");
    }
  }
  return WG_OK;
}

wg_status wg_upload_forcing(wg_ctx *ctx, int32_t day0, int32_t ndays, const float *prec, const float *temp,
                            const float *swrad) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  join_uploads(ctx);   // after the overlapped uploads, in the order of the calls
  return upload_forcing_on(ctx, ctx->stream, ctx->staging, day0, ndays, prec, temp, swrad);
}

}  // extern "C"

// cell-major forcing [ncell][nd_file] to the device as it is; transpose (and the
// byte swap of big-endian file bytes) there
static wg_status upload_cell_major(wg_ctx *ctx, int32_t day0, int32_t nd_file, int32_t d_first, int32_t ndays,
                                   const void *prec, const void *temp, const void *swrad, int32_t overlap,
                                   bool big_endian) {
  if (!ctx || !prec || !temp || !swrad || nd_file <= 0 || d_first < 0 || ndays < 0 || d_first + ndays > nd_file ||
      day0 < 0 || day0 + ndays > ctx->max_days)
    return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  cudaSetDevice(ctx->device);
  const int which = overlap ? 1 : 0;
  const size_t per = (size_t)ctx->n * nd_file;
  if (ctx->unf_cap[which] < per) {
    ctx->unf_raw[which] = ctx->alloc<uint32_t>(per);   // freed with the context
    if (!ctx->unf_raw[which]) return WG_ERR_NOMEM;
    ctx->unf_cap[which] = per;
  }
  if (!overlap) join_uploads(ctx);
  cudaStream_t st = overlap ? ctx->copy_stream : ctx->stream;
  const void *src[3] = {prec, temp, swrad};
  float *dst[3] = {(float *)ctx->forcing.prec, (float *)ctx->forcing.temp, (float *)ctx->forcing.swrad};
  for (int k = 0; k < 3; ++k) {
    cudaError_t e = cudaMemcpyAsync(ctx->unf_raw[which], src[k], per * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = launch_unf_forcing(ctx->unf_raw[which], dst[k] + (size_t)day0 * ctx->n, ctx->d_cell_of_slot, ctx->n,
                             nd_file, d_first, ndays, st, big_endian);
    ctx->launches++;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "upload_forcing_unf");
  }
  if (overlap) {
    cudaError_t e = cudaEventRecord(ctx->upload_done, ctx->copy_stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "upload_forcing_unf");
    ctx->upload_pending = true;
  }
  return WG_OK;
}

extern "C" {

wg_status wg_upload_forcing_unf(wg_ctx *ctx, int32_t day0, int32_t nd_file, int32_t d_first, int32_t ndays,
                                const void *prec, const void *temp, const void *swrad, int32_t overlap) {
  return upload_cell_major(ctx, day0, nd_file, d_first, ndays, prec, temp, swrad, overlap, true);
}

wg_status wg_upload_forcing_cells(wg_ctx *ctx, int32_t day0, int32_t nd_file, int32_t d_first, int32_t ndays,
                                  const float *prec, const float *temp, const float *swrad, int32_t overlap) {
  return upload_cell_major(ctx, day0, nd_file, d_first, ndays, prec, temp, swrad, overlap, false);
}

wg_status wg_math_eval(int32_t device, int32_t fn, const double *x, const double *y, int64_t n, double *out) {
  if (!x || !out || n < 0 || fn < 0 || fn > 4 || (fn == 2 && !y)) return WG_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return WG_ERR_DEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return WG_ERR_DEVICE;
  double e2[64], lf[129], inv[129];
  fill_fastmath_tables(e2, lf, inv);
  cudaError_t e = upload_fastmath_tables(e2, lf, inv);
  const size_t bytes = (size_t)std::max<int64_t>(n, 1) * sizeof(double);
  double *d = nullptr;
  if (e == cudaSuccess) e = cudaMalloc((void **)&d, 3 * bytes);
  if (e == cudaSuccess) e = cudaMemcpy(d, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && fn == 2) e = cudaMemcpy(d + n, y, (size_t)n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_math_eval(fn, d, d + n, d + 2 * n, (size_t)n, 0);
  if (e == cudaSuccess) e = cudaMemcpy(out, d + 2 * n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  return e == cudaSuccess ? WG_OK : WG_ERR_CUDA;
}

wg_status wg_upload_longwave(wg_ctx *ctx, int32_t day0, int32_t ndays, const float *longwave) {
  if (!ctx || !longwave || day0 < 0 || ndays < 0 || day0 + ndays > ctx->max_days) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!ctx->wt.enabled) return WG_ERR_UNSUPPORTED;
  cudaSetDevice(ctx->device);
  join_uploads(ctx);
  const int n = ctx->n;
  for (int d = 0; d < ndays; d += ctx->staging_days) {
    const int nd = std::min(ctx->staging_days, ndays - d);
    cudaError_t e = cudaMemcpyAsync(ctx->staging, longwave + (size_t)d * n, (size_t)nd * n * sizeof(float),
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
      e = launch_gather_forcing(ctx->staging, (float *)ctx->wt.lw + (size_t)(day0 + d) * n, ctx->d_cell_of_slot, n, nd,
                                ctx->stream);
    ctx->launches++;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "upload_longwave");
  }
  return WG_OK;
}

wg_status wg_set_water_temp_inputs(wg_ctx *ctx, const float *gw_temp, const double *river_length_check) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!ctx->wt.enabled) return WG_ERR_UNSUPPORTED;
  cudaSetDevice(ctx->device);
  wg_status st = wg_synchronize(ctx);
  if (st == WG_OK && gw_temp) st = to_slots(ctx, gw_temp, (float *)ctx->wt.gwt);
  if (st == WG_OK && river_length_check) st = to_slots(ctx, river_length_check, (double *)ctx->wt.len_check);
  return st;
}

// [6][ncell] cell order <-> [6][N] slot order
static wg_status water_temp_io(wg_ctx *ctx, double *temp, double *ice, const double *temp_in, const double *ice_in) {
  if (!ctx) return WG_ERR_INVALID;
  if (!ctx->wt.enabled) return WG_ERR_UNSUPPORTED;
  cudaSetDevice(ctx->device);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  const int n = ctx->n;
  std::vector<double> buf((size_t)6 * n);
  double *dev[2] = {ctx->wt.temp, ctx->wt.ice};
  double *out[2] = {temp, ice};
  const double *in[2] = {temp_in, ice_in};
  for (int k = 0; k < 2; ++k) {
    cudaError_t e = cudaSuccess;
    if (in[k]) {
      for (int j = 0; j < 6; ++j)
        for (int s = 0; s < n; ++s) buf[(size_t)j * n + s] = in[k][(size_t)j * n + ctx->topo.cell_of_slot[s]];
      e = cudaMemcpy(dev[k], buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice);
    } else if (out[k]) {
      e = cudaMemcpy(buf.data(), dev[k], buf.size() * sizeof(double), cudaMemcpyDeviceToHost);
      for (int j = 0; j < 6 && e == cudaSuccess; ++j)
        for (int s = 0; s < n; ++s) out[k][(size_t)j * n + ctx->topo.cell_of_slot[s]] = buf[(size_t)j * n + s];
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "water temperature");
  }
  return WG_OK;
}

wg_status wg_get_water_temp(wg_ctx *ctx, double *temp, double *ice) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!temp && !ice) return WG_ERR_INVALID;
  return water_temp_io(ctx, temp, ice, nullptr, nullptr);
}

wg_status wg_set_water_temp(wg_ctx *ctx, const double *temp, const double *ice) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!temp && !ice) return WG_ERR_INVALID;
  return water_temp_io(ctx, nullptr, nullptr, temp, ice);
}

wg_status wg_get_river_temp(wg_ctx *ctx, int32_t day0, int32_t ndays, double *out) {
  if (!ctx || !out || day0 < 0 || ndays < 0 || day0 + ndays > ctx->max_days) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!ctx->wt.enabled) return WG_ERR_UNSUPPORTED;
  cudaSetDevice(ctx->device);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  const size_t k = (size_t)std::max(1, ctx->nstation);
  return cuda_fail(ctx,
                   cudaMemcpy(out, ctx->wt.qst_t + (size_t)day0 * k, (size_t)ndays * ctx->nstation * sizeof(double),
                              cudaMemcpyDeviceToHost),
                   "get_river_temp");
}

wg_status wg_upload_water_use(wg_ctx *ctx, int32_t fday0, int32_t ndays, int32_t doy0, const double *nus_m3,
                              const double *nug_m3, const double *irrig_withdrawal_sw_m3,
                              const double *irrig_consumptive_sw_m3) {
  if (!ctx || !nus_m3 || !nug_m3 || !irrig_withdrawal_sw_m3 || !irrig_consumptive_sw_m3) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (fday0 < 0 || ndays < 1 || fday0 + ndays > ctx->max_days || doy0 < 1 || doy0 + ndays - 1 > 365)
    return WG_ERR_INVALID;
  if (!ctx->wu.enabled) return WG_ERR_UNSUPPORTED;
  cudaSetDevice(ctx->device);
  wg_status st = wg_synchronize(ctx);   // no launch may still read the block this call fills
  if (st != WG_OK) return st;
  static const int days_in_month[12] = {31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31};   // routing.cpp:107
  const int n = ctx->n;
  const size_t N = (size_t)n;   // tables per cell
  const int F = wg::WU_FIELDS;
  const int b = 1 + (ctx->wu_next++ % (ctx->wu_blocks - 1));
  const size_t block = (size_t)12 * F * N;
  std::vector<double> buf(block, 0.);
  const double *src[4] = {nus_m3, nug_m3, irrig_withdrawal_sw_m3, irrig_consumptive_sw_m3};
  std::vector<double> agg(ctx->glwd.on ? n : 0);
  for (int m = 0; m < 12; ++m) {
    const double per_day = 1000000000. * (double)days_in_month[m];   // dailyNUInit, routing.cpp:966-975
    for (int k = 0; k < 4; ++k) {
      double *row = buf.data() + ((size_t)m * F + k) * N;
      const double *in = src[k] + (size_t)m * n;
      for (int s = 0; s < n; ++s) row[s] = in[ctx->topo.cell_of_slot[s]] / per_day;
    }
    if (ctx->glwd.on) {   // NUs aggregated over the GLWD units, then per day (routing.cpp:926-975)
      glwd_aggregate(ctx->glwd, nus_m3 + (size_t)m * n, agg.data(), n);
      double *row = buf.data() + ((size_t)m * F + 5) * N;
      for (int s = 0; s < n; ++s) row[s] = agg[ctx->topo.cell_of_slot[s]] / per_day;
    }
    double *prov = buf.data() + ((size_t)m * F + 4) * N;
    std::copy(ctx->wu_prov0.begin(), ctx->wu_prov0.end(), prov);
    for (const auto &res : ctx->wu_res) {   // routing.cpp:2970-2994
      const double dailyUse = buf[((size_t)m * F + 0) * N + res.slot];
      double monthlyUse = dailyUse * days_in_month[m];
      monthlyUse = monthlyUse * 1000000000. / (days_in_month[m] * 86400.);
      prov[res.slot] = provisional_release(res.type, res.mean_outflow, res.mean_demand, monthlyUse);
    }
  }
  std::vector<int32_t> rows(ndays);
  for (int d = 0; d < ndays; ++d) {
    const int doy = doy0 + d;
    int mo = 0;
    for (int k = 1; k < 12; ++k) mo += (doy >= kFirstDayInMonth[k]) ? 1 : 0;
    rows[d] = 12 * b + mo;
  }
  cudaError_t e = cudaMemcpy((void *)(ctx->wu.tab + (size_t)b * block), buf.data(), block * sizeof(double),
                             cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy((void *)(ctx->wu.row_of_fday + fday0), rows.data(), (size_t)ndays * sizeof(int32_t),
                   cudaMemcpyHostToDevice);
  return cuda_fail(ctx, e, "upload_water_use");
}

wg_status wg_set_water_use_inputs(wg_ctx *ctx, const double *frac_return_gw_irrig) {
  if (!ctx || !frac_return_gw_irrig) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!ctx->wu.enabled) return WG_ERR_UNSUPPORTED;
  cudaSetDevice(ctx->device);
  wg_status st = wg_synchronize(ctx);
  if (st == WG_OK) st = to_slots(ctx, frac_return_gw_irrig, (double *)ctx->wu.frgi);   // per cell
  return st;
}

// [WG_WU_NSTATE][ncell] cell order <-> [WG_WU_NSTATE][N] slot order
static wg_status water_use_io(wg_ctx *ctx, double *out, const double *in) {
  if (!ctx || (!out && !in)) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!ctx->wu.enabled) return WG_ERR_UNSUPPORTED;
  cudaSetDevice(ctx->device);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  const int n = ctx->n, K = wg::WU_NSTATE, M = ctx->members;
  const size_t N = ctx->nstate();
  std::vector<double> buf((size_t)K * N);
  cudaError_t e;
  if (in) {
    for (int j = 0; j < K; ++j)
      for (int s = 0; s < n; ++s)
        for (int mm = 0; mm < M; ++mm)
          buf[(size_t)j * N + (size_t)s * M + mm] = in[(size_t)j * N + (size_t)ctx->topo.cell_of_slot[s] * M + mm];
    e = cudaMemcpy(ctx->wu.st, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice);
  } else {
    e = cudaMemcpy(buf.data(), ctx->wu.st, buf.size() * sizeof(double), cudaMemcpyDeviceToHost);
    for (int j = 0; j < K && e == cudaSuccess; ++j)
      for (int s = 0; s < n; ++s)
        for (int mm = 0; mm < M; ++mm)
          out[(size_t)j * N + (size_t)ctx->topo.cell_of_slot[s] * M + mm] = buf[(size_t)j * N + (size_t)s * M + mm];
  }
  return cuda_fail(ctx, e, "water use");
}

wg_status wg_get_water_use(wg_ctx *ctx, double *out) { return out ? water_use_io(ctx, out, nullptr) : WG_ERR_INVALID; }
wg_status wg_set_water_use(wg_ctx *ctx, const double *in) { return in ? water_use_io(ctx, nullptr, in) : WG_ERR_INVALID; }

int64_t wg_read_unf(const char *path, void *dst, int64_t bytes) {
  if (!path || !dst || bytes < 0) return -1;
  FILE *f = std::fopen(path, "rb");
  if (!f) return -1;
  const size_t got = std::fread(dst, 1, (size_t)bytes, f);
  std::fclose(f);
  return (int64_t)got;
}

wg_status wg_upload_forcing_async(wg_ctx *ctx, int32_t day0, int32_t ndays, const float *prec, const float *temp,
                                  const float *swrad) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  // its own staging buffer: the copy stream is not ordered after uploads on the
  // context's stream
  if (!ctx->staging_async) ctx->staging_async = ctx->alloc<float>((size_t)ctx->staging_days * ctx->n);
  if (!ctx->staging_async) return WG_ERR_NOMEM;
  wg_status st = upload_forcing_on(ctx, ctx->copy_stream, ctx->staging_async, day0, ndays, prec, temp, swrad);
  if (st != WG_OK) return st;
  cudaError_t e = cudaEventRecord(ctx->upload_done, ctx->copy_stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "upload_forcing_async");
  ctx->upload_pending = true;
  return WG_OK;
}

wg_status wg_step_vertical(wg_ctx *ctx, int32_t doy, int32_t fday) {
  if (!ctx || doy < 1 || doy > 365 || fday < 0 || fday >= ctx->max_days) return WG_ERR_INVALID;
  if (ctx->members != 1) return WG_ERR_UNSUPPORTED;
  auto &q = ctx->defer;
  if (!q.on) return vertical_now(ctx, doy, fday);
  if (q.vpending) WG_FLUSH(ctx);   // two vertical calls in a row: the first runs alone
  q.vpending = true;
  q.vdoy = doy;
  q.vfday = fday;
  return WG_OK;
}

wg_status wg_step_routing(wg_ctx *ctx, int32_t doy, int32_t oday) {
  if (!ctx || doy < 1 || doy > 365 || oday < 0 || oday >= ctx->max_days) return WG_ERR_INVALID;
  if (ctx->members != 1) return WG_ERR_UNSUPPORTED;
  auto &q = ctx->defer;
  if (!q.on) return routing_now(ctx, doy, oday);
  if (!q.vpending || q.vdoy != doy) {   // not the pair of a queued vertical call: in order, now
    WG_FLUSH(ctx);
    return routing_now(ctx, doy, oday);
  }
  q.vpending = false;   // this day's vertical call is consumed by the queue
  const bool follows = q.ndays > 0 && doy == (q.doy0 - 1 + q.ndays) % 365 + 1 && q.vfday == q.fday0 + q.ndays &&
                       oday == q.oday0 + q.ndays;
  if (!follows) {
    if (q.ndays > 0) {   // the queued run first, then this day starts a new one
      wg_status st = flush_deferred(ctx);
      if (st != WG_OK) return st;
    }
    q.doy0 = doy;
    q.fday0 = q.vfday;
    q.oday0 = oday;
    q.ndays = 0;
  }
  q.ndays++;
  return WG_OK;
}

}  // extern "C"

// Steps [t_b, t_e) of the day-pipelined wavefront of a run of ndays days, in
// chunks: the vertical balance of the cells without water bodies runs ahead of
// each chunk's routing wavefront (one cooperative launch).  Without the overlap it
// is one launch before each chunk; with it, the first chunk's runs alone and every
// wavefront launch carries warps that compute the next chunk's, so the FP64 pipe
// has their work while the routing warps wait on loads and step barriers.  Every
// call ends with the vertical state exactly at step t_e either way.
template <class R>
static wg_status run_steps_impl(wg_ctx *ctx, const DevCellsT<R> &c, const DevStateT<R> &s, const DevVertT<R> &v,
                                const DevRingT<R> &ring, int doy0, int fday0, int oday0, int ndays, int t_b,
                                int t_e) {
  const bool ov = ctx->overlap();
  const int chunk = ctx->eff_chunk();
  if (ctx->ens_overlap && ctx->members > 1 && ctx->va_stream) {
    // the next chunk's vertical balance on the second stream, beside this chunk's
    // wavefront launch: the vertical balance of chunk k+1 writes ring slots that
    // the wavefront launch of chunk k-1 read (the ring holds two chunks), and the
    // wavefront launch of chunk k waits for chunk k's vertical balance; the call
    // ends with both streams joined on the context's stream
    auto va = [&](int a, int b) {
      ctx->launches++;
      return launch_vertical_ahead(c, s, ctx->forcing, ctx->mem, ctx->balance, ring, doy0, fday0, ndays, a, b,
                                   ctx->blocks_va, ctx->threads, ctx->va_stream, ctx->mon, oday0);
    };
    cudaError_t e = cudaEventRecord(ctx->ev_fork, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->va_stream, ctx->ev_fork, 0);
    if (e == cudaSuccess) e = va(t_b, std::min(t_e, t_b + chunk));
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_va, ctx->va_stream);
    int k = 0;
    for (int a = t_b; a < t_e && e == cudaSuccess; a += chunk, ++k) {
      const int b = std::min(t_e, a + chunk);
      e = cudaStreamWaitEvent(ctx->stream, ctx->ev_va, 0);
      if (e == cudaSuccess)
        e = launch_pipeline(true, c, s, v, ctx->forcing, ctx->mem, ctx->balance, ring, ctx->sync, ctx->outq, ctx->qst,
                            doy0, fday0, oday0, ndays, a, b, ctx->blocks_fused, ctx->threads, ctx->layout, ctx->mon,
                            DevVaWork{}, ctx->wt, ctx->wu, ctx->stream);
      ctx->launches++;
      if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_pipe[k & 1], ctx->stream);
      if (e == cudaSuccess && b < t_e) {
        if (k >= 1) e = cudaStreamWaitEvent(ctx->va_stream, ctx->ev_pipe[(k - 1) & 1], 0);
        if (e == cudaSuccess) e = va(b, std::min(t_e, b + chunk));
        if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_va, ctx->va_stream);
      }
    }
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_va, ctx->va_stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->ev_va, 0);
    return e == cudaSuccess ? WG_OK : cuda_fail(ctx, e, "run_steps");
  }
  DevVaWork vw{};
  vw.next = ctx->va_next;
  vw.nitems = (int)((ctx->nstate() + 31) / 32);
  for (int a = t_b; a < t_e; a += chunk) {
    const int b = std::min(t_e, a + chunk);
    cudaEvent_t *ev = ctx->timing ? ctx->timing_events() : nullptr;
    if (ev) cudaEventRecord(ev[0], ctx->stream);
    cudaError_t e = cudaSuccess;
    if (!ov || a == t_b) {
      e = launch_vertical_ahead(c, s, ctx->forcing, ctx->mem, ctx->balance, ring, doy0, fday0, ndays, a, b,
                                ctx->blocks_fused, ctx->threads, ctx->stream, ctx->mon, oday0);
      ctx->launches++;
    }
    if (ev) cudaEventRecord(ev[1], ctx->stream);
    vw.t_b = b;
    vw.t_e = std::min(t_e, b + chunk);
    vw.warps = (ov && vw.t_e > vw.t_b) ? ctx->layout.va_warps : 0;
    if (e == cudaSuccess)
      e = launch_pipeline(true, c, s, v, ctx->forcing, ctx->mem, ctx->balance, ring, ctx->sync, ctx->outq, ctx->qst,
                          doy0, fday0, oday0, ndays, a, b, ctx->blocks_fused, ctx->threads, ctx->layout, ctx->mon,
                          vw, ctx->wt, ctx->wu, ctx->stream);
    ctx->launches++;
    if (ev) cudaEventRecord(ev[2], ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "run_steps");
  }
  return WG_OK;
}

extern "C" {

}  // extern "C"

// steps [t_begin, t_end) of a run whose station and monthly outputs start at slot oday0
static wg_status run_steps_at(wg_ctx *ctx, int doy0, int fday0, int oday0, int ndays, int t_begin, int t_end) {
  cudaSetDevice(ctx->device);
  join_uploads(ctx);
  return ctx->precision == 0
             ? run_steps_impl(ctx, ctx->cd, ctx->sd, ctx->vd, ctx->rd, doy0, fday0, oday0, ndays, t_begin, t_end)
             : run_steps_impl(ctx, ctx->cf, ctx->sf, ctx->vf, ctx->rf, doy0, fday0, oday0, ndays, t_begin, t_end);
}

static wg_status vertical_now(wg_ctx *ctx, int doy, int fday) {
  // the per-day kernel fills no output grids: wg_set_deferred runs the per-day calls through the wavefront
  if (ctx->mon.vert || ctx->mon.dvert) return WG_ERR_UNSUPPORTED;
  cudaSetDevice(ctx->device);
  join_uploads(ctx);
  ctx->launches++;
  ctx->last_vertical_fday = fday;   // the day's forcing slot, for the water temperature of wg_step_routing
  cudaError_t e = ctx->precision == 0
                      ? launch_vertical(ctx->cd, ctx->sd, ctx->vd, ctx->forcing, doy, fday, ctx->stream)
                      : launch_vertical(ctx->cf, ctx->sf, ctx->vf, ctx->forcing, doy, fday, ctx->stream);
  return cuda_fail(ctx, e, "step_vertical");
}

static wg_status routing_now(wg_ctx *ctx, int doy, int oday) {
  cudaSetDevice(ctx->device);
  join_uploads(ctx);
  ctx->launches++;
  cudaError_t e = ctx->precision == 0
                      ? launch_pipeline(false, ctx->cd, ctx->sd, ctx->vd, ctx->forcing, ctx->mem, ctx->balance,
                                        ctx->rd, ctx->sync, ctx->outq, ctx->qst, doy, ctx->last_vertical_fday, oday, 1,
                                        0, ctx->topo.nlevel, ctx->blocks_route, ctx->threads, ctx->layout, ctx->mon,
                                        DevVaWork{}, ctx->wt, ctx->wu, ctx->stream)
                      : launch_pipeline(false, ctx->cf, ctx->sf, ctx->vf, ctx->forcing, ctx->mem, ctx->balance,
                                        ctx->rf, ctx->sync, ctx->outq, ctx->qst, doy, ctx->last_vertical_fday, oday, 1,
                                        0, ctx->topo.nlevel, ctx->blocks_route, ctx->threads, ctx->layout, ctx->mon,
                                        DevVaWork{}, ctx->wt, ctx->wu, ctx->stream);
  return cuda_fail(ctx, e, "step_routing");
}

// Run what the deferred per-day calls have queued: the consecutive days as one
// day-pipelined run (the same results as their per-day launches), then a
// vertical balance still waiting for its routing call.
wg_status flush_deferred(wg_ctx *ctx) {
  auto &q = ctx->defer;
  wg_status st = WG_OK;
  if (q.ndays > 0) {
    const int nd = q.ndays;
    q.ndays = 0;
    st = run_steps_at(ctx, q.doy0, q.fday0, q.oday0, nd, 0, ctx->total_steps(nd));
    if (st == WG_OK) ctx->last_vertical_fday = q.fday0 + nd - 1;
  }
  if (st == WG_OK && q.vpending) {
    q.vpending = false;
    st = vertical_now(ctx, q.vdoy, q.vfday);
  }
  return st;
}

extern "C" {

wg_status wg_set_deferred(wg_ctx *ctx, int32_t enable) {
  if (!ctx) return WG_ERR_INVALID;
  if (ctx->members != 1) return WG_ERR_UNSUPPORTED;
  wg_status st = flush_deferred(ctx);
  ctx->defer.on = enable != 0;
  return st;
}

wg_status wg_run_steps(wg_ctx *ctx, int32_t doy0, int32_t fday0, int32_t ndays, int32_t t_begin, int32_t t_end) {
  if (!ctx || doy0 < 1 || doy0 > 365 || fday0 < 0 || ndays <= 0 || fday0 + ndays > ctx->max_days) return WG_ERR_INVALID;
  const int total = ctx->total_steps(ndays);
  if (t_begin < 0 || t_end > total || t_begin > t_end) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (t_begin == t_end) return WG_OK;
  return run_steps_at(ctx, doy0, fday0, fday0, ndays, t_begin, t_end);
}

int32_t wg_run_num_steps(const wg_ctx *ctx, int32_t ndays) { return ctx ? ctx->total_steps(ndays) : 0; }

wg_status wg_run_days(wg_ctx *ctx, int32_t doy0, int32_t fday0, int32_t ndays) {
  if (!ctx) return WG_ERR_INVALID;
  return wg_run_steps(ctx, doy0, fday0, ndays, 0, ctx->total_steps(ndays));
}

wg_status wg_synchronize(wg_ctx *ctx) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->copy_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
  int flag = 0;
  e = cudaMemcpy(&flag, ctx->sync.error, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
  if (flag) {
    ctx->err = "grid barrier wait exceeded its iteration limit";
    return WG_ERR_TIMEOUT;
  }
  return WG_OK;
}

wg_status wg_clear_error(wg_ctx *ctx) {
  if (!ctx) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaMemset(ctx->sync.error, 0, sizeof(int));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "clear_error");
  ctx->err.clear();
  return WG_OK;
}

wg_status wg_set_barrier_test(wg_ctx *ctx, int32_t extra_arrivals) {
  if (!ctx || extra_arrivals < 0) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  ctx->sync.extra_arrivals = (uint32_t)extra_arrivals;
  return WG_OK;
}

wg_status wg_get_discharge(wg_ctx *ctx, int32_t day0, int32_t ndays, double *out) {
  if (!ctx || !out || day0 < 0 || ndays < 0 || day0 + ndays > ctx->max_days) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (ctx->nstation == 0 || ndays == 0) return WG_OK;
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  const size_t per_day = (size_t)ctx->nstation * ctx->members;
  return cuda_fail(ctx,
                   cudaMemcpy(out, ctx->qst + (size_t)day0 * per_day, (size_t)ndays * per_day * sizeof(double),
                              cudaMemcpyDeviceToHost),
                   "get_discharge");
}

wg_status wg_get_member_discharge(wg_ctx *ctx, int32_t member, int32_t day0, int32_t ndays, double *out) {
  if (!ctx || !out || member < 0 || member >= ctx->members || day0 < 0 || ndays < 0 ||
      day0 + ndays > ctx->max_days)
    return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (ctx->nstation == 0 || ndays == 0) return WG_OK;
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  const size_t M = ctx->members, rows = (size_t)ndays * ctx->nstation;
  // [day][station][member]: one element of every (day, station) row
  return cuda_fail(ctx,
                   cudaMemcpy2D(out, sizeof(double), ctx->qst + (size_t)day0 * ctx->nstation * M + member,
                                M * sizeof(double), sizeof(double), rows, cudaMemcpyDeviceToHost),
                   "get_member_discharge");
}

wg_status wg_record_daily_storages(wg_ctx *ctx, int32_t enable) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (ctx->members != 1) return WG_ERR_UNSUPPORTED;
  cudaSetDevice(ctx->device);
  if (enable && !ctx->daily_storage_buf) {
    ctx->daily_storage_buf = ctx->alloc<double>((size_t)ctx->max_days * 7 * ctx->nstate());
    if (!ctx->daily_storage_buf) return WG_ERR_NOMEM;
  }
  ctx->mon.daily_storage = enable ? ctx->daily_storage_buf : nullptr;
  ctx->mon.daily_days = enable ? ctx->max_days : 0;
  return WG_OK;
}

wg_status wg_get_daily_storages(wg_ctx *ctx, int32_t day0, int32_t ndays, double *out) {
  if (!ctx || !out || day0 < 0 || ndays < 0 || day0 + ndays > ctx->max_days) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!ctx->mon.daily_storage) return WG_ERR_INVALID;
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  const int n = ctx->n;
  std::vector<double> slots((size_t)ndays * 7 * n);
  cudaError_t e = cudaMemcpy(slots.data(), ctx->mon.daily_storage + (size_t)day0 * 7 * n,
                             slots.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "get_daily_storages");
  const auto &c2s = ctx->topo.cell_of_slot;
  for (size_t r = 0; r < (size_t)ndays * 7; ++r)
    for (int sl = 0; sl < n; ++sl) out[r * n + c2s[sl]] = slots[r * n + sl];
  return WG_OK;
}

wg_status wg_reset_balance(wg_ctx *ctx) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaSuccess;
  if (ctx->balance.enabled)
    e = cudaMemsetAsync(ctx->balance.acc, 0, (size_t)WG_BALANCE_ARRAYS * ctx->nstate() * sizeof(double), ctx->stream);
  if (e == cudaSuccess)
    e = ctx->precision == 0 ? launch_volume(ctx->cd, ctx->sd, ctx->members, ctx->vol0, ctx->stream)
                            : launch_volume(ctx->cf, ctx->sf, ctx->members, ctx->vol0, ctx->stream);
  ctx->launches++;
  return cuda_fail(ctx, e, "reset_balance");
}

wg_status wg_get_balance(wg_ctx *ctx, double out[6]) {
  if (!ctx || !out) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!ctx->balance.enabled) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  int nb = 0;
  cudaError_t e = ctx->precision == 0 ? launch_balance_sum(ctx->cd, ctx->sd, ctx->members, ctx->balance, ctx->vol0,
                                                           ctx->partial, &nb, ctx->stream)
                                      : launch_balance_sum(ctx->cf, ctx->sf, ctx->members, ctx->balance, ctx->vol0,
                                                           ctx->partial, &nb, ctx->stream);
  ctx->launches++;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "get_balance");
  std::vector<double> part((size_t)nb * 8);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  e = cudaMemcpy(part.data(), ctx->partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "get_balance");
  double sum[5] = {0, 0, 0, 0, 0}, comp[5] = {0, 0, 0, 0, 0}, mx = 0.;
  for (int b = 0; b < nb; ++b) {
    for (int k = 0; k < 5; ++k) {
      const double x = part[(size_t)b * 8 + k], s = sum[k], t = s + x;
      comp[k] += (std::fabs(s) >= std::fabs(x)) ? (s - t) + x : (x - t) + s;
      sum[k] = t;
    }
    mx = std::max(mx, part[(size_t)b * 8 + 5]);
  }
  for (int k = 0; k < 5; ++k) out[k] = sum[k] + comp[k];
  out[5] = mx;
  return WG_OK;
}

wg_status wg_get_balance_noalloc(wg_ctx *ctx, double out[6]) {
  if (!ctx || !out) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (!ctx->balance.enabled) return WG_ERR_INVALID;
  if ((int64_t)ctx->nstate() > noalloc_max_states()) {
    ctx->err = "wg_get_balance_noalloc: " + std::to_string(ctx->nstate()) + " states exceed its fixed scratch of " +
               std::to_string(noalloc_max_states()) + " states";
    return WG_ERR_INVALID;
  }
  cudaSetDevice(ctx->device);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  cudaError_t e = ctx->precision == 0
                      ? balance_noalloc(ctx->device, ctx->cd, ctx->sd, ctx->members, ctx->balance, ctx->vol0,
                                        ctx->stream, out)
                      : balance_noalloc(ctx->device, ctx->cf, ctx->sf, ctx->members, ctx->balance, ctx->vol0,
                                        ctx->stream, out);
  ctx->launches += 2;
  return cuda_fail(ctx, e, "get_balance_noalloc");
}


wg_status wg_set_member_factors(wg_ctx *ctx, const float *prec_factor, const float *gamma_factor) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  cudaSetDevice(ctx->device);
  const int M = ctx->members;
  std::vector<float> fac(2 * (size_t)M, 1.0f);
  for (int k = 0; k < M; ++k) {
    if (prec_factor) fac[k] = prec_factor[k];
    if (gamma_factor) fac[M + k] = gamma_factor[k];
    if (!(fac[k] >= 0.f) || !(fac[M + k] > 0.f)) return WG_ERR_INVALID;
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy((float *)ctx->mem.prec_factor, fac.data(), fac.size() * sizeof(float), cudaMemcpyHostToDevice);
  return cuda_fail(ctx, e, "set_member_factors");
}

wg_status wg_set_step_sync(wg_ctx *ctx, int32_t flags) {
  if (!ctx || (flags != 0 && flags != 1)) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (flags == 1 && !ctx->sync.wstep) return WG_ERR_UNSUPPORTED;
  ctx->sync.flow = flags;
  return WG_OK;
}

static cudaError_t vconst_upload(wg_ctx *ctx);

wg_status wg_monthly_outputs(wg_ctx *ctx, int32_t nmonths, int32_t doy_day0) {
  if (!ctx || nmonths < 0 || doy_day0 < 1 || doy_day0 > 365) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "monthly_outputs");
  if (ctx->mon_buf) {
    cudaFree(ctx->mon_buf);
    ctx->mon_buf = nullptr;
  }
  if (ctx->mon_vbuf) {
    cudaFree(ctx->mon_vbuf);
    ctx->mon_vbuf = nullptr;
  }
  if (ctx->mon_rbuf) {
    cudaFree(ctx->mon_rbuf);
    ctx->mon_rbuf = nullptr;
  }
  if (ctx->mon_tbuf) {
    cudaFree(ctx->mon_tbuf);
    ctx->mon_tbuf = nullptr;
  }
  {   // the daily storage record and the daily grids are kept
    const DevMonthly keep = ctx->mon;
    ctx->mon = DevMonthly{};
    ctx->mon.daily_storage = keep.daily_storage;
    ctx->mon.daily_days = keep.daily_days;
    ctx->mon.dvert = keep.dvert;
    ctx->mon.dvert_days = keep.dvert_days;
    ctx->mon.vconst = keep.vconst;
    ctx->mon.drout = keep.drout;
    ctx->mon.drout_days = keep.drout_days;
  }
  if (nmonths == 0) return WG_OK;
  const size_t per = (size_t)nmonths * ctx->nstate();
  e = cudaMalloc((void **)&ctx->mon_buf, 6 * per * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "monthly_outputs");
  DevMonthly &m = ctx->mon;
  m.river_avail = ctx->mon_buf;
  m.storage = ctx->mon_buf + per;
  m.min_avail = ctx->mon_buf + 2 * per;
  m.max_avail = ctx->mon_buf + 3 * per;
  m.cell_runoff = ctx->mon_buf + 4 * per;
  m.velocity = ctx->mon_buf + 5 * per;
  m.nmonths = nmonths;
  m.doy_day0 = doy_day0;
  int mo = 0;
  for (int k = 1; k < 12; ++k) mo += (doy_day0 >= kFirstDayInMonth[k]) ? 1 : 0;
  m.month0 = mo;
  m.enabled = 1;
  e = cudaMemsetAsync(ctx->mon_buf, 0, 6 * per * sizeof(double), ctx->stream);
  if (e == cudaSuccess) e = launch_fill(m.min_avail, per, INFINITY, ctx->stream);
  if (e == cudaSuccess) e = launch_fill(m.max_avail, per, -INFINITY, ctx->stream);
  if (e == cudaSuccess && ctx->mon_vert_on) {   // the vertical balance's grids, on the same calendar
    e = cudaMalloc((void **)&ctx->mon_vbuf, (size_t)wg::VOUT_FIELDS * per * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->mon_vbuf, 0, (size_t)wg::VOUT_FIELDS * per * sizeof(double), ctx->stream);
    if (e == cudaSuccess) e = vconst_upload(ctx);
    if (e == cudaSuccess) m.vert = ctx->mon_vbuf;
  }
  if (e == cudaSuccess && ctx->wt.enabled) {   // the monthly mean water temperatures (sums and day counts)
    const size_t b = (size_t)12 * per * sizeof(double);
    e = cudaMalloc((void **)&ctx->mon_tbuf, b);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->mon_tbuf, 0, b, ctx->stream);
    if (e == cudaSuccess) m.wtemp = ctx->mon_tbuf;
  }
  if (e == cudaSuccess && ctx->mon_rout_on) {   // routing's further grids, on the same calendar
    const size_t b = (size_t)wg::ROUT_FIELDS * per * sizeof(double);
    e = cudaMalloc((void **)&ctx->mon_rbuf, b);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->mon_rbuf, 0, b, ctx->stream);
    if (e == cudaSuccess) e = vconst_upload(ctx);
    if (e == cudaSuccess) m.rext = ctx->mon_rbuf;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return cuda_fail(ctx, e, "monthly_outputs");
}

// the output grids' conditions: FP64, one member; with the water temperature
// only the vertical balance's, and not with water use too; routing's further
// grids also without fractional routing (its groundwater runoff splits between
// the river and the water bodies)
static wg_status outputs_supported(const wg_ctx *ctx, bool routing) {
  if (ctx->precision != 0 || ctx->members != 1) return WG_ERR_UNSUPPORTED;
  if (ctx->wt.enabled && (routing || ctx->wu.enabled)) return WG_ERR_UNSUPPORTED;
  if (routing && ctx->frac_routing) return WG_ERR_UNSUPPORTED;
  return WG_OK;
}

wg_status wg_monthly_outputs_routing(wg_ctx *ctx, int32_t enable) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (enable) {
    const wg_status st = outputs_supported(ctx, true);
    if (st != WG_OK) return st;
  }
  ctx->mon_rout_on = enable != 0;
  if (!ctx->mon.enabled) return WG_OK;   // takes effect with wg_monthly_outputs
  return wg_monthly_outputs(ctx, ctx->mon.nmonths, ctx->mon.doy_day0);
}

wg_status wg_daily_outputs_routing(wg_ctx *ctx, int32_t ndays) {
  if (!ctx || ndays < 0) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (ndays > 0) {
    const wg_status st = outputs_supported(ctx, true);
    if (st != WG_OK) return st;
  }
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "daily_outputs_routing");
  if (ctx->mon_drbuf) {
    cudaFree(ctx->mon_drbuf);
    ctx->mon_drbuf = nullptr;
  }
  ctx->mon.drout = nullptr;
  ctx->mon.drout_days = 0;
  if (ndays == 0) return WG_OK;
  const size_t bytes = (size_t)wg::DROUT_FIELDS * ndays * (size_t)ctx->n * sizeof(double);
  e = cudaMalloc((void **)&ctx->mon_drbuf, bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->mon_drbuf, 0, bytes, ctx->stream);
  if (e == cudaSuccess) e = vconst_upload(ctx);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "daily_outputs_routing");
  ctx->mon.drout = ctx->mon_drbuf;
  ctx->mon.drout_days = ndays;
  return WG_OK;
}

wg_status wg_get_daily_routing(wg_ctx *ctx, int32_t field, int32_t day0, int32_t nd, double *out) {
  if (!ctx || !out || field < 0 || field > wg::DROUT_FIELDS || day0 < 0 || nd < 0 || day0 + nd > ctx->mon.drout_days)
    return WG_ERR_INVALID;
  // the cell AET (field DROUT_FIELDS) adds the land part from the vertical balance's daily grids
  if (field == wg::DROUT_FIELDS && (!ctx->mon.dvert || day0 + nd > ctx->mon.dvert_days)) return WG_ERR_UNSUPPORTED;
  WG_FLUSH(ctx);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  const size_t N = (size_t)ctx->n;
  std::vector<double> buf((size_t)nd * N), land;
  const int f = field == wg::DROUT_FIELDS ? 8 : field;
  cudaError_t e = cudaMemcpy(buf.data(), ctx->mon_drbuf + ((size_t)f * ctx->mon.drout_days + day0) * N,
                             buf.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && field == wg::DROUT_FIELDS) {
    land.resize(buf.size());
    e = cudaMemcpy(land.data(), ctx->mon_dbuf + ((size_t)26 * ctx->mon.dvert_days + day0) * N,
                   land.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      for (size_t k = 0; k < buf.size(); ++k) buf[k] += land[k];
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "get_daily_routing");
  const auto &c2s = ctx->topo.cell_of_slot;
  for (int d = 0; d < nd; ++d)
    for (size_t sl = 0; sl < N; ++sl) out[(size_t)d * N + c2s[sl]] = buf[(size_t)d * N + sl];
  return WG_OK;
}

// The output grids' constants on the device (DevMonthly::vconst), in slot order:
// those of wg_create, and for the cells routed already the freshwater share of
// the current local lakes, as routing.annualInit takes it after the first year
// (routing.cpp:1249-1259, 5045-5048).
static cudaError_t vconst_upload(wg_ctx *ctx) {
  const int n = ctx->n;
  const size_t nn = (size_t)n;
  cudaError_t e = cudaSuccess;
  if (!ctx->mon_vconst) e = cudaMalloc((void **)&ctx->mon_vconst, (size_t)wg::VCONST_FIELDS * nn * sizeof(double));
  if (e != cudaSuccess) return e;
  std::vector<int32_t> started(nn);
  std::vector<double> rf(nn), v((size_t)wg::VCONST_FIELDS * nn);
  e = cudaMemcpy(started.data(), ctx->sd.laf_started, nn * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(rf.data(), ctx->sd.rf_loclake, nn * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  const double *vs = ctx->vstatic.data();
  for (int sl = 0; sl < n; ++sl) {
    const size_t c = (size_t)ctx->topo.cell_of_slot[sl];
    for (int k = 0; k < wg::VCONST_FIELDS; ++k) v[k * nn + sl] = vs[k * nn + c];
    if (started[sl] == 1) {
      const double ll = vs[6 * nn + c];
      const double fll = (ll > 0. && rf[sl] > 0.) ? rf[sl] * ll : 0.;
      v[3 * nn + sl] = v[4 * nn + sl] + fll * 100. + v[5 * nn + sl];
    }
  }
  e = cudaMemcpy(ctx->mon_vconst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) ctx->mon.vconst = ctx->mon_vconst;
  return e;
}

wg_status wg_daily_outputs_vertical(wg_ctx *ctx, int32_t ndays) {
  if (!ctx || ndays < 0) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (ndays > 0) {
    const wg_status st = outputs_supported(ctx, false);
    if (st != WG_OK) return st;
  }
  if (ndays > 0 && !ctx->has_kc) {
    ctx->err = "the daily grids need the region's lct_kc_min and lct_kc_max (Kc)";
    return WG_ERR_INVALID;
  }
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "daily_outputs_vertical");
  if (ctx->mon_dbuf) {
    cudaFree(ctx->mon_dbuf);
    ctx->mon_dbuf = nullptr;
  }
  ctx->mon.dvert = nullptr;
  ctx->mon.dvert_days = 0;
  if (ndays == 0) return WG_OK;
  const size_t bytes = (size_t)wg::DOUT_FIELDS * ndays * (size_t)ctx->n * sizeof(double);
  e = cudaMalloc((void **)&ctx->mon_dbuf, bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->mon_dbuf, 0, bytes, ctx->stream);
  if (e == cudaSuccess) e = vconst_upload(ctx);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "daily_outputs_vertical");
  ctx->mon.dvert = ctx->mon_dbuf;
  ctx->mon.dvert_days = ndays;
  return WG_OK;
}

wg_status wg_get_daily_vertical(wg_ctx *ctx, int32_t field, int32_t day0, int32_t nd, double *out) {
  if (!ctx || !out || field < 0 || field >= wg::DOUT_FIELDS || day0 < 0 || nd < 0 ||
      day0 + nd > ctx->mon.dvert_days)
    return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  const size_t N = (size_t)ctx->n;
  std::vector<double> buf((size_t)nd * N);
  const double *src = ctx->mon_dbuf + ((size_t)field * ctx->mon.dvert_days + day0) * N;
  cudaError_t e = cudaMemcpy(buf.data(), src, buf.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "get_daily_vertical");
  const auto &c2s = ctx->topo.cell_of_slot;
  for (int d = 0; d < nd; ++d)
    for (size_t sl = 0; sl < N; ++sl) out[(size_t)d * N + c2s[sl]] = buf[(size_t)d * N + sl];
  return WG_OK;
}

wg_status wg_monthly_outputs_vertical(wg_ctx *ctx, int32_t enable) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (enable) {
    const wg_status st = outputs_supported(ctx, false);
    if (st != WG_OK) return st;
  }
  ctx->mon_vert_on = enable != 0;
  if (!ctx->mon.enabled) return WG_OK;   // takes effect with wg_monthly_outputs
  return wg_monthly_outputs(ctx, ctx->mon.nmonths, ctx->mon.doy_day0);
}

wg_status wg_get_monthly(wg_ctx *ctx, int32_t which, int32_t m0, int32_t nm, double *out) {
  constexpr int V0 = 6, R0 = V0 + wg::VOUT_FIELDS, AET = R0 + wg::ROUT_FIELDS, WT0 = AET + 2;   // 6, 39, 51, 53
  if (!ctx || !out || which < 0 || which >= WT0 + 6 || m0 < 0 || nm < 0 || m0 + nm > ctx->mon.nmonths)
    return WG_ERR_INVALID;
  if (which >= WT0) {   // the monthly mean water temperatures: -9999 without a computed day
    if (!ctx->mon.wtemp) return WG_ERR_UNSUPPORTED;
    WG_FLUSH(ctx);
    wg_status st = wg_synchronize(ctx);
    if (st != WG_OK) return st;
    const size_t N = ctx->nstate(), per = (size_t)ctx->mon.nmonths * N;
    const int k = which - WT0;
    std::vector<double> sum((size_t)nm * N), cnt((size_t)nm * N);
    cudaError_t e = cudaMemcpy(sum.data(), ctx->mon_tbuf + k * per + (size_t)m0 * N, sum.size() * sizeof(double),
                               cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      e = cudaMemcpy(cnt.data(), ctx->mon_tbuf + (6 + k) * per + (size_t)m0 * N, cnt.size() * sizeof(double),
                     cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "get_monthly");
    const auto &c2s = ctx->topo.cell_of_slot;
    for (int mm = 0; mm < nm; ++mm)
      for (int sl = 0; sl < ctx->n; ++sl) {
        const size_t j = (size_t)mm * N + sl;
        out[(size_t)mm * ctx->n + c2s[sl]] = cnt[j] > 0. ? sum[j] / cnt[j] : -9999.;
      }
    return WG_OK;
  }
  if (which >= V0 && which < R0 && !ctx->mon.vert) return WG_ERR_UNSUPPORTED;
  if (which >= R0 && !ctx->mon.rext) return WG_ERR_UNSUPPORTED;
  if (which >= AET && !ctx->mon.vert) return WG_ERR_UNSUPPORTED;   // cell AET: land AET + open-water evaporation
  WG_FLUSH(ctx);
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  const size_t N = ctx->nstate(), per = (size_t)ctx->mon.nmonths * N;
  const int M = ctx->members;
  std::vector<double> buf((size_t)nm * N);
  auto grid = [&](int w) -> const double * {
    return w < V0 ? ctx->mon_buf + w * per
                  : (w < R0 ? ctx->mon_vbuf + (size_t)(w - V0) * per : ctx->mon_rbuf + (size_t)(w - R0) * per);
  };
  const double *src = grid(which >= AET ? R0 : which);
  cudaError_t e = cudaMemcpy(buf.data(), src + (size_t)m0 * N, buf.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && which >= AET) {
    // G_monthlyCellAET [mm] (routing.cpp:4572-4580): the land AET grid (field 11)
    // plus the open-water evaporation; G_monthlyCellAETWCa [km3] the same over
    // the continental area
    std::vector<double> land(buf.size());
    e = cudaMemcpy(land.data(), grid(V0 + 11) + (size_t)m0 * N, land.size() * sizeof(double), cudaMemcpyDeviceToHost);
    for (size_t k = 0; k < buf.size(); ++k) buf[k] += land[k];
    if (which == AET + 1)
      for (int k = 0; k < nm; ++k)
        for (int sl = 0; sl < ctx->n; ++sl) {
          const int c = ctx->topo.cell_of_slot[sl];
          buf[(size_t)k * N + sl] *= ctx->cell_area[c] * ctx->cell_cont[c] * 1e-8;
        }
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "get_monthly");
  if (which == 2 || which == 3)   // no day in the month, or an inland sink: 0, as the reference's reset grids
    for (double &v : buf)
      if (std::isinf(v)) v = 0.;
  const auto &c2s = ctx->topo.cell_of_slot;
  for (int k = 0; k < nm; ++k)
    for (int sl = 0; sl < ctx->n; ++sl)
      for (int mm = 0; mm < M; ++mm)
        out[((size_t)k * ctx->n + c2s[sl]) * M + mm] = buf[(size_t)k * N + (size_t)sl * M + mm];
  return WG_OK;
}

wg_status wg_set_active_cells(wg_ctx *ctx, const uint8_t *active) {
  if (!ctx) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "set_active_cells");
  uint8_t *dev = nullptr;
  if (active) {
    if (!ctx->d_active) ctx->d_active = ctx->alloc<uint8_t>(ctx->n);
    if (!ctx->d_active) return WG_ERR_NOMEM;
    std::vector<uint8_t> by_slot(ctx->n);
    for (int s = 0; s < ctx->n; ++s) by_slot[s] = active[ctx->topo.cell_of_slot[s]] ? 1 : 0;
    e = cudaMemcpy(ctx->d_active, by_slot.data(), ctx->n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "set_active_cells");
    dev = ctx->d_active;
  }
  ctx->cd.active = dev;
  ctx->cf.active = dev;
  return WG_OK;
}

wg_status wg_set_calib_param(wg_ctx *ctx, int32_t k, const double *values) {
  if (!ctx || !values) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  if (k != 0 && k != 1) return WG_ERR_UNSUPPORTED;
  for (int i = 0; i < ctx->n; ++i)
    if (!(values[i] > 0.) || !std::isfinite(values[i])) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  return ctx->precision == 0 ? set_calib_param(ctx, ctx->cd, k, values) : set_calib_param(ctx, ctx->cf, k, values);
}

wg_status wg_launch_shape(wg_ctx *ctx, int32_t threads, int32_t blocks) {
  if (!ctx || !valid_block_threads(threads, ctx->precision, ctx->members) || blocks < 0) return WG_ERR_INVALID;
  WG_FLUSH(ctx);
  const bool ens = ctx->members > 1;
  const int maxb = ctx->precision == 0 ? pipeline_max_blocks<double>(true, ens, threads)
                                       : pipeline_max_blocks<float>(true, ens, threads);
  const int maxr = ctx->precision == 0 ? pipeline_max_blocks<double>(false, ens, threads)
                                       : pipeline_max_blocks<float>(false, ens, threads);
  const int need = (int)std::min<size_t>((ctx->nstate() + threads - 1) / threads, (size_t)1 << 30);
  if (maxb <= 0 || maxr <= 0) return WG_ERR_DEVICE;
  ctx->layout.idle_warp = -1;   // plain mapping (slot i -> thread i mod the grid)
  ctx->threads = threads;
  ctx->blocks_fused = std::min(blocks > 0 ? std::min(blocks, maxb) : maxb, need);
  ctx->blocks_route = std::min(blocks > 0 ? std::min(blocks, maxr) : maxr, need);
  if (ens && ctx->precision == 1) ctx->blocks_va = std::min(vertical_ahead_max_blocks<float>(true, threads), need);
  return WG_OK;
}

wg_status wg_get_launch_shape(const wg_ctx *ctx, int32_t *threads, int32_t *blocks, int32_t *max_blocks) {
  if (!ctx || !threads || !blocks || !max_blocks) return WG_ERR_INVALID;
  *threads = ctx->threads;
  *blocks = ctx->blocks_fused;
  *max_blocks = ctx->precision == 0 ? pipeline_max_blocks<double>(true, ctx->members > 1, ctx->threads)
                                    : pipeline_max_blocks<float>(true, ctx->members > 1, ctx->threads);
  return WG_OK;
}

}  // extern "C"
