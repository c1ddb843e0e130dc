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
// evaluated here once, with the reference's expressions, so that the device
// sees the identical double values.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wg_gpu.h"
#include "wg_device.h"
#include "wg_kernels.h"

using namespace wg;

namespace {

const double kPi = 3.141592653589793;   // daily.cpp:73

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

struct Topology {
  std::vector<int32_t> rout_pos;      // position of each cell in the reference routing order
  std::vector<int32_t> offset;        // per cell: pipeline step offset
  std::vector<int32_t> cell_of_slot;  // slot -> cell
  std::vector<int32_t> slot_of_cell;  // cell -> slot
  std::vector<int32_t> level_start;   // [nlevel+1]
  std::vector<int32_t> up_ptr, up_idx;// slot space
  int32_t nlevel = 0;
};

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
  std::vector<char> listed(n, 0);
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

wg_status build_topology(int n, const int32_t *down, const int32_t *rout_order, Topology &t) {
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
  for (int k = n - 1; k >= 0; --k) {
    const int c = order[k];
    depth[c] = down[c] < 0 ? 0 : depth[down[c]] + 1;
    dmax = std::max(dmax, depth[c]);
  }
  t.nlevel = dmax + 1;
  t.offset.resize(n);
  for (int i = 0; i < n; ++i) t.offset[i] = dmax - depth[i];
  // slots: by offset, ties in routing order (a stable bucket pass over the routing order)
  t.level_start.assign(t.nlevel + 1, 0);
  for (int i = 0; i < n; ++i) t.level_start[t.offset[i] + 1]++;
  for (int l = 0; l < t.nlevel; ++l) t.level_start[l + 1] += t.level_start[l];
  std::vector<int32_t> fill(t.level_start.begin(), t.level_start.end() - 1);
  t.cell_of_slot.resize(n);
  t.slot_of_cell.resize(n);
  for (int k = 0; k < n; ++k) {
    const int c = order[k];
    const int s = fill[t.offset[c]]++;
    t.cell_of_slot[s] = c;
    t.slot_of_cell[c] = s;
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

}  // namespace

struct wg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int n = 0, nband = 0, max_days = 0, nstation = 0;
  Topology topo;
  DevCells cells{};
  DevState state{};
  DevVert vert{};
  DevForcing forcing{};
  DevBalance balance{};
  DevSync sync{};
  double *outq = nullptr, *qst = nullptr, *vol0 = nullptr, *partial = nullptr;
  float *staging = nullptr;
  int32_t *d_cell_of_slot = nullptr;
  int staging_days = 0;
  int blocks_fused = 0, blocks_route = 0;
  int64_t launches = 0;
  std::vector<void *> allocs;
  std::string err;

  ~wg_ctx() {
    for (void *p : allocs) cudaFree(p);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
  template <class T>
  T *alloc(size_t count) {
    void *p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return (T *)p;
  }
};

namespace {

wg_status cuda_fail(wg_ctx *ctx, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return WG_OK;
  if (ctx) ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? WG_ERR_NOMEM : WG_ERR_CUDA;
}

// upload a per-cell host array (cell order) into slot order
template <class T>
const T *upload_slots(wg_ctx *ctx, const std::vector<T> &by_cell, wg_status &st) {
  std::vector<T> by_slot(by_cell.size());
  for (size_t s = 0; s < by_slot.size(); ++s) by_slot[s] = by_cell[ctx->topo.cell_of_slot[s]];
  T *d = ctx->alloc<T>(by_slot.size());
  if (!d) { st = WG_ERR_NOMEM; return nullptr; }
  cudaError_t e = cudaMemcpy(d, by_slot.data(), by_slot.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) st = cuda_fail(ctx, e, "upload");
  return d;
}

template <class T>
const T *upload_raw(wg_ctx *ctx, const std::vector<T> &v, wg_status &st) {
  T *d = ctx->alloc<T>(v.size());
  if (!d) { st = WG_ERR_NOMEM; return nullptr; }
  cudaError_t e = cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) st = cuda_fail(ctx, e, "upload");
  return d;
}

// band-major slot layout of a cell-major [ncell][nb] array
template <class T>
std::vector<T> bands_to_slots(const wg_ctx *ctx, const T *cellmajor, int nb) {
  const int n = ctx->n;
  std::vector<T> out((size_t)n * nb);
  for (int s = 0; s < n; ++s) {
    const int c = ctx->topo.cell_of_slot[s];
    for (int b = 0; b < nb; ++b) out[(size_t)b * n + s] = cellmajor[(size_t)c * nb + b];
  }
  return out;
}

struct HostState {
  std::vector<double> canopy, soil, snow, band, precsum, gw, river, loclake, locwetl, glolake, glowetl, res;
  std::vector<double> rf_loclake, rf_locwetl, rf_glolake, rf_glowetl, rf_res, k_release, laf, laf_prev, fswb_next;
  std::vector<int32_t> days, status, started;
};

#define WG_STATE_FIELDS(X)                                                                                     \
  X(canopy) X(soil) X(snow) X(lai_precsum) X(gw) X(river) X(loclake) X(locwetl) X(glolake) X(glowetl) X(res) \
  X(rf_loclake) X(rf_locwetl) X(rf_glolake) X(rf_glowetl) X(rf_res) X(k_release) X(laf) X(laf_prev) X(fswb_next)

wg_status copy_state(wg_ctx *ctx, const wg_state_view *v, bool to_device) {
  const int n = ctx->n, B = ctx->nband;
  const auto &c2s = ctx->topo.cell_of_slot;
  std::vector<double> tmp(n);
  std::vector<int32_t> itmp(n);
  cudaError_t e = cudaSuccess;
  auto dbl = [&](double *host, double *dev) {
    if (!host) return;
    if (to_device) {
      for (int s = 0; s < n; ++s) tmp[s] = host[c2s[s]];
      e = e ? e : cudaMemcpy(dev, tmp.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    } else {
      e = e ? e : cudaMemcpy(tmp.data(), dev, n * sizeof(double), cudaMemcpyDeviceToHost);
      for (int s = 0; s < n; ++s) host[c2s[s]] = tmp[s];
    }
  };
  auto i32 = [&](int32_t *host, int32_t *dev) {
    if (!host) return;
    if (to_device) {
      for (int s = 0; s < n; ++s) itmp[s] = host[c2s[s]];
      e = e ? e : cudaMemcpy(dev, itmp.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice);
    } else {
      e = e ? e : cudaMemcpy(itmp.data(), dev, n * sizeof(int32_t), cudaMemcpyDeviceToHost);
      for (int s = 0; s < n; ++s) host[c2s[s]] = itmp[s];
    }
  };
  cudaStreamSynchronize(ctx->stream);
#define X(f) dbl(v->f, ctx->state.f);
  WG_STATE_FIELDS(X)
#undef X
  i32(v->lai_days, ctx->state.lai_days);
  i32(v->lai_status, ctx->state.lai_status);
  i32(v->laf_started, ctx->state.laf_started);
  if (v->snow_band) {
    std::vector<double> b((size_t)n * B);
    if (to_device) {
      b = bands_to_slots(ctx, v->snow_band, B);
      e = e ? e : cudaMemcpy(ctx->state.snow_band, b.data(), b.size() * sizeof(double), cudaMemcpyHostToDevice);
    } else {
      e = e ? e : cudaMemcpy(b.data(), ctx->state.snow_band, b.size() * sizeof(double), cudaMemcpyDeviceToHost);
      for (int s = 0; s < n; ++s)
        for (int k = 0; k < B; ++k) v->snow_band[(size_t)c2s[s] * B + k] = b[(size_t)k * n + s];
    }
  }
  return cuda_fail(ctx, e, to_device ? "set_state" : "get_state");
}

}  // namespace

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

const char *wg_last_error(const wg_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }
int32_t wg_num_levels(const wg_ctx *ctx) { return ctx ? ctx->topo.nlevel : 0; }
int64_t wg_launch_count(const wg_ctx *ctx) { return ctx ? ctx->launches : 0; }

wg_status wg_create(const wg_region *r, const wg_options *opt, wg_ctx **out) {
  if (!r || !opt || !out) return WG_ERR_INVALID;
  *out = nullptr;
  if (r->ncell <= 0 || r->nband <= 0 || r->nband > 256 || opt->max_days <= 0) return WG_ERR_INVALID;
  if (r->river_velo_opt < 0 || r->river_velo_opt > 2) return WG_ERR_UNSUPPORTED;
  if (opt->nstation < 0 || (opt->nstation > 0 && !opt->stations)) return WG_ERR_INVALID;
  const int n = r->ncell, B = r->nband;
  for (int i = 0; i < n; ++i) {
    if (r->lct[i] < 1 || r->lct[i] > WG_NLCT) return WG_ERR_INVALID;
    if (r->res_area[i] > 0.) {
      if (r->res_type[i] != 1 && r->res_type[i] != 2) return WG_ERR_INVALID;
      if (!(r->mean_outflow[i] > 0.) || r->start_month[i] < 1 || r->start_month[i] > 12) return WG_ERR_INVALID;
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= opt->device) return WG_ERR_DEVICE;
  wg_ctx *ctx = new wg_ctx();
  ctx->device = opt->device;
  ctx->n = n;
  ctx->nband = B;
  ctx->max_days = opt->max_days;
  ctx->nstation = opt->nstation;
  wg_status st = WG_OK;
  cudaError_t e = cudaSetDevice(opt->device);
  if (e != cudaSuccess) { delete ctx; return WG_ERR_DEVICE; }
  if (opt->stream) {
    ctx->stream = (cudaStream_t)opt->stream;
  } else {
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete ctx; return WG_ERR_CUDA; }
    ctx->own_stream = true;
  }
  st = build_topology(n, r->downstream, r->rout_order, ctx->topo);
  if (st != WG_OK) { delete ctx; return st; }

  // ----- per-cell constants, cell order (names as in DevCells)
  auto P = [&](int k, int i) { return r->param[(size_t)k * n + i]; };
  enum { GAMRUN = 0, CFA = 1, RIVRGH = 4, LAK_D = 5, WET_D = 6, SWOUTF = 7, EVAREDEX = 8, NETRAD = 9, PTC_HUM = 10,
         PTC_ARI = 11, PET_MXDY = 12, MCWH = 13, T_SNOWFZ = 15, T_SNOWMT = 16, DEGDAY = 17, T_GRADNT = 18,
         PCRITGWA = 21, GWOUTF = 22, PREC = 25 };
  std::vector<uint32_t> flags(n);
  std::vector<int32_t> ext_row(n), station(n, -1);
  std::vector<int16_t> init_days(n);
  std::vector<int8_t> start_month(n);
  std::vector<double> area(n), a6(n), albedo(n), albedo_snow(n), ddf_m(n), lai_min(n), lai_max(n), mprec(n),
      alpha(n), pet_mxdy(n), mnetrad(n), mcwh(n), t_snowfz(n), t_snowmt(n), pcritgwa(n), gamma(n), cfa(n), smax(n),
      fg(n), rgmax(n), built_up(n), t_gradnt(n), elev0(n), gw_e(n), gw_ik(n), gw_ome(n), sw_k(n), sw_e(n), sw_ik(n),
      sw_ome(n), evx(n), ll100(n), maxs_ll(n), lw100(n), maxs_lw(n), la6(n), maxs_gl(n), ra6(n), rcap(n), rcap01(n),
      rcap085(n), c_ratio(n), c4(n), one_m_c4(n), prov_rel(n), gw100(n), maxs_gw(n), ll(n), lw(n), gwet(n), bw(n),
      inv_mr(n), sqrt_slope(n), rlen(n);
  std::vector<double> band_dt((size_t)n * B);
  std::vector<int16_t> band_el((size_t)n * B);
  std::vector<double> lats;
  for (int i = 0; i < n; ++i) {
    const int lct = r->lct[i];
    uint32_t f = 0;
    if (r->aindex[i] == 1) f |= F_ARID;
    if (r->aindex[i] == 1 && r->texture[i] < 21) f |= F_ARID_GW;
    if (r->ldd[i] < 0) f |= F_SINK;
    if (lct <= 2) f |= F_EVERGREEN;
    if (r->loc_lake[i] > 0.) f |= F_LOCLAKE;
    if (r->loc_wetl[i] > 0.) f |= F_LOCWETL;
    if (r->lake_area[i] > 0.) f |= F_GLOLAKE;
    if (r->res_area[i] > 0.) f |= F_RES;
    if (r->glo_wetl[i] > 0) f |= F_GLOWETL;
    if (r->res_type[i] == 1) f |= F_RES_IRRIG;
    if (r->downstream[i] < 0) f |= F_OUTLET;
    flags[i] = f;
    const double ar = r->area_km2[i];
    area[i] = ar;
    a6[i] = ar / 1000000.;
    albedo[i] = r->lct_albedo[lct - 1];
    albedo_snow[i] = r->lct_albedo_snow[lct - 1];
    ddf_m[i] = P(DEGDAY, i) * r->lct_ddf[lct - 1];
    const float lmin = r->lct_lai_a[lct - 1] + r->lct_lai_b[lct - 1] * r->lai_max[i];   // lai.cpp:154 (float)
    lai_min[i] = lmin;
    lai_max[i] = r->lai_max[i];
    init_days[i] = r->lct_initial_days[lct - 1];
    mprec[i] = P(PREC, i);
    alpha[i] = (r->aindex[i] == 1) ? P(PTC_ARI, i) : P(PTC_HUM, i);
    pet_mxdy[i] = P(PET_MXDY, i);
    mnetrad[i] = P(NETRAD, i);
    mcwh[i] = P(MCWH, i);
    t_snowfz[i] = P(T_SNOWFZ, i);
    t_snowmt[i] = P(T_SNOWMT, i);
    pcritgwa[i] = P(PCRITGWA, i);
    gamma[i] = P(GAMRUN, i);
    cfa[i] = P(CFA, i);
    smax[i] = r->smax[i];
    fg[i] = r->gw_factor[i];
    rgmax[i] = r->rg_max[i] / 100.;
    built_up[i] = r->built_up[i];
    t_gradnt[i] = P(T_GRADNT, i);
    const int16_t *el = r->elev + (size_t)i * (B + 1);
    elev0[i] = el[0];
    for (int b = 0; b < B; ++b) {
      band_dt[(size_t)i * B + b] = (el[b + 1] - el[0]) * P(T_GRADNT, i);
      band_el[(size_t)i * B + b] = el[b + 1];
    }
    const double kg = P(GWOUTF, i);
    gw_e[i] = exp(-1. * kg);
    gw_ik[i] = 1. / kg;
    gw_ome[i] = 1. - exp(-1. * kg);
    const double ks = P(SWOUTF, i);
    sw_k[i] = ks;
    sw_e[i] = exp(-1. * ks);
    sw_ik[i] = 1. / ks;
    sw_ome[i] = 1. - exp(-1. * ks);
    evx[i] = P(EVAREDEX, i) * 3.32193;
    const double lakeDepth = P(LAK_D, i) * 0.001, wetlDepth = P(WET_D, i) * 0.001;
    ll[i] = r->loc_lake[i];
    lw[i] = r->loc_wetl[i];
    gwet[i] = r->glo_wetl[i];
    ll100[i] = r->loc_lake[i] / 100.;
    maxs_ll[i] = ((r->loc_lake[i]) / 100.) * ar * lakeDepth;
    lw100[i] = r->loc_wetl[i] / 100.;
    maxs_lw[i] = ((r->loc_wetl[i]) / 100.) * ar * wetlDepth;
    la6[i] = r->lake_area[i] / 1000000.;
    maxs_gl[i] = (r->lake_area[i]) * lakeDepth;
    ra6[i] = r->res_area[i] / 1000000.;
    rcap[i] = r->stor_cap[i];
    rcap01[i] = r->stor_cap[i] * 0.1;
    rcap085[i] = r->stor_cap[i] * 0.85;
    if (r->res_area[i] > 0.) {
      c_ratio[i] = r->stor_cap[i] / (r->mean_outflow[i] * 31536000. / 1000000000.);
      c4[i] = (4. * c_ratio[i] * c_ratio[i]);
      one_m_c4[i] = (1.0 - ((4. * c_ratio[i] * c_ratio[i])));
      if (r->res_type[i] == 1) {
        // net use is out of scope: the downstream monthly demand is 0 (routing.cpp:2961-2983)
        const double monthlyUse = 0.0;
        if (r->mean_demand[i] >= 0.5 * r->mean_outflow[i])
          prov_rel[i] = r->mean_outflow[i] / 2. * (1. + monthlyUse / r->mean_demand[i]);
        else
          prov_rel[i] = r->mean_outflow[i] + monthlyUse - r->mean_demand[i];
      } else {
        prov_rel[i] = r->mean_outflow[i];
      }
    }
    start_month[i] = r->start_month[i];
    gw100[i] = r->glo_wetl[i] / 100.;
    maxs_gw[i] = ((r->glo_wetl[i]) / 100.) * ar * wetlDepth;
    double bf = r->bankfull[i];                       // routing.cpp:488-495
    if (bf < 0.05) bf = 0.05;
    bw[i] = 2.71 * pow(bf, 0.557) - 2.0 * 2.0 * (0.349 * pow(bf, 0.341));
    inv_mr[i] = 1. / (P(RIVRGH, i) * r->roughness[i]);
    sqrt_slope[i] = pow(r->river_slope[i], 0.5);
    rlen[i] = r->river_length[i];
    // latitude row of the extraterrestrial-radiation table
    auto it = std::find(lats.begin(), lats.end(), r->lat_deg[i]);
    if (it == lats.end()) { lats.push_back(r->lat_deg[i]); ext_row[i] = (int32_t)lats.size() - 1; }
    else ext_row[i] = (int32_t)(it - lats.begin());
  }
  for (int k = 0; k < opt->nstation; ++k) {
    const int cidx = opt->stations[k];
    if (cidx < 0 || cidx >= n) { delete ctx; return WG_ERR_INVALID; }
    station[cidx] = k;
  }
  const int nrow = (int)lats.size();
  std::vector<double> ext((size_t)365 * nrow);
  for (int d = 1; d <= 365; ++d)
    for (int k = 0; k < nrow; ++k) ext[(size_t)(d - 1) * nrow + k] = calc_ext_rad((short)d, lats[k]);

  DevCells &c = ctx->cells;
  c.n = n;
  c.nband = B;
  c.velo_opt = r->river_velo_opt;
  c.nrow = nrow;
  c.default_velocity = r->default_velocity;
  c.nlevel = ctx->topo.nlevel;
  c.nstation = opt->nstation;
#define UP(field) c.field = upload_slots(ctx, field, st);
  UP(flags) UP(ext_row) UP(init_days) UP(start_month) UP(station) UP(area) UP(a6) UP(albedo) UP(albedo_snow)
  UP(ddf_m) UP(lai_min) UP(lai_max) UP(mprec) UP(alpha) UP(pet_mxdy) UP(mnetrad) UP(mcwh) UP(t_snowfz)
  UP(t_snowmt) UP(pcritgwa) UP(gamma) UP(cfa) UP(smax) UP(fg) UP(rgmax) UP(built_up) UP(t_gradnt) UP(elev0)
  UP(gw_e) UP(gw_ik) UP(gw_ome) UP(sw_k) UP(sw_e) UP(sw_ik) UP(sw_ome) UP(evx) UP(ll100) UP(maxs_ll) UP(lw100)
  UP(maxs_lw) UP(la6) UP(maxs_gl) UP(ra6) UP(rcap) UP(rcap01) UP(rcap085) UP(c_ratio) UP(c4) UP(one_m_c4)
  UP(prov_rel) UP(gw100) UP(maxs_gw) UP(ll) UP(lw) UP(gwet) UP(bw) UP(inv_mr) UP(sqrt_slope) UP(rlen)
#undef UP
  c.band_dt = upload_raw(ctx, bands_to_slots(ctx, band_dt.data(), B), st);
  c.band_el = upload_raw(ctx, bands_to_slots(ctx, band_el.data(), B), st);
  c.ext_rad = upload_raw(ctx, ext, st);
  std::vector<int32_t> off_slot(n);
  for (int s = 0; s < n; ++s) off_slot[s] = ctx->topo.offset[ctx->topo.cell_of_slot[s]];
  c.offset = upload_raw(ctx, off_slot, st);
  c.level_start = upload_raw(ctx, ctx->topo.level_start, st);
  c.up_ptr = upload_raw(ctx, ctx->topo.up_ptr, st);
  c.up_idx = upload_raw(ctx, ctx->topo.up_idx, st);
  ctx->d_cell_of_slot = (int32_t *)upload_raw(ctx, ctx->topo.cell_of_slot, st);
  if (st != WG_OK) { wg_destroy(ctx); return st; }

  // ----- dynamic buffers
  DevState &s = ctx->state;
#define AL(f, T) s.f = ctx->alloc<T>(n);
  AL(canopy, double) AL(soil, double) AL(snow, double) AL(lai_days, int32_t) AL(lai_status, int32_t)
  AL(lai_precsum, double) AL(gw, double) AL(river, double) AL(loclake, double) AL(locwetl, double)
  AL(glolake, double) AL(glowetl, double) AL(res, double) AL(rf_loclake, double) AL(rf_locwetl, double)
  AL(rf_glolake, double) AL(rf_glowetl, double) AL(rf_res, double) AL(k_release, double) AL(laf, double)
  AL(laf_prev, double) AL(fswb_next, double) AL(laf_started, int32_t)
#undef AL
  s.snow_band = ctx->alloc<double>((size_t)n * B);
  DevVert &v = ctx->vert;
  v.rs = ctx->alloc<double>(n); v.gwr = ctx->alloc<double>(n); v.transfer = ctx->alloc<double>(n);
  v.owp = ctx->alloc<double>(n); v.owpet = ctx->alloc<double>(n); v.land_in = ctx->alloc<double>(n);
  v.land_evap = ctx->alloc<double>(n); v.land_leak = ctx->alloc<double>(n);
  float *fb = ctx->alloc<float>((size_t)3 * ctx->max_days * n);
  ctx->forcing.prec = fb;
  ctx->forcing.temp = fb ? fb + (size_t)ctx->max_days * n : nullptr;
  ctx->forcing.swrad = fb ? fb + (size_t)2 * ctx->max_days * n : nullptr;
  ctx->forcing.max_days = ctx->max_days;
  ctx->staging_days = std::min(ctx->max_days, 32);
  ctx->staging = ctx->alloc<float>((size_t)ctx->staging_days * n);
  ctx->outq = ctx->alloc<double>((size_t)2 * n);
  ctx->qst = ctx->alloc<double>((size_t)ctx->max_days * std::max(1, ctx->nstation));
  ctx->balance.acc = ctx->alloc<double>((size_t)10 * n);
  ctx->balance.enabled = opt->record_balance ? 1 : 0;
  ctx->vol0 = ctx->alloc<double>(n);
  ctx->partial = ctx->alloc<double>((size_t)8 * ((n + 255) / 256));
  ctx->sync.counter = ctx->alloc<unsigned int>(1);
  ctx->sync.error = ctx->alloc<int>(1);
  if (!s.snow_band || !v.land_leak || !fb || !ctx->staging || !ctx->outq || !ctx->qst || !ctx->balance.acc ||
      !ctx->vol0 || !ctx->partial || !ctx->sync.counter || !ctx->sync.error || !s.laf_started) {
    wg_destroy(ctx);
    return WG_ERR_NOMEM;
  }
  cudaMemset(ctx->sync.error, 0, sizeof(int));
  cudaMemset(ctx->outq, 0, (size_t)2 * n * sizeof(double));
  cudaMemset(ctx->qst, 0, (size_t)ctx->max_days * std::max(1, ctx->nstation) * sizeof(double));

  // ----- start-of-run state, cell order (the reference's set-up sequence; see file header)
  std::vector<double> z(n, 0.), one(n, 1.), rf_res(n, 0.), kr(n, 0.1), loclake(n), locwetl(n), glolake(n), glowetl(n),
      resv(n), laf(n), fswb(n), bands((size_t)n * B, 0.), river(n, 0.);
  std::vector<int32_t> iz(n, 0);
  for (int i = 0; i < n; ++i) {
    const double ar = r->area_km2[i];
    const double lakeDepth = P(LAK_D, i) * 0.001, wetlDepth = P(WET_D, i) * 0.001;
    loclake[i] = (r->loc_lake[i] / 100.) * ar * lakeDepth;
    locwetl[i] = (r->loc_wetl[i] / 100.) * ar * wetlDepth;
    glolake[i] = r->lake_area[i] * lakeDepth;
    glowetl[i] = (r->glo_wetl[i] / 100.) * ar * wetlDepth;
    resv[i] = (r->res_area[i] > 0.) ? r->stor_cap[i] : 0.;
    fswb[i] = r->loc_lake[i] / 100. + r->loc_wetl[i] / 100. + r->glo_wetl[i] / 100.;
    double l = (r->contfreq[i] - (r->glo_lake[i] + r->glo_wetl[i] + r->loc_lake[i] + r->loc_wetl[i] + r->glo_res[i]));
    laf[i] = l < 0. ? 0. : l;
    if (r->river_velo_opt == 2) {   // setStoragesToZero starts from G_riverStorageMax (routing.cpp:807-812)
      double bf = r->bankfull[i] < 0.05 ? 0.05 : r->bankfull[i];
      double wbf = 2.71 * pow(bf, 0.557), dbf = 0.349 * pow(bf, 0.341);
      double bwi = wbf - 2.0 * 2.0 * dbf;
      river[i] = r->river_length[i] * 0.5 * dbf / 1000. * (bwi / 1000. + wbf / 1000.);
    }
  }
  wg_state_view init{};
  init.canopy = z.data();
  std::vector<double> z2(n, 0.), z3(n, 0.), z4(n, 0.), z5(n, 0.);
  init.soil = z2.data();
  init.snow = z3.data();
  init.snow_band = bands.data();
  std::vector<int32_t> iz2(n, 0);
  init.lai_days = iz.data();
  init.lai_status = iz2.data();
  init.lai_precsum = z4.data();
  init.gw = z5.data();
  init.river = river.data();
  init.loclake = loclake.data();
  init.locwetl = locwetl.data();
  init.glolake = glolake.data();
  init.glowetl = glowetl.data();
  init.res = resv.data();
  std::vector<double> o1(n, 1.), o2(n, 1.), o3(n, 1.), o4(n, 1.);
  init.rf_loclake = o1.data();
  init.rf_locwetl = o2.data();
  init.rf_glolake = o3.data();
  init.rf_glowetl = o4.data();
  init.rf_res = rf_res.data();
  init.k_release = kr.data();
  init.laf = laf.data();
  std::vector<double> lp(n, 0.);
  init.laf_prev = lp.data();
  init.fswb_next = fswb.data();
  std::vector<int32_t> started(n, 0);
  init.laf_started = started.data();
  st = copy_state(ctx, &init, true);
  if (st != WG_OK) { wg_destroy(ctx); return st; }
  ctx->blocks_fused = std::min(pipeline_max_blocks(true), (n + 255) / 256);
  ctx->blocks_route = std::min(pipeline_max_blocks(false), (n + 255) / 256);
  if (ctx->blocks_fused <= 0 || ctx->blocks_route <= 0) {
    ctx->err = "cooperative launch not possible";
    wg_destroy(ctx);
    return WG_ERR_DEVICE;
  }
  st = wg_reset_balance(ctx);
  if (st != WG_OK) { wg_destroy(ctx); return st; }
  *out = ctx;
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
  cudaSetDevice(ctx->device);
  return copy_state(ctx, v, true);
}

wg_status wg_get_state(wg_ctx *ctx, wg_state_view *v) {
  if (!ctx || !v) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  return copy_state(ctx, v, false);
}

}  // extern "C"

namespace wg {
cudaError_t launch_gather_forcing(const float *src, float *dst, const int32_t *cell_of_slot, int n, int ndays,
                                  cudaStream_t st);
}

extern "C" {

wg_status wg_upload_forcing(wg_ctx *ctx, int32_t day0, int32_t ndays, const float *prec, const float *temp,
                            const float *swrad) {
  if (!ctx || !prec || !temp || !swrad || day0 < 0 || ndays < 0 || day0 + ndays > ctx->max_days)
    return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  const int n = ctx->n;
  const float *src[3] = {prec, temp, swrad};
  float *dst[3] = {(float *)ctx->forcing.prec, (float *)ctx->forcing.temp, (float *)ctx->forcing.swrad};
  for (int d = 0; d < ndays; d += ctx->staging_days) {
    const int nd = std::min(ctx->staging_days, ndays - d);
    for (int k = 0; k < 3; ++k) {
      cudaError_t e = cudaMemcpyAsync(ctx->staging, src[k] + (size_t)d * n, (size_t)nd * n * sizeof(float),
                                      cudaMemcpyHostToDevice, ctx->stream);
      if (e == cudaSuccess)
        e = launch_gather_forcing(ctx->staging, dst[k] + (size_t)(day0 + d) * n, ctx->d_cell_of_slot, n, nd,
                                  ctx->stream);
      ctx->launches++;
      if (e != cudaSuccess) return cuda_fail(ctx, e, "upload_forcing");
    }
  }
  return WG_OK;
}

wg_status wg_step_vertical(wg_ctx *ctx, int32_t doy, int32_t fday) {
  if (!ctx || doy < 1 || doy > 365 || fday < 0 || fday >= ctx->max_days) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  ctx->launches++;
  return cuda_fail(ctx, launch_vertical(ctx->cells, ctx->state, ctx->vert, ctx->forcing, doy, fday, ctx->stream),
                   "step_vertical");
}

wg_status wg_step_routing(wg_ctx *ctx, int32_t doy, int32_t oday) {
  if (!ctx || doy < 1 || doy > 365 || oday < 0 || oday >= ctx->max_days) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  ctx->launches++;
  return cuda_fail(ctx,
                   launch_pipeline(false, ctx->cells, ctx->state, ctx->vert, ctx->forcing, ctx->balance, ctx->sync,
                                   ctx->outq, ctx->qst, doy, 0, oday, 1, ctx->blocks_route, ctx->stream),
                   "step_routing");
}

wg_status wg_run_days(wg_ctx *ctx, int32_t doy0, int32_t fday0, int32_t ndays) {
  if (!ctx || doy0 < 1 || doy0 > 365 || fday0 < 0 || ndays <= 0 || fday0 + ndays > ctx->max_days)
    return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  ctx->launches++;
  return cuda_fail(ctx,
                   launch_pipeline(true, ctx->cells, ctx->state, ctx->vert, ctx->forcing, ctx->balance, ctx->sync,
                                   ctx->outq, ctx->qst, doy0, fday0, fday0, ndays, ctx->blocks_fused, ctx->stream),
                   "run_days");
}

wg_status wg_synchronize(wg_ctx *ctx) {
  if (!ctx) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
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

wg_status wg_get_discharge(wg_ctx *ctx, int32_t day0, int32_t ndays, double *out) {
  if (!ctx || !out || day0 < 0 || ndays < 0 || day0 + ndays > ctx->max_days) return WG_ERR_INVALID;
  if (ctx->nstation == 0 || ndays == 0) return WG_OK;
  wg_status st = wg_synchronize(ctx);
  if (st != WG_OK) return st;
  return cuda_fail(ctx,
                   cudaMemcpy(out, ctx->qst + (size_t)day0 * ctx->nstation,
                              (size_t)ndays * ctx->nstation * sizeof(double), cudaMemcpyDeviceToHost),
                   "get_discharge");
}

wg_status wg_reset_balance(wg_ctx *ctx) {
  if (!ctx) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaMemsetAsync(ctx->balance.acc, 0, (size_t)10 * ctx->n * sizeof(double), ctx->stream);
  if (e == cudaSuccess) e = launch_volume(ctx->cells, ctx->state, ctx->vol0, ctx->stream);
  ctx->launches++;
  return cuda_fail(ctx, e, "reset_balance");
}

wg_status wg_get_balance(wg_ctx *ctx, double out[6]) {
  if (!ctx || !out) return WG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  int nb = 0;
  cudaError_t e = launch_balance_sum(ctx->cells, ctx->state, ctx->balance, ctx->vol0, ctx->partial, &nb, ctx->stream);
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

}  // extern "C"
