// wg_device.h -- device-side data layout of the GB300 WaterGAP2 daily step.
//
// Every per-cell array lives in "slot" order: cells sorted by their step
// offset in the day-pipelined drainage wavefront (offset = longest flow path
// in the region - distance of the cell to its outlet), ties broken by the
// reference's routing order (source/rout_prepare.cpp:834-886).  A warp
// therefore covers cells of one drainage level, and the cells of one level are
// a contiguous slot range.  Arrays are struct-of-arrays so that the loads of a
// warp coalesce; multi-band arrays are band-major ([band][slot]).
//
// Static quantities that the reference recomputes every day from per-cell
// constants (exp(-k) of the linear reservoirs, lake capacities, 1/(n*M_RIVRGH_C),
// pow(slope, 0.5), the extraterrestrial radiation per latitude and day, ...)
// are evaluated once on the host, with the same expression, and stored here.
#pragma once
#include <stdint.h>

namespace wg {

// flag bits of DevCells::flags
enum : uint32_t {
  F_ARID = 1u << 0,       // G_aindex == 1                                   (daily.cpp:322-341)
  F_ARID_GW = 1u << 1,    // arid and texture < 21: arid recharge rule         (daily.cpp:1165)
  F_SINK = 1u << 2,       // G_LDD < 0: inland sink                             (routing.cpp:2123, 3935)
  F_EVERGREEN = 1u << 3,  // land cover 1 or 2: status switch in senescence     (lai.cpp:214-216)
  F_LOCLAKE = 1u << 4, F_LOCWETL = 1u << 5, F_GLOLAKE = 1u << 6, F_RES = 1u << 7, F_GLOWETL = 1u << 8,
  F_RES_IRRIG = 1u << 9,  // reservoir type 1
  F_STATION = 1u << 10,
  F_OUTLET = 1u << 11,    // no downstream cell (ocean outlet or inland sink)
};

struct DevCells {
  int32_t n;        // cells
  int32_t nband;    // snow bands
  int32_t velo_opt; // riverveloOpt
  int32_t nrow;     // rows of the extraterrestrial-radiation table
  double default_velocity;
  // per slot
  const uint32_t *flags;
  const int32_t *ext_row;       // row of ext_rad table
  const int16_t *init_days;     // LAI initial days of the cell's land cover
  const int8_t *start_month;    // reservoir start of operational year (1..12)
  const int32_t *station;       // station index or -1
  const double *area, *a6;      // km2, km2/1e6
  const double *albedo, *albedo_snow, *ddf_m;  // lct albedo, snow albedo, M_DEGDAY_F*ddf
  const double *lai_min, *lai_max;
  const double *mprec, *alpha, *pet_mxdy, *mnetrad, *mcwh, *t_snowfz, *t_snowmt, *pcritgwa, *gamma, *cfa;
  const double *smax, *fg, *rgmax, *built_up;
  const double *band_dt;        // [nband][n] (elev_b - elev_0) * P_T_GRADNT
  const int16_t *band_el;       // [nband][n] band elevation [m]
  const double *t_gradnt, *elev0;
  // routing constants
  const double *gw_e, *gw_ik, *gw_ome;          // exp(-k_g), 1/k_g, 1-exp(-k_g)
  const double *sw_k, *sw_e, *sw_ik, *sw_ome;   // P_SWOUTF_C and its exponentials
  const double *evx;                            // M_EVAREDEX * 3.32193
  const double *ll100, *maxs_ll;                // local lake
  const double *lw100, *maxs_lw;                // local wetland
  const double *la6, *maxs_gl;                  // global lake
  const double *ra6, *rcap, *rcap01, *rcap085, *c_ratio, *c4, *one_m_c4, *prov_rel;  // reservoir
  const double *gw100, *maxs_gw;                // global wetland
  const double *ll, *lw, *gwet;                 // fractions [%] for the next-day land fraction
  const double *bw, *inv_mr, *sqrt_slope, *rlen;// river
  // topology in slot space
  const int32_t *up_ptr, *up_idx;               // upstream CSR, sorted by reference routing order
  const int32_t *offset;                        // pipeline step offset of the slot
  const int32_t *level_start;                   // [nlevel+1] first slot of each offset
  int32_t nlevel;
  int32_t nstation;
  const double *ext_rad;                        // [365][nrow]
};

struct DevState {
  double *canopy, *soil, *snow, *snow_band;   // snow_band [nband][n]
  int32_t *lai_days, *lai_status;
  double *lai_precsum;
  double *gw, *river, *loclake, *locwetl, *glolake, *glowetl, *res;
  double *rf_loclake, *rf_locwetl, *rf_glolake, *rf_glowetl, *rf_res;
  double *k_release;
  double *laf, *laf_prev, *fswb_next;
  int32_t *laf_started;
};

// Vertical outputs handed to routing in the per-day path.
struct DevVert {
  double *rs, *gwr, *transfer, *owp, *owpet;   // G_dailyLocalSurfaceRunoff, G_dailyGwRecharge, ...
  double *land_in, *land_evap, *land_leak;     // balance terms (mm over the land fraction)
};

// Per-slot water-balance accumulators (Neumaier-compensated: value + compensation).
struct DevBalance {
  double *acc;      // [10][n]: in, evap, out, up, leak and their compensations
  int32_t enabled;
};

struct DevForcing {
  const float *prec, *temp, *swrad;   // [max_days][n] slot order
  int32_t max_days;
};

struct DevSync {
  unsigned int *counter;   // monotonic arrival counter of the grid barrier
  int *error;              // 0 ok, nonzero: barrier wait exceeded (WG_ERR_TIMEOUT)
};

}  // namespace wg
