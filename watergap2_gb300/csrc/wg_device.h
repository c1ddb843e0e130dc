// wg_device.h -- device-side data layout of the GB300 WaterGAP2 daily step.
//
// Every per-cell array lives in "slot" order: cells sorted by their step
// offset in the day-pipelined drainage wavefront (offset = longest flow path
// in the region - distance of the cell to its outlet), ties broken by the
// reference's routing order (source/rout_prepare.cpp:834-886).  The cells of
// one drainage level are therefore a contiguous slot range, and a warp covers
// cells of one level.  Arrays are struct-of-arrays so that a warp's loads
// coalesce; multi-band arrays are band-major ([band][slot]).  An ensemble keeps
// its members innermost ([slot][member]) so that a warp holds 32 members of one
// cell: state loads coalesce and the cell's forcing and constants are one
// broadcast load per warp.
//
// Static quantities that the reference recomputes every day from per-cell
// constants (exp(-k) of the linear reservoirs, lake capacities and their
// reciprocals, 1/(n*M_RIVRGH_C), pow(slope, 0.5), the extraterrestrial
// radiation per latitude and day, ...) are evaluated once on the host and
// stored here in the precision R of the path (double or float).
#pragma once
#include <stdint.h>

namespace wg {

// flag bits of DevCellsT::flags
enum : uint32_t {
  F_ARID = 1u << 0,       // G_aindex == 1                                   (daily.cpp:322-341)
  F_ARID_GW = 1u << 1,    // arid and texture < 21: arid recharge rule         (daily.cpp:1165)
  F_SINK = 1u << 2,       // G_LDD < 0: inland sink                             (routing.cpp:2123, 3935)
  F_EVERGREEN = 1u << 3,  // land cover 1 or 2: status switch in senescence     (lai.cpp:214-216)
  F_LOCLAKE = 1u << 4, F_LOCWETL = 1u << 5, F_GLOLAKE = 1u << 6, F_RES = 1u << 7, F_GLOWETL = 1u << 8,
  F_RES_IRRIG = 1u << 9,  // reservoir type 1
  F_STATION = 1u << 10,
  F_OUTLET = 1u << 11,    // no downstream cell (ocean outlet or inland sink)
  F_VINLINE = 1u << 12,   // vertical balance runs inside the routing wavefront: the cell has a
                          // water body (its land fraction or open-water fluxes depend on routing)
                          // or no land; all other cells run their vertical balance ahead
  F_NOCONT = 1u << 13,    // continental share below limit_contcell_pct (geo.cpp:50-60): the
                          // reference runs no vertical balance there (integrateWGHM.cpp:770-780),
                          // its daily terms stay 0; always with F_VINLINE
};

template <class R>
struct DevCellsT {
  int32_t n;        // cells
  int32_t nband;    // snow bands
  int32_t velo_opt; // riverveloOpt
  int32_t frac_routing;   // fractionalRoutingOpt
  int32_t nrow;     // rows of the extraterrestrial-radiation table
  R default_velocity;
  R invB;           // 1 / nband
  // per slot
  const uint32_t *flags;
  const int32_t *ext_row;       // row of the ext_rad table
  const int16_t *init_days;     // LAI initial days of the cell's land cover
  const int8_t *start_month;    // reservoir start of the operational year (1..12)
  const int32_t *station;       // station index or -1
  // vertical balance
  const R *cfa, *inv_cfa, *mprec, *alpha, *pet_mxdy, *mnetrad, *mcwh, *t_snowfz, *t_snowmt, *pcritgwa, *gamma;
  const R *albedo, *albedo_snow, *ddf_m, *lai_min, *lai_max, *smax, *inv_smax, *fg, *rgmax, *built_up;
  const R *t_gradnt, *elev0;
  const R *contfreq;            // continental share of the cell [%] (the monthly output grids)
  const R *band_dt;             // [nband][n] (elev_b - elev_0) * P_T_GRADNT
  const float *snow_thr;        // FP32 paths: [nband][n] the largest float temperature at which the
                                // band gets snowfall as the FP64 path decides it (null in FP64)
  const double *thr64;          // FP32 paths: [2][n] P_T_GRADNT and P_T_SNOWFZ in FP64 (null in FP64)
  const int16_t *band_el;       // [nband][n] band elevation [m]
  // routing
  const R *area, *area_f;       // km2, km2 * 1e-8 (mm x % -> km3)
  const R *gw_e, *gw_ik, *gw_ome;                 // exp(-k_g), 1/k_g, 1-exp(-k_g)
  const R *sw_k, *sw_e, *sw_ik, *sw_ome;          // P_SWOUTF_C and its exponentials
  const R *evx, *a6;                              // M_EVAREDEX * 3.32193, area/1e6
  const R *ll100, *maxs_ll, *inv_maxs_ll;         // local lake
  const R *lw100, *maxs_lw, *inv_maxs_lw;         // local wetland
  const R *la6, *maxs_gl, *inv_maxs_gl;           // global lake
  const R *ra6, *rcap, *rcap01, *c_ratio, *c4, *one_m_c4, *prov_rel;   // reservoir
  const R *gw100, *maxs_gw, *inv_maxs_gw;         // global wetland
  const R *bw, *inv_mr, *sqrt_slope, *inv_len, *rlen;   // river
  const R *fcatch;                                // fractional routing: share of the runoff through the water bodies
  const R *statcorr;                              // station correction factor P_CFS (statcorrOpt = 1), else null
  // topology in slot space
  const int32_t *up_ptr, *up_idx;               // upstream CSR, each list in reference routing order
  const int32_t *offset;                        // pipeline step offset of the slot
  const uint8_t *active;                        // per slot: 0 = skipped by the day step (null: all run)
  int32_t nlevel;
  int32_t nstation;
  const R *ext_rad, *inv_s0;                    // [365][nrow]: ext_rad and 1/((a_s+b_s) ext_rad)
};

template <class R>
struct DevStateT {
  R *canopy, *soil, *snow, *snow_band;   // snow_band [nband][n*members]
  int32_t *lai_days, *lai_status;
  R *lai_precsum;
  R *gw, *river, *loclake, *locwetl, *glolake, *glowetl, *res;
  R *rf_loclake, *rf_locwetl, *rf_glolake, *rf_glowetl, *rf_res;
  R *k_release;
  R *laf, *laf_prev, *fswb_next;
  int32_t *laf_started;
};

// Vertical outputs handed to routing in the per-day path (single member).
template <class R>
struct DevVertT {
  R *rs, *gwr, *transfer, *owp, *owpet;   // G_dailyLocalSurfaceRunoff, G_dailyGwRecharge, ...
  R *land_in, *land_evap, *land_leak;     // balance terms (mm over the land fraction)
};

// Per-(cell, member) water-balance accumulators, FP64, Neumaier-compensated.
// Arrays 0-4: in, evap, out, up, leak; 5-9 their compensations; 10/11 the land leak
// of the cells whose vertical balance runs ahead of routing and its compensation
// (kept apart from 4, which the wavefront adds the river's leak of those cells to,
// so that both can run at the same time); 12/13 the net abstractions (water use)
// routing takes from such cells, apart from 1 for the same reason.  The wavefront
// adds no in/evap for such cells: their routing adds exactly zero open-water terms.
struct DevBalance {
  double *acc;      // [14][n*members]
  int32_t enabled;
};
constexpr int WG_BALANCE_ARRAYS = 14;

// Monthly aggregates of the routing outputs (routing.cpp:3964-4238: G_monthlyRiverAvail,
// G_monthlyMin/MaxRiverAvail, monthly storage), [nmonths][n*members] each; month m
// of the output calendar = year * 12 + month - month0 of output day od, the
// calendar starting at day-of-year doy_day0 for output day 0.
// The vertical balance's monthly output grids (daily.cpp:1281-1386, grid_store 2),
// field k at vert[k * nmonths * N + month * N + state]: 0 precipitation [mm],
// 1 temperature [degC], 2-7 radiation [W/m2 x days]: extraterrestrial, reflected
// and incoming shortwave, net shortwave, net longwave, net, 8 open-water PET,
// 9 PET, 10 AET of the soil, 11 land AET (cell-corrected), 12 land AET
// uncorrected, 13 LAI, 14 albedo, 15 interception, 16 canopy water content,
// 17 its capacity, 18 snowfall, 19 rainfall, 20 snowmelt, 21 snow evaporation,
// 22 snow water equivalent, 23 snow-covered fraction, 24 soil water, 25 total
// runoff, 26 urban runoff, 27 surface runoff, 28 groundwater recharge [mm
// (x days for states), per day's land share of the continental area where the
// reference weighs it so]; 29-31 canopy, snow and soil storage at the month's
// end [km3]; 32 total PET over land and fresh water (daily.cpp:1303) [mm].
constexpr int VOUT_FIELDS = 33;

// The vertical balance's daily grids (daily.cpp:1388-1399, 1472-1540, grid_store
// 5/6), field k at dvert[k * dvert_days * N + day * N + state]: 0 precipitation,
// 1 temperature, 2 PET, 3 total PET, 4 LAI, 5 crop coefficient Kc, 6 albedo,
// 7 interception, 8 canopy water content, 9 its capacity, 10 snowfall,
// 11 snowmelt, 12 snow water equivalent, 13 snow-covered fraction, 14 soil water,
// 15 surface runoff, 16 groundwater recharge, 17-22 radiation [W/m2]:
// extraterrestrial, incoming and reflected shortwave, net shortwave, net
// longwave, net, 23-25 canopy, snow and soil storage [km3], 26 land AET
// (dailyCellLandAET weighted by the land share of the continental area [mm]:
// the land part of routing's daily cell AET, routing.cpp:4533-4634).
constexpr int DOUT_FIELDS = 27;

// Routing's further monthly grids (routing.cpp:3964-4238, 4525-4737, 5183-5186),
// field k at rext[k * nmonths * N + month * N + state]: 0 open-water evaporation
// [mm] (G_monthlyOpenWaterEvap), 1 cell surface runoff [mm]
// (G_monthlyCellSurfaceRunoff), 2 groundwater runoff [km3] (G_monthlyGwRunoff),
// 3 land-area fraction [% x days] (G_monthlyLandAreaFrac), 4 local and 5 global
// wetland extent [km2 x days], 6 reservoir inflow and 7 outflow [km3] (twice
// the month's flows, as the reference adds them twice a day, routing.cpp:4049-4050
// and 4653-4655),
// 8 consistent precipitation [km3] (G_monthlyConsistentPrecip), 9 surface-water
// storage at the month's end [km3] (G_monthlySurfStor); with water use 10 the
// actual use from surface water [km3] (G_monthlyActualUse) and 11 the net
// abstraction from groundwater [km3] (G_monthlyNUg), routing.cpp:3744-3747.
constexpr int ROUT_FIELDS = 12;
// Routing's daily grids (routing.cpp:4113-4210, 4620-4634), field k at
// drout[k * drout_days * N + day * N + state]: 0 river availability [km3]
// (outside inland sinks), 1 velocity [m/s], 2 cell runoff [km3] and 3 [mm],
// 4 cell surface runoff [mm], 5 groundwater runoff [km3], 6 land-area fraction
// [%], 7 consistent precipitation [km3], 8 open-water evaporation [mm] (the
// open-water part of G_daily365CellAET).
constexpr int DROUT_FIELDS = 9;
// Per state index, for the grids' Kc and total PET: [0] Kc at LAImin
// (kc_min), [1] (kc_max - kc_min) / (LAImax - LAImin) (0 where they are equal),
// [2] LAImin, [3] the freshwater share of the cell for total PET [%]
// (G_fwaterfreq, routing.cpp:1205-1262: updated on the first day of each year
// after the first by the thread that routes the cell), [4] its global-lake and
// [5] its reservoir share [%].
constexpr int VCONST_FIELDS = 6;

struct DevMonthly {
  double *river_avail;   // sum of the day's transported volume [km3/month]   (G_monthlyRiverAvail)
  double *storage;       // sum of the day-end surface-water + groundwater storage [km3 x days]
  double *min_avail, *max_avail;   // (G_monthlyMin/MaxRiverAvail)
  double *cell_runoff;   // sum of transported minus upstream inflow [km3/month] (G_monthlyCellRunoff)
  double *velocity;      // sum of the river velocity [m/s x days]                (G_monthlyVelocity)
  int32_t nmonths, doy_day0, month0, enabled;
  double *vert;          // null, or the vertical balance's grids [VOUT_FIELDS][nmonths][N]
  double *dvert;         // null, or the vertical balance's daily grids [DOUT_FIELDS][dvert_days][N]
  int32_t dvert_days;
  double *vconst;        // with any of vert, dvert, rext, drout: [VCONST_FIELDS][N]
  double *rext;          // null, or routing's further monthly grids [ROUT_FIELDS][nmonths][N]
  // null, or with the water temperature the monthly mean temperatures' sums
  // (fields 0-5: the river, local lake, local wetland, global lake, reservoir,
  // global wetland) and day counts (6-11) [12][nmonths][N]
  double *wtemp;
  double *drout;         // null, or routing's daily grids [DROUT_FIELDS][drout_days][N]
  int32_t drout_days;
  // the day-end routing storages of every cell and output day, [day][7][n*members]
  // in the order the reference writes them into its state file (routing.cpp:5001-5020):
  // local lake, local wetland, global lake, global wetland, reservoir, river,
  // groundwater [km3]; null: not recorded
  double *daily_storage;
  int32_t daily_days;
};

struct DevForcing {
  const float *prec, *temp, *swrad;   // [max_days][n] slot order
  int32_t max_days;
};

// Ensemble members: state index = slot * members + member.
struct DevMembers {
  int32_t members;
  const float *prec_factor;    // [members] multiplicative precipitation perturbation
  const float *gamma_factor;   // [members] multiplicative factor on P_GAMRUN_C
};

// Vertical outputs of the cells that run their vertical balance ahead of routing,
// [ring_days][n*members]: surface runoff and groundwater recharge per cell-day.
template <class R>
struct DevRingT {
  R *rs, *gwr;
  R *owp, *owpet;          // open-water precipitation and PET (only with the water temperature, else null)
  int32_t ring_days;
  int32_t days_per_step;   // days every cell advances per wavefront step (K >= 1)
};

// Water temperature (routing.cpp:4241-4513): state and inputs, slot order.
// swb index [0] river, [1] local lake, [2] local wetland, [3] global lake,
// [4] reservoir, [5] global wetland.
struct DevWaterTemp {
  double *temp;              // [6][N] the previous day's temperatures [degC]
  double *ice;               // [6][N] ice thickness [km] (-9999 where a water body has none)
  double *outt;              // [2][days_per_step][N] river temperature of the step, read downstream
  const float *lw;           // [max_days][n] downward longwave radiation [W/m2]
  const float *gwt;          // [n] yearly groundwater temperature [degC]
  const double *len_check;   // [n] river length as read (55: no river in the cell)
  const double *lake_km2, *res_km2;   // [n] global lake and reservoir area [km2]
  const double *ll_pct, *lw_pct, *gw_pct;   // [n] local lake, local and global wetland [% of the cell]
  double *qst_t;             // [max_days][nstation] river temperature at the stations
  int32_t enabled;
};

// Water use (subtract_use = 2, demand satisfied in the cell itself), slot order.
// Table row r of forcing day f is row_of_fday[f]; row r holds, for every cell slot,
// the day's net abstraction from surface water (NUs) and from groundwater (NUg),
// irrigation withdrawal and consumptive use from surface water [km3/d], and the
// provisional release of a reservoir [m3/s] (routing.cpp:2974-2994), and NUs
// aggregated over GLWD units (routing.cpp:926-965; NUs where none); rows 0-11
// are zero use.  State rows (k * N): 0 remaining use, 1/2 unsatisfied NAs from
// irrigation / other sectors, 3 reduced return flow, 4/5 irrigation withdrawal /
// consumptive use of the last day, 6 total unsatisfied use, 7-10 the previous
// year's 6, 1, 2, 3, 11 actual use of the year, 12 a riparian cell's share of
// its outflow cell's unmet use (G_unsatUseRiparian).
constexpr int WU_FIELDS = 6;
constexpr int WU_NSTATE = 13;
struct DevWaterUse {
  const double *tab;          // [rows][WU_FIELDS][n] (per cell, shared by the members)
  const int32_t *row_of_fday; // [max_days]
  const double *frgi;         // [n] fraction of irrigation return flow into groundwater
  double *st;                 // [WU_NSTATE][N]
  int32_t enabled;
  int32_t delayed;            // unmet demand adds to the next day's (delayedUseSatisfaction)
  // GLWD units (aggrNUsGloLakResOpt = 1, one member): per slot its unit index
  // (-1 no unit, -2 a unit without a global lake or reservoir outflow cell);
  // the slots of unit u in routing order unit_mem[unit_ptr[u] .. unit_ptr[u+1])
  // and in cell order unit_idx[...]
  const int32_t *unit_of, *unit_ptr, *unit_mem, *unit_idx;
  int32_t glwd;
};

// Vertical balance of the cells without water bodies run by extra warps of the
// wavefront launch (warps >= the block's routing warps) for the NEXT launch's
// steps [t_b, t_e): the warps take 32 consecutive slots at a time from the
// counter `next` until nitems groups are taken; warps = 0: no such warps.
struct DevVaWork {
  unsigned int *next;
  int32_t warps, t_b, t_e, nitems;
};

struct DevSync {
  unsigned int *counter;   // monotonic arrival counter of the grid barrier
  int *error;              // 0 ok, nonzero: a barrier wait exceeded its limit (WG_ERR_TIMEOUT)
  // step flags of the single-member layout (flow != 0): instead of a grid barrier
  // per step, each warp of cells publishes the last step it completed (relative
  // to the launch's first step, -1 before it) and waits only for the warps that
  // hold its cells' upstream and downstream cells (CSR dep_ptr/dep_idx by warp)
  int *wstep;
  const int32_t *dep_ptr, *dep_idx;
  int32_t nwarps, flow;
  // failure-detection test: arrivals the grid barrier waits for beyond the grid's
  // blocks (0 in every run; 1 makes each wait run out, see wg_set_barrier_test)
  uint32_t extra_arrivals;
};

}  // namespace wg
