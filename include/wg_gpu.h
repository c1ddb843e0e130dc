/*
 * wg_gpu.h -- C ABI of the GB300 WaterGAP2 daily step (libwg_gpu.so).
 *
 * The library replaces, for one region held on one GPU, the per-day hot path
 * of the reference:
 *   dailyWaterBalanceClass::calcNewDay   source/daily.h:24, daily.cpp:94-1541
 *   routingClass::routing                source/routing.h:44-45, routing.cpp:1629-5244
 *   routingClass::updateLandAreaFrac     source/routing.h:46, routing.cpp:5343-5352
 * together with the state set-up the reference performs before its day loop
 * (setStoragesToZero, setLakeWetlToMaximum, initFractionStatus, annualInit:
 * source/daily.cpp:1882-1894, routing.cpp:748-848, 979-1205, 5647-5716).
 *
 * Conventions: plain pointers and sizes only; every entry point returns a
 * wg_status (no exceptions, no process exit).  Host buffers are owned by the
 * caller; device buffers are owned by the context.  A context is bound to one
 * CUDA device and one stream and is not thread-safe.  Device-side faults of
 * the library's own kernels (an exceeded wait, an inconsistent topology) come
 * back as status codes, never as traps.
 *
 * Option set (the reference's optionClass, source/option.h:43-68), given by
 * wg_model_options (wg_options.model) and the region: time_series=1, cloud=2,
 * petOpt=0, intercept=1, use_kc=0, calc_albedo=0, clclOpt=0, permaOpt=0,
 * glacierOpt=0, landCoverOpt=0, aridareaOpt=0, riverEvapoOpt=0, statcorrOpt 0/1,
 * use_alloc=0, aggrNUsGloLakResOpt=0, antNatOpt=0, resYearOpt=0, resOpt 0/1,
 * climate_spatial_resolution=0, riverveloOpt 0/1/2, fractionalRoutingOpt 0/1,
 * subtract_use 0/2 with delayedUseSatisfaction 0/1 and calc_wtemp 0/1
 * (wg_options.water_use, water_temp).  Other option values are out of scope
 * and rejected with WG_ERR_UNSUPPORTED; wg_last_error(NULL) names the option.
 */
#ifndef WG_GPU_H
#define WG_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  WG_OK = 0,
  WG_ERR_INVALID = 1,      /* bad argument or size                                 */
  WG_ERR_UNSUPPORTED = 2,  /* option outside the supported set                      */
  WG_ERR_CUDA = 3,         /* CUDA runtime error (see wg_last_error)                */
  WG_ERR_NOMEM = 4,        /* device allocation failed                              */
  WG_ERR_TOPOLOGY = 5,     /* drainage network has a cycle or a bad index           */
  WG_ERR_TIMEOUT = 6,      /* a device-side wait exceeded its iteration limit       */
  WG_ERR_DEVICE = 7        /* no usable sm_103a device                               */
} wg_status;

/* Number of calibration parameters (eCalibParam, source/calib_param.h:72-101). */
#define WG_NPARAM 26
#define WG_NLCT 18

/* Static description of a region (host pointers, read once by wg_create).
 * Field types follow the reference's storage types; the parameter block is
 * [WG_NPARAM][ncell] in eCalibParam order. */
typedef struct wg_region {
  int32_t ncell;
  int32_t nband;            /* snow elevation bands (the reference fixes 100)        */
  int32_t river_velo_opt;   /* options.riverveloOpt                                   */
  int32_t frac_routing;     /* options.fractionalRoutingOpt (0/1): runoff from outside
                               the water bodies' catchment goes directly to the river
                               (routing.cpp:1895-2046, 3408-3412); aridareaOpt = 0   */
  double default_velocity;  /* routingClass::defaultRiverVelocity [km/d]              */
  const double *lct_albedo, *lct_albedo_snow, *lct_ddf;        /* [18] LCT_22.DAT    */
  const float *lct_lai_a, *lct_lai_b;                           /* [18] laiClass      */
  const int16_t *lct_initial_days;                              /* [18] LAI_22.DAT    */
  const double *area_km2, *lat_deg;
  const double *contfreq;   /* GCONTFREQ [%] as read; the library raises it to the cell's
                               local-lake + global-lake + reservoir share as geo.init does
                               (geo.cpp:25-45), and cells whose share stays below 1e-6 %
                               (the Caspian Sea in the standard land mask) run neither the
                               vertical balance nor routing (integrateWGHM.cpp:770-780,
                               routing.cpp:1878-4518): their storages stay, their outflow
                               is 0, their inflow leaves the system                     */
  const uint8_t *lct;
  const float *built_up, *smax, *lai_max, *gw_factor;
  const int16_t *rg_max;
  const int8_t *texture, *ldd;
  const int16_t *aindex;
  const int16_t *elev;                                          /* [ncell*(nband+1)]  */
  const double *param;                                          /* [26*ncell]         */
  const double *loc_lake, *loc_wetl, *glo_wetl, *glo_lake, *glo_res;   /* [%]         */
  const double *lake_area, *res_area, *stor_cap, *mean_outflow, *mean_demand;
  const int8_t *res_type, *start_month;
  const double *river_length;  /* G_riverLength as routing.init leaves it: the file's length
                                  times the raised continental share / 100
                                  (routing.cpp:476-482)                                 */
  const double *river_slope, *roughness, *bankfull;
  const int32_t *downstream;   /* 0-based downstream cell, -1 at outlets and sinks   */
  const int32_t *rout_order;   /* reference routing order (G_routingCell - 1)          */
  const int32_t *glwd_unit;    /* G_glwdUnit (GLWDunits.UNF4, 0: none), or NULL; used with
                                  wg_model_options.aggr_nus_glo_lak_res_opt = 1: every
                                  global lake or reservoir outflow cell has a unit > 0,
                                  one outflow cell per unit, and the cells of a unit do
                                  not drain out of it and back in                     */
  const double *lct_kc_min, *lct_kc_max;   /* [18] LAI_22.DAT crop coefficients, or NULL;
                                              needed by wg_daily_outputs_vertical (Kc,
                                              laiClass::getDailyKc, lai.cpp:295-306)  */
} wg_region;

/* Host view of the dynamic state (caller-owned arrays, length ncell unless noted;
 * snow_band is [ncell*nband], cell-major).  A NULL field is skipped: a get or set
 * copies only the fields given. */
typedef struct wg_state_view {
  double *canopy, *soil, *snow, *snow_band;
  int32_t *lai_days, *lai_status;
  double *lai_precsum;
  double *gw, *river, *loclake, *locwetl, *glolake, *glowetl, *res;
  double *rf_loclake, *rf_locwetl, *rf_glolake, *rf_glowetl, *rf_res;
  double *k_release;
  double *laf, *laf_prev, *fswb_next;
  int32_t *laf_started;
} wg_state_view;

/* The reference's model switches (optionClass members, source/option.h:43-68;
 * the option file's values, option.cpp:125-165 and 400-600) as a caller that
 * runs the reference has them.  wg_create refuses every value outside the built
 * set with WG_ERR_UNSUPPORTED, so a configuration the library does not compute
 * never runs silently as a different model.  wg_model_options_default fills
 * the built defaults (the values in brackets). */
typedef struct wg_model_options {
  int32_t time_series;         /* [1] daily forcing from the yearly .365 grids (daily.cpp:194-248) */
  int32_t cloud;               /* [2] net longwave from the extraterrestrial radiation, no
                                  longwave or cloud forcing (daily.cpp:203, 241, 412-440) */
  int32_t intercept;           /* [1] canopy interception (daily.cpp:825-895)             */
  int32_t calc_albedo;         /* [0] land-cover albedo table (daily.cpp:369-380, 1679)   */
  int32_t use_kc;              /* [0] no crop coefficient on PET (daily.cpp:373, 768)     */
  int32_t pet_opt;             /* [0] Priestley-Taylor PET (daily.cpp:208, 272, 489-725)  */
  int32_t clcl_opt;            /* [0] no climate-land-cover classification (daily.cpp:273, 303) */
  int32_t perma_opt;           /* [0] no permafrost input (integrateWGHM.cpp:578-604)     */
  int32_t glacier_opt;         /* [0] no glacier input (daily.cpp:2063, routing.cpp:617, 811) */
  int32_t land_cover_opt;      /* [0] one land-cover map for the run (integrateWGHM.cpp:530-549) */
  int32_t arid_area_opt;       /* [0] no arid-area groundwater routing (routing.cpp:1924-2059,
                                  2392, 3305)                                               */
  int32_t river_evapo_opt;     /* [0] no river evaporation (routing.cpp:3441, 3546, 4562)  */
  int32_t statcorr_opt;        /* [0] or 1: each cell's outflow multiplied by its station
                                  correction factor G_statCorrFact, the calibration
                                  parameter P_CFS of wg_region.param (routing.cpp:3929-3931) */
  int32_t use_alloc;           /* [0] no second-cell allocation of unmet water use
                                  (routing.cpp:2249-2271)                                 */
  int32_t aggr_nus_glo_lak_res_opt;  /* [0] no aggregation of water use over a global lake's
                                        riparian cells (routing.cpp:926-971); 1 with water
                                        use and wg_region.glwd_unit: a riparian cell's
                                        positive NUs is met by its unit's outflow cell,
                                        which hands what it cannot meet back
                                        (routing.cpp:2199-2222, 3083-3165)               */
  int32_t ant_nat_opt;         /* [0] anthropogenic run (routing.cpp:435-440)             */
  int32_t res_year_opt;        /* [0] reservoirs by the reference year (routing.cpp:1054-1072,
                                  5670)                                                   */
  int32_t res_opt;             /* [1] reservoir algorithm; 0 only for a region without
                                  reservoir cells (the reference then treats regulated
                                  lakes as global lakes, routing.cpp:411-430)            */
  int32_t climate_spatial_resolution;   /* [0] the standard land mask (geo.cpp:65,
                                           integrateWGHM.cpp:474-478)                     */
} wg_model_options;

void wg_model_options_default(wg_model_options *opt);

typedef struct wg_options {
  int32_t device;          /* CUDA device ordinal                                     */
  int32_t max_days;        /* capacity of the device forcing buffer, in days          */
  int32_t nstation;        /* cells whose daily discharge is recorded                 */
  int32_t record_balance;  /* 1: keep per-cell water-balance accumulators             */
  const int32_t *stations; /* [nstation] cell indices                                  */
  uint64_t stream;         /* cudaStream_t to use (0 = the context's own stream)      */
  int32_t precision;       /* 0: FP64 state and fluxes (the reference's arithmetic);
                              1: FP32 state and fluxes, FP64 confluence and balance sums */
  int32_t members;         /* ensemble members sharing the forcing (>1 needs precision 1);
                              each member is an independent model state, as one
                              process per member in the reference's data assimilation
                              (source/enKF2wghmState.cpp:17-121)                       */
  const float *member_prec_factor;   /* [members] precipitation multiplier, or NULL   */
  const float *member_gamma_factor;  /* [members] multiplier on P_GAMRUN_C, or NULL   */
  int32_t block_threads;   /* threads per block, a multiple of 32: up to 512 (FP64),   */
                           /* 256 (FP32), 128 (ensembles); 0 = one block per SM for    */
                           /* one FP64 member, 256 for one FP32 member, 64 for         */
                           /* ensembles                                                */
  int32_t ring_days;       /* days of vertical outputs buffered between the vertical
                              balance run ahead and routing; 0 = as many as fit in 8 GB
                              or an eighth of the free device memory, the smaller */
  int32_t days_per_step;   /* days every cell advances per step of the day-pipelined
                              wavefront (1..31; 0 = 1): a run of D days takes
                              ceil(D / days_per_step) + levels - 1 steps.  Results
                              do not depend on it                                    */
  int32_t water_temp;      /* 1: water temperature of the river and every surface water
                              body after each cell's routing (options.calc_wtemp = 1,
                              routing.cpp:4241-4513; fractional routing stays off);
                              FP64, one member.  Needs wg_upload_longwave and
                              wg_set_water_temp_inputs                               */
  int32_t water_use;       /* 1: net water abstractions (options.subtract_use = 2,
                              with use_alloc, delayedUseSatisfaction and
                              aggrNUsGloLakResOpt 0); 2: the same with
                              delayedUseSatisfaction = 1 (a day's unmet demand adds
                              to the next day's); with
                              model->aggr_nus_glo_lak_res_opt = 1 and
                              wg_region.glwd_unit, the riparian cells' net
                              abstractions are met by their global lake's or
                              reservoir's outflow cell (FP64, one member, no
                              water temperature).  Otherwise every cell meets its demand
                              from its own global lake, reservoir, river and local
                              lake and from groundwater.  Any precision and member
                              count (with water_temp: FP64, one member); the
                              members share the tables.  Tables by
                              wg_upload_water_use (days without one: no use)      */
  const wg_model_options *model;   /* the reference's model switches; NULL = the defaults
                              of wg_model_options_default                          */
} wg_options;

typedef struct wg_ctx wg_ctx;

/* Create a context: copies the region to the device in schedule order, builds
 * the drainage topology, and sets the reference's start-of-run state.
 * Replaces dailyWaterBalanceClass::init/setStoragesToZero and routingClass::init/
 * setStoragesToZero/setLakeWetlToMaximum/initFractionStatus/annualInit
 * (source/daily.cpp:1566-1894, routing.cpp:131-1205, 5647-5716). */
wg_status wg_create(const wg_region *region, const wg_options *opt, wg_ctx **out);
wg_status wg_destroy(wg_ctx *ctx);

/* Copy the state host->device / device->host (the reference's setStorages and
 * its wghmState writes: source/daily.cpp:1896-1924, routing.cpp:851-882, 5001-5020). */
wg_status wg_set_state(wg_ctx *ctx, const wg_state_view *state);
wg_status wg_get_state(wg_ctx *ctx, wg_state_view *state);

/* The same for one member of an ensemble context (member 0 is what wg_get_state
 * and wg_set_state address). */
wg_status wg_set_member_state(wg_ctx *ctx, int32_t member, const wg_state_view *state);
wg_status wg_get_member_state(wg_ctx *ctx, int32_t member, wg_state_view *state);

/* Copy ndays of day-major forcing [ndays*ncell] (precipitation mm, temperature C,
 * shortwave W/m2; the reference's climateYear.G_*_d365 floats, climateYear.h:12-15)
 * into forcing slots [day0, day0+ndays) of the device buffer.  A NULL variable
 * keeps the slots' current values (e.g. a precipitation scenario over the same
 * temperature and radiation). */
wg_status wg_upload_forcing(wg_ctx *ctx, int32_t day0, int32_t ndays, const float *prec,
                            const float *temp, const float *swrad);
/* The same upload on the context's copy stream, overlapped with runs already
 * queued: it waits only for earlier uploads, and later runs and steps wait for
 * it.  The caller guarantees that the days it writes are not read by runs still
 * in flight (e.g. next year's forcing while this year runs) and keeps pinned
 * source arrays unchanged until the next wg_synchronize.  No counterpart in the
 * reference (it reads each year's forcing before the year's day loop,
 * climateYear.cpp:38-79). */
wg_status wg_upload_forcing_async(wg_ctx *ctx, int32_t day0, int32_t ndays, const float *prec, const float *temp,
                                  const float *swrad);

/* Forcing straight from the reference's yearly climate files: prec, temp and
 * swrad each hold one `.365.UNF0` file as read from disk -- big-endian float,
 * cell-major [ncell][nd_file] (G_GPCC_..., G_TEMP_..., G_SSRD_...; read by
 * climateYearClass::read_climate_data_daily_per_year, climateYear.cpp:38-79,
 * through GridUNFAdapter::readGrid, grid_io_adapters.h:91-129).  Days
 * [d_first, d_first + ndays) of the files go to day slots day0.. .  The raw
 * bytes are copied to the device as they are; the byte swap and the transpose
 * to the day-major slot layout run on the GPU.  overlap != 0: on the copy
 * stream, as wg_upload_forcing_async. */
wg_status wg_upload_forcing_unf(wg_ctx *ctx, int32_t day0, int32_t nd_file, int32_t d_first, int32_t ndays,
                                const void *prec, const void *temp, const void *swrad, int32_t overlap);

/* The same from native float arrays, cell-major [ncell][nd_file] -- the layout of
 * the reference's yearly grids in memory (climateYear.G_*_d365(n, day - 1),
 * DailyGrid, grid.h:471-474), so a driver passes them without a transpose. */
wg_status wg_upload_forcing_cells(wg_ctx *ctx, int32_t day0, int32_t nd_file, int32_t d_first, int32_t ndays,
                                  const float *prec, const float *temp, const float *swrad, int32_t overlap);

/* Read `bytes` bytes of a file into dst (e.g. a pinned buffer for
 * wg_upload_forcing_unf); returns the bytes read, -1 if the file cannot be
 * opened. */
int64_t wg_read_unf(const char *path, void *dst, int64_t bytes);

/* Water temperature (wg_options.water_temp = 1).  Downward longwave radiation
 * [W/m2], day-major [ndays][ncell] cell order, into forcing slots day0.. (the
 * reference's climate.G_longwave_d, climate.cpp:117-124). */
wg_status wg_upload_longwave(wg_ctx *ctx, int32_t day0, int32_t ndays, const float *longwave);

/* The yearly groundwater temperature [degC] (climate.G_GW_Temperature_y,
 * climate.cpp:109-111; negative values count as 0) and the river length as read
 * from the input file (G_riverLengthCheck, routing.cpp:477; 55 marks a cell
 * without a river), cell order; either may be NULL to keep the current values
 * (start: 10 degC, the region's river length). */
wg_status wg_set_water_temp_inputs(wg_ctx *ctx, const float *gw_temp, const double *river_length_check);

/* Water temperature state, swb-major [6][ncell] cell order, swb 0 river,
 * 1 local lake, 2 local wetland, 3 global lake, 4 reservoir, 5 global wetland:
 * the previous day's temperature [degC] (G_RiverWTempPreStep and the
 * *TempPrevStep grids; start 15) and ice thickness [km] (the G_iceThickness*
 * grids; -9999 where the reference records none). */
wg_status wg_get_water_temp(wg_ctx *ctx, double *temp, double *ice);
wg_status wg_set_water_temp(wg_ctx *ctx, const double *temp, const double *ice);

/* River temperature of the stations' cells after each output day [degC],
 * [ndays][nstation] (the river entry of the state above, day by day). */
wg_status wg_get_river_temp(wg_ctx *ctx, int32_t day0, int32_t ndays, double *out);

/* Water use (wg_options.water_use = 1).  One year's monthly net abstractions
 * [12][ncell] cell order, m3 per month, as the reference's yearly input files
 * hold them (G_NETUSE_SW_m3 / G_NETUSE_GW_m3 already multiplied by the
 * M_NETABSSW / M_NETABSGW calibration factors; G_IRRIG_WITHDRAWAL_USE_SW_m3,
 * G_IRRIG_CONS_USE_SW_m3; dailyNUInit, routing.cpp:884-976), for forcing slots
 * fday0 .. fday0+ndays-1, whose first day is day of year doy0; the days must
 * lie in one year (doy0 + ndays - 1 <= 365).  Converted to km3 per day as the
 * reference does; the tables of the last ceil(max_days / 365) + 1 calls are
 * kept (a call reuses the oldest).  Irrigation reservoirs' provisional release
 * follows the month's use of their cell (routing.cpp:2970-2994; the downstream
 * allocation coefficients are zero). */
wg_status wg_upload_water_use(wg_ctx *ctx, int32_t fday0, int32_t ndays, int32_t doy0, const double *nus_m3,
                              const double *nug_m3, const double *irrig_withdrawal_sw_m3,
                              const double *irrig_consumptive_sw_m3);

/* Fraction of irrigation return flow that reaches groundwater [ncell]
 * (G_fractreturngw_irrig, read by routingClass::init, routing.cpp:540-543);
 * start: 0. */
wg_status wg_set_water_use_inputs(wg_ctx *ctx, const double *frac_return_gw_irrig);

/* Water-use state of routingClass, [WG_WU_NSTATE][ncell][members] cell order, km3:
 * 0 G_dailyRemainingUse, 1 G_unsatisfiedNAsFromIrrig,
 * 2 G_unsatisfiedNAsFromOtherSectors, 3 G_reducedReturnFlow,
 * 4 G_withdrawalIrrigFromSwb, 5 G_consumptiveUseIrrigFromSwb (per day),
 * 6 G_totalUnsatisfiedUse, 7 G_UnsatisfiedUsePrevYear,
 * 8 G_unsatisfiedNAsFromIrrigPrevYear, 9 G_unsatisfiedNAsFromOtherSectorsPrevYear,
 * 10 G_reducedReturnFlowPrevYear, 11 G_actualUse (this year),
 * 12 G_unsatUseRiparian; start: 0.
 * The balance of wg_get_balance counts the net abstractions with the
 * evaporation (out[2]). */
#define WG_WU_NSTATE 13
wg_status wg_get_water_use(wg_ctx *ctx, double *out);
wg_status wg_set_water_use(wg_ctx *ctx, const double *in);

/* One day, the reference's call granularity: the vertical balance of every cell
 * (the OpenMP calcNewDay loop, source/integrateWGHM.cpp:767-783) for day of year
 * doy (1..365) from forcing slot fday ... */
wg_status wg_step_vertical(wg_ctx *ctx, int32_t doy, int32_t fday);
/* ... then routing through the drainage tree and the land-area-fraction update
 * (source/integrateWGHM.cpp:797-798).  Discharge of the stations is recorded at
 * output slot oday. */
wg_status wg_step_routing(wg_ctx *ctx, int32_t doy, int32_t oday);

/* Deferred per-day calls (one member): with enable != 0 the two entry points
 * above only queue their day; consecutive days (day of year, forcing slot and
 * output slot each one more than the day before) run as one day-pipelined run
 * -- the same results as their per-day launches -- when the caller next needs
 * a result or changes an input: every other entry point of this header that
 * takes the context runs the queue first (reads of state, discharge, balance,
 * water use or temperature, uploads, parameter changes, wg_synchronize).  So a
 * driver that keeps the reference's day loop (a calcNewDay pass and a routing
 * call per day, integrateWGHM.cpp:767-798) and reads the model once a month
 * gets the pipelined speed.  Errors of the queued days are reported by the
 * call that runs them.  enable = 0 runs the queue and returns to immediate
 * launches.  No counterpart in the reference. */
wg_status wg_set_deferred(wg_ctx *ctx, int32_t enable);

/* ndays consecutive days in one persistent launch (days pipelined along the
 * drainage depth); identical results to ndays calls of the two entry points
 * above.  Forcing slots fday0.., discharge output slots from fday0 too. */
wg_status wg_run_days(wg_ctx *ctx, int32_t doy0, int32_t fday0, int32_t ndays);

/* A run of ndays days is a wavefront of ndays + levels - 1 steps (step t routes
 * day t - offset(cell) of every cell).  wg_run_steps executes steps [t_begin,
 * t_end) of such a run, so a long run can be split over several calls (for
 * example one call per simulated year) without draining the wavefront between
 * them; the results equal one wg_run_days call.  The state is only consistent
 * (all cells on the same day) after the last step. */
wg_status wg_run_steps(wg_ctx *ctx, int32_t doy0, int32_t fday0, int32_t ndays, int32_t t_begin, int32_t t_end);
int32_t wg_run_num_steps(const wg_ctx *ctx, int32_t ndays);

/* Daily discharge (transported volume, km3/d) of the stations,
 * [ndays][nstation][members], for output slots [day0, day0+ndays). */
wg_status wg_get_discharge(wg_ctx *ctx, int32_t day0, int32_t ndays, double *out);
/* The same for one member of an ensemble, [ndays][nstation] (a data-assimilation
 * driver reads one member's simulated discharge, as each member process of the
 * reference writes its own, enKF2wghmState.cpp:17-121). */
wg_status wg_get_member_discharge(wg_ctx *ctx, int32_t member, int32_t day0, int32_t ndays, double *out);

/* Daily routing storages (one member): with enable != 0 the day step records,
 * for every cell and output day, the day-end storages the reference writes into
 * its state file each day (routing.cpp:5001-5020; WghmStateFile cells,
 * wghmStateFile.h:38-47): local lake, local wetland, global lake, global
 * wetland, reservoir, river, groundwater [km3].  Allocates max_days x 7 x ncell
 * doubles on the device at the first enable.  wg_get_daily_storages returns
 * output days [day0, day0+ndays) as [ndays][7][ncell], cell order. */
wg_status wg_record_daily_storages(wg_ctx *ctx, int32_t enable);
wg_status wg_get_daily_storages(wg_ctx *ctx, int32_t day0, int32_t ndays, double *out);

/* Water balance: out[0] total storage [km3] (land storages over the land fraction
 * plus all surface-water and groundwater storages), out[1..4] accumulated
 * inflow (precipitation), evaporation (with water use: and net abstractions),
 * outflow at outlets and sinks, and clamp
 * corrections since the last wg_reset_balance, out[5] the largest per-cell
 * closure residual relative to the cell's throughput.  Sums are compensated FP64. */
wg_status wg_get_balance(wg_ctx *ctx, double out[6]);
wg_status wg_reset_balance(wg_ctx *ctx);

/* The same sums as wg_get_balance, for callers that cannot allocate device
 * memory after set-up -- for example a process whose free device memory is held
 * by another framework's caching allocator, or a driver that sizes every buffer
 * at start and must not allocate afterwards.  No counterpart in the reference
 * (it has no balance check).  Allocates nothing: the per-block partial sums go
 * to a fixed 4 MiB device array inside the library, which limits the context to
 * 16,777,216 states (cells x members); larger contexts get WG_ERR_INVALID and a
 * message in wg_last_error.  The call waits for the context's stream and copies
 * the sums to `out`, so it is made outside CUDA stream capture.  The first call
 * on a device looks up the array's device address (a failed lookup is retried
 * by the next call).  All calls share the array: calls that overlap on the GPU
 * race.  Needs record_balance. */
wg_status wg_get_balance_noalloc(wg_ctx *ctx, double out[6]);

/* Launch shape of the persistent kernels: threads per block (a multiple of 32
 * up to 512) and blocks (0 = as many as fit on the device at once).  Used by
 * the autotuner. */
wg_status wg_launch_shape(wg_ctx *ctx, int32_t threads, int32_t blocks);
wg_status wg_get_launch_shape(const wg_ctx *ctx, int32_t *threads, int32_t *blocks, int32_t *max_blocks);

/* Replace calibration parameter k of every cell (cell order; eCalibParam index,
 * source/calib_param.h:72-101): 0 = P_GAMRUN_C (runoff coefficient gamma),
 * 1 = P_CFA (areal correction factor); other k give WG_ERR_UNSUPPORTED, values
 * must be positive.  Replaces the reference's calibration loop changing gamma
 * and the correction factor between simulation runs
 * (calibGammaClass::findNewGamma, source/calibration.cpp:266-636;
 * integrateWGHM.cpp:414-417). */
wg_status wg_set_calib_param(wg_ctx *ctx, int32_t k, const double *values);

/* How the wavefront's steps synchronise: 0 = one grid barrier per step (the
 * default); 1 = per-warp step flags, each warp of cells waiting only for the
 * warps that hold its cells' upstream and downstream cells (single-member
 * layout only, WG_ERR_UNSUPPORTED elsewhere).  Results are the same either way;
 * on the global grid the flags measured 3.6 % slower (each warp polls 30-60
 * neighbours scattered by the slot order). */
wg_status wg_set_step_sync(wg_ctx *ctx, int32_t flags);

/* Monthly aggregates of the routing outputs, accumulated by the wavefront
 * kernel as it routes each cell-day (the reference's monthly output grids,
 * routing.cpp:3964-4238: G_monthlyRiverAvail, G_monthlyMin/MaxRiverAvail, the
 * monthly surface-water storage).  nmonths months of an output calendar whose
 * output day 0 (wg_get_discharge's day 0) is day-of-year doy_day0; 0 months
 * switches them off.  Enabling (again) zeroes them. */
wg_status wg_monthly_outputs(wg_ctx *ctx, int32_t nmonths, int32_t doy_day0);
/* The vertical balance's monthly output grids as well (daily.cpp:1281-1386, the
 * reference's grid_store = 2 with grid_store_TypeForStorages = 0), on the calendar
 * of wg_monthly_outputs: FP64, one member, and not with both the water
 * temperature and water use (WG_ERR_UNSUPPORTED otherwise); accumulated by the wavefront's kernels, so the
 * per-day wg_step_vertical refuses while they are on (the deferred per-day calls
 * of wg_set_deferred run through the wavefront).  enable 0 switches them off. */
wg_status wg_monthly_outputs_vertical(wg_ctx *ctx, int32_t enable);
/* which: 0 river availability [km3/month] (sum of the daily transported volume
 * outside inland sinks, routing.cpp:4010-4011),
 * 1 sum of the day-end surface-water + groundwater storage [km3 x days],
 * 2 smallest and 3 largest daily transported volume [km3/day] (outside inland
 * sinks; 0 where the month has no routed day and in sinks, as the reference),
 * 4 cell runoff: transported volume minus upstream inflow (routing.cpp:3933-3939;
 * in inland sinks minus the inflow) [km3/month],
 * 5 sum of the daily river velocity [m/s x days];
 * 6 + k: field k of the vertical balance's grids (wg_monthly_outputs_vertical):
 * 0 G_monthlyPrecipitation [mm], 1 Temperature [degC x days], 2 ExtRad, 3 ShortUpRad,
 * 4 ShortDownRad, 5 NetShortRad, 6 NetLongRad, 7 NetRadiation [W/m2 x days],
 * 8 OpenWaterPET, 9 PET, 10 AET, 11 LandAET, 12 LandAET_uncorr, 13 LAI [x days],
 * 14 Albedo [x days], 15 Interception, 16 canopyWaterContent, 17
 * maxcanopyWaterContent, 18 SnowFall, 19 RainFall, 20 SnowMelt, 21 SnowEvap,
 * 22 SWE, 23 SnowCoverAvg [x days], 24 SoilWaterAvg, 25 Runoff, 26 UrbanRunoff,
 * 27 SurfaceRunoff, 28 GwRecharge [mm, water terms weighted by the land share of
 * the continental area], 29 CanopyStorage, 30 SnowStorage, 31 SoilStorage at
 * the month's end [km3], 32 TotalPET [mm] (daily.cpp:1303: PET over the land
 * and open-water PET over the freshwater share of the continental area);
 * 39 + k: field k of routing's further grids (wg_monthly_outputs_routing):
 * 0 G_monthlyOpenWaterEvap [mm], 1 CellSurfaceRunoff [mm], 2 GwRunoff [km3],
 * 3 LandAreaFrac [% x days], 4 LocWetlExtent and 5 GloWetlExtent [km2 x days],
 * 6 ResInflow and 7 ResOutflow [km3] (twice the month's flows, as the reference
 * adds them twice a day, routing.cpp:4049-4050 and 4653-4655), 8 ConsistentPrecip
 * [km3], 9 SurfStor at the
 * month's end [km3], with water use 10 ActualUse and 11 NUg [km3]
 * (routing.cpp:3744-3747); 51 CellAET [mm] and 52 CellAETWCa [km3]
 * (routing.cpp:4572-4580; both sets of grids needed); with the water
 * temperature 53-58 G_monthlyMeanWaterTempRiver, -LocLake, -LocWetl, -GloLake,
 * -Reservoir, -GloWetl [degC]: the mean over the month's days with a computed
 * temperature, -9999 without one (routing.cpp:4375-4458);
 * out [nm][ncell][members], cell order. */
wg_status wg_get_monthly(wg_ctx *ctx, int32_t which, int32_t m0, int32_t nm, double *out);
/* Routing's further monthly grids (routing.cpp:3964-4238, 4525-4737, 5183-5186,
 * grid_store = 2), on the calendar of wg_monthly_outputs: the same conditions as
 * wg_monthly_outputs_vertical, and without fractional routing
 * (WG_ERR_UNSUPPORTED).  enable 0 switches them off. */
wg_status wg_monthly_outputs_routing(wg_ctx *ctx, int32_t enable);
/* Routing's daily grids (routing.cpp:4113-4210, 4620-4634, grid_store 5/6) for
 * output days 0 .. ndays-1; conditions as wg_monthly_outputs_routing; 0 days
 * switches them off.  A cell without continental area keeps 0. */
wg_status wg_daily_outputs_routing(wg_ctx *ctx, int32_t ndays);
/* field: 0 G_daily365RiverAvail [km3] (0 in inland sinks), 1 Velocity [m/s],
 * 2 CellRunoff [km3], 3 CellRunoff_mm, 4 CellSurfaceRunoff [mm], 5 GwRunoff [km3],
 * 6 LandAreaFrac [%], 7 ConsistentPrecip [km3], 8 the open-water evaporation
 * [mm], 9 CellAET [mm] (field 8 plus the vertical balance's daily land AET:
 * wg_daily_outputs_vertical needed); out [nd][ncell], cell order. */
wg_status wg_get_daily_routing(wg_ctx *ctx, int32_t field, int32_t day0, int32_t nd, double *out);

/* The vertical balance's daily grids (daily.cpp:1388-1399, 1472-1540: the
 * reference's grid_store 5/6 with the daily output options on) for output days
 * 0 .. ndays-1 (wg_get_discharge's days), kept on the device; 0 days switches
 * them off.  Same conditions as wg_monthly_outputs_vertical, and the region's
 * lct_kc_min / lct_kc_max are needed (WG_ERR_INVALID without them).  Enabling
 * (again) zeroes them; a cell without continental area keeps 0, as the
 * reference, which runs no vertical balance there.  Total PET's freshwater share
 * starts from the state at the call (the first year's shares before the first
 * routed day) and follows the local lakes at each year's start as
 * routing.annualInit does (routing.cpp:1205-1262). */
wg_status wg_daily_outputs_vertical(wg_ctx *ctx, int32_t ndays);
/* field: 0 G_daily365Precip [mm], 1 temp [degC], 2 PET, 3 TotalPET, 4 LAI, 5 Kc,
 * 6 Albedo, 7 Interception, 8 canopyWaterContent, 9 maxcanopyWaterContent,
 * 10 SnowFall, 11 SnowMelt, 12 SWE, 13 SnowCoverAvg, 14 SoilWaterAvg,
 * 15 SurfaceRunoff, 16 GwRecharge [mm, water terms weighted by the land share of
 * the continental area], 17 ExtRad, 18 ShortDownRad, 19 ShortUpRad,
 * 20 NetShortRad, 21 NetLongRad, 22 NetRadiation [W/m2], 23 CanopyStorage,
 * 24 SnowStorage, 25 SoilStorage [km3], 26 land AET [mm] (dailyCellLandAET times
 * the land share of the continental area: the land part of routing's cell AET);
 * out [nd][ncell], cell order. */
wg_status wg_get_daily_vertical(wg_ctx *ctx, int32_t field, int32_t day0, int32_t nd, double *out);

/* Cells the day step runs (cell order, nonzero = run; NULL = all).  A skipped
 * cell keeps its state and produces no outflow, so skip whole basins only (a
 * cell and everything upstream of it): the calibration loop drops the basins it
 * has finished, as the reference runs only the cells of the station being
 * calibrated (G_toBeCalculated, integrateWGHM.cpp:421-442). */
wg_status wg_set_active_cells(wg_ctx *ctx, const uint8_t *active);

/* Replace the per-member precipitation and gamma factors of an ensemble
 * (as wg_options.member_prec_factor / member_gamma_factor; NULL = all 1). */
wg_status wg_set_member_factors(wg_ctx *ctx, const float *prec_factor, const float *gamma_factor);

/* Device snapshot of the model state (storages, snow bands, LAI state, land
 * fractions, the wavefront's outflow buffer and the balance sums): save, and
 * restore as often as needed -- e.g. the start state of each calibration run,
 * or a forecast state of data assimilation.  One snapshot per context; the
 * autotuner uses the same one (its trial runs leave the monthly output grids
 * alone).  The output grids and the station discharge are not part of it: days
 * run again after a restore add to the monthly sums again (switch the grids off,
 * or on again to zero them).  No counterpart in the reference (it re-reads state
 * files). */
wg_status wg_save_snapshot(wg_ctx *ctx);
wg_status wg_restore_snapshot(wg_ctx *ctx);

/* Kernel timing: with enable != 0, wg_run_steps records CUDA events on the
 * context's stream around each launch of the vertical-ahead kernel and of the
 * wavefront kernel; wg_get_kernel_times synchronises and returns the summed
 * device time of each since the last call (or since enabling), and the number
 * of launch pairs.  Launches inside a captured graph are not timed. */
wg_status wg_kernel_timing(wg_ctx *ctx, int32_t enable);
wg_status wg_get_kernel_times(wg_ctx *ctx, double *vertical_ahead_ms, double *wavefront_ms, int32_t *launch_pairs);

/* Wavefront steps per launch of wg_run_steps: 1 .. the ring capacity in steps
 * (wg_options.ring_days / days_per_step; half of it with the vertical overlap
 * below); 0 = the default: the ring capacity, or ceil(16 / days_per_step)
 * steps with the overlap.
 * No counterpart in the reference (it has no day pipelining). */
wg_status wg_set_chunk_steps(wg_ctx *ctx, int32_t steps);
int32_t wg_get_chunk_steps(const wg_ctx *ctx);

/* Vertical overlap (one FP64 member with the default launch shape): each
 * wavefront launch of wg_run_steps carries extra warps that run the vertical
 * balance of the cells without water bodies for the next launch's steps, so the
 * FP64 pipe has that work while the routing warps wait; the first chunk of each
 * call runs its vertical balance in a launch of its own.  On by default where
 * the shape allows it.  enable = 0 switches it off (one vertical-ahead launch
 * before each wavefront launch); WG_ERR_UNSUPPORTED where the shape has no room
 * for the extra warps.  wg_get_vertical_overlap returns the extra warps per
 * block (0: off).  Results are the same bits either way. */
wg_status wg_set_vertical_overlap(wg_ctx *ctx, int32_t enable);
int32_t wg_get_vertical_overlap(const wg_ctx *ctx);

/* Autotuner: times wg_run_steps(doy0, fday0, ndays, t_begin, t_begin + trial_steps)
 * for each launch shape -- the context's own (with and without the vertical
 * overlap), threads per block 64 to 512 as the kernels allow
 * (FP64 up to 512, FP32 up to 256, ensembles 64 and 128; for an ensemble,
 * the members of one cell that share a block) and chunk steps 8, 16, ... up to
 * the ring capacity -- restoring the model state from a device snapshot before
 * each trial and after the last, and keeps the fastest shape.  The state, the
 * balance sums and the wavefront buffers are as before the call; station
 * discharge of the trial days is overwritten.  No counterpart in the reference. */
typedef struct wg_tune_result {
  int32_t threads, blocks, chunk_steps, trials;
  double ms_per_step;   /* of the chosen shape, on the trial steps */
} wg_tune_result;
wg_status wg_autotune(wg_ctx *ctx, int32_t doy0, int32_t fday0, int32_t ndays, int32_t t_begin,
                      int32_t trial_steps, wg_tune_result *out);

/* Capture wg_run_steps(doy0, fday0, ndays, t_begin, t_end) -- every launch of
 * the run, the cooperative wavefront launches included -- into a CUDA graph of
 * the context (replacing an earlier one), and replay it on the context's stream
 * with wg_graph_launch.  Each replay runs the same steps again on the state it
 * finds.  No counterpart in the reference. */
wg_status wg_graph_capture(wg_ctx *ctx, int32_t doy0, int32_t fday0, int32_t ndays, int32_t t_begin, int32_t t_end);
wg_status wg_graph_launch(wg_ctx *ctx);

/* Wait for the context's stream.  WG_ERR_TIMEOUT: a device-side wait (the grid
 * barrier of the wavefront, or a step flag) ran out of its iteration limit; the
 * kernel returned without trapping, the CUDA context stays usable, and the
 * library refuses further results until wg_clear_error (after restoring a
 * state: the run stopped part way). */
wg_status wg_synchronize(wg_ctx *ctx);
wg_status wg_clear_error(wg_ctx *ctx);

/* Failure-detection test hook: with extra_arrivals > 0 every grid-barrier wait
 * of the following wavefront launches waits for that many arrivals that never
 * come, runs out after its iteration limit (about a second) and reports
 * WG_ERR_TIMEOUT through wg_synchronize.  0 (the default) for normal runs. */
wg_status wg_set_barrier_test(wg_ctx *ctx, int32_t extra_arrivals);

/* Diagnostic: FP64 fused-multiply-add throughput of a device in TFLOP/s, from a
 * loop of independent DFMA chains (the FP64 ceiling of the plain FP64 path). */
wg_status wg_measure_fp64_peak(int32_t device, double *tflops);

/* Diagnostic (numerics tests): the FP64 path's own math functions on n host
 * values: fn 0 exp(x), 1 log(x), 2 pow(x, y), 3 the refined reciprocal 1/x,
 * 4 the hardware's approximate reciprocal alone (the refinement's start).  y is
 * read for fn 2 only. */
wg_status wg_math_eval(int32_t device, int32_t fn, const double *x, const double *y, int64_t n, double *out);

/* Information: number of drainage levels (longest flow path + 1), kernel
 * launches issued so far, and the last CUDA error string. */
int32_t wg_num_levels(const wg_ctx *ctx);
int64_t wg_launch_count(const wg_ctx *ctx);
/* wg_last_error(NULL): why the calling thread's last wg_create failed. */
const char *wg_last_error(const wg_ctx *ctx);
const char *wg_status_string(wg_status s);

#ifdef __cplusplus
}
#endif
#endif
