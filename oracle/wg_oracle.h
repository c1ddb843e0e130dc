/*
 * wg_oracle.h -- CPU restatement of the WaterGAP2 daily step (oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker for the GPU library, never a
 * part of it: only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
 * leg load it.  It restates, in plain C and cell by cell, the reference's
 *   dailyWaterBalanceClass::calcNewDay   (source/daily.cpp:94-1257)
 *   laiClass::getDailyLai / dailyLai_*    (source/lai.cpp:152-293)
 *   dailyWaterBalanceClass::calc_ext_rad  (source/daily.cpp:2398-2449)
 *   routingClass::routing                 (source/routing.cpp:1629-4520, 5034-5188)
 *   routingClass::updateLandAreaFrac      (source/routing.cpp:5343-5352)
 *   routingClass::getRiverVelocity / getNewRiverVelocity (source/routing.cpp:7274-7341)
 * for the option set of the hot path (time_series=1, cloud=2, petOpt=0,
 * intercept=1, use_kc=0, calc_albedo=0, clclOpt=0, subtract_use 0/2,
 * fractionalRoutingOpt 0/1, aridareaOpt=0, riverEvapoOpt=0, statcorrOpt=0,
 * use_alloc=0, glacierOpt=0, calc_wtemp 0/1, riverveloOpt 0/1/2), and
 *   calcWaterTempClass::calcWTemp         (source/calcWaterTemp.cpp:48-1324)
 * with its call in routing (source/routing.cpp:4241-4513).
 *
 * Parity pin: in the build container this restatement is compared with the
 * reference's own daily.cpp/routing.cpp object code, linked into a harness
 * (oracle/ref_harness.cpp); the comparison produced the golden fixtures in
 * tests/golden/.  All arithmetic keeps the reference's expression order and
 * is compiled with -ffp-contract=off so that x86 and Arm agree.
 */
#ifndef WG_ORACLE_H
#define WG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A cell is continental when its continental share is at least this many per cent
   (limit_contcell_pct, geo.h:32; geo.cpp:50-60); only continental cells run the
   vertical balance (integrateWGHM.cpp:770-780). */
#define WGO_LIMIT_CONTCELL_PCT 0.000001

/* Calibration parameters, in the order of eCalibParam (source/calib_param.h:72-101). */
enum {
  WGO_P_GAMRUN_C = 0, WGO_P_CFA, WGO_P_CFS, WGO_M_ROOT_D, WGO_M_RIVRGH_C, WGO_P_LAK_D,
  WGO_P_WET_D, WGO_P_SWOUTF_C, WGO_M_EVAREDEX, WGO_M_NETRAD, WGO_P_PTC_HUM, WGO_P_PTC_ARI,
  WGO_P_PET_MXDY, WGO_P_MCWH, WGO_M_LAI, WGO_P_T_SNOWFZ, WGO_P_T_SNOWMT, WGO_M_DEGDAY_F,
  WGO_P_T_GRADNT, WGO_M_GW_F, WGO_M_RG_MAX, WGO_P_PCRITGWA, WGO_P_GWOUTF_C, WGO_M_NETABSSW,
  WGO_M_NETABSGW, WGO_M_PREC, WGO_NPARAM
};

/* Static description of a region: all arrays are caller-owned, length ncell
 * unless stated.  Value types follow the reference's storage types. */
typedef struct {
  int32_t ncell;
  int32_t nband;            /* snow elevation bands (reference: 100)            */
  int32_t river_velo_opt;   /* options.riverveloOpt: 0 constant, 1 inflow-, 2 storage-based */
  int32_t frac_routing;     /* options.fractionalRoutingOpt (aridareaOpt stays 0)     */
  double  default_velocity; /* routingClass::defaultRiverVelocity [km/d]       */
  /* land-cover tables, 18 entries (LCT_22.DAT, LAI_22.DAT)                    */
  const double  *lct_albedo, *lct_albedo_snow, *lct_ddf;
  const float   *lct_lai_a, *lct_lai_b;     /* 0.1*fdp, (1-fdp)*rfep (float)  */
  const int16_t *lct_initial_days;
  /* geometry                                                                  */
  const double  *area_km2;    /* geo.areaOfCellByArrayPos                      */
  const double  *lat_deg;     /* -(G_row/2 - 90.25)                             */
  const double  *contfreq;    /* geo.G_contfreq [%]                            */
  /* land                                                                      */
  const uint8_t *lct;         /* land.G_landCover, 1..18                       */
  const float   *built_up;    /* land.G_built_up                               */
  const float   *smax;        /* maxSoilWaterCap.G_Smax [mm]                   */
  const float   *lai_max;     /* laiClass::G_LAImax                            */
  const float   *gw_factor;   /* GW.getgwFactor                                 */
  const int16_t *rg_max;      /* GW.getRgmax (x100)                            */
  const int8_t  *texture;     /* GW.G_texture                                   */
  const int8_t  *ldd;         /* G_LDD (sign: <0 inland sink)                  */
  const int16_t *aindex;      /* G_aindex (1 arid, 0 humid)                    */
  const int16_t *elev;        /* [ncell*(nband+1)]: [0] mean, [1..] bands asc  */
  const double  *param;       /* [WGO_NPARAM*ncell] calibParam values           */
  /* surface water bodies                                                      */
  const double  *loc_lake, *loc_wetl, *glo_wetl, *glo_lake, *glo_res; /* [%]  */
  const double  *lake_area, *res_area;   /* km2 (outflow cell)                 */
  const double  *stor_cap;    /* km3                                           */
  const double  *mean_outflow;/* m3/s (after routing.init conversion)          */
  const double  *mean_demand; /* m3/s                                          */
  const int8_t  *res_type;    /* 1 irrigation, 2 other                         */
  const int8_t  *start_month; /* 1..12                                          */
  /* river                                                                     */
  const double  *river_length;/* km, already x contfreq/100                    */
  const double  *river_slope, *roughness, *bankfull; /* as read (float values) */
  /* topology                                                                  */
  const int32_t *downstream;  /* 0-based, -1 outlet / sink                      */
  const int32_t *rout_order;  /* cells in processing order (G_routingCell-1)   */
  int32_t statcorr_opt;       /* options.statcorrOpt: 1 multiplies each cell's
                                 outflow by its G_statCorrFact = P_CFS
                                 (routing.cpp:3929-3931)                       */
} wgo_static;

/* Dynamic state, caller-owned, updated in place. */
typedef struct {
  double *canopy, *soil, *snow /* G_snow */, *snow_band /* [ncell*nband] */;
  int32_t *lai_days, *lai_status; double *lai_precsum;
  double *gw, *river, *loclake, *locwetl, *glolake, *glowetl, *res;
  double *rf_loclake, *rf_locwetl, *rf_glolake, *rf_glowetl, *rf_res;
  double *k_release;
  double *laf, *laf_prev, *fswb_next; int32_t *laf_started;
} wgo_state;

/* Initial state as set by setStoragesToZero + setLakeWetlToMaximum +
 * initFractionStatus + annualInit (first year) of the reference. */
int wgo_init_state(const wgo_static *s, wgo_state *st);

/* Run ndays consecutive days starting at day-of-year doy0 (1..365, wraps).
 * Forcing is day-major float [ndays*ncell] (precipitation mm, temperature C,
 * shortwave W/m2).  Optional outputs (may be NULL):
 *   discharge [ndays*ncell]  transported volume per cell and day [km3/d]
 *   balance   [ndays*6]      storage total, P in, E out, Q out (outlets+sinks),
 *                            sum of per-cell closure residuals, max |residual|
 * nthreads > 1 runs the vertical pass with OpenMP (routing stays serial, as in
 * the reference). */
int wgo_run(const wgo_static *s, wgo_state *st, int doy0, int ndays,
            const float *prec, const float *temp, const float *swrad,
            double *discharge, double *balance, int nthreads);

/* Derived river bottom width [m] (routing.cpp:490-495), exposed for tests. */
double wgo_bottom_width(double bankfull);

/* ---- water temperature (options.calc_wtemp = 1) ----------------------------
 * Input record of one cell and day, the fields of the reference's
 * calcWaterTempClass::transfer (source/calcWaterTemp.h:23-95) in that order,
 * all as double (the two flags 0/1).  Indices of the swb arrays: [0] river,
 * [1] local lake, [2] local wetland, [3] global lake, [4] reservoir,
 * [5] global wetland. */
typedef struct {
  double calc_temp_pp, pp_withdrawal, pp_consumption;
  double short_rad, long_rad, air_temp, cfa, ow_pet, ow_prec, cell_area, gw_temp;
  double inflow[9], inflow_temp[9];     /* by inflow direction, [4] = the cell itself */
  double ice[6];
  double river_stor, gw_runoff_into_river, runoff_into_river, river_bottom_width, river_length,
         river_length_check, river_inflow, has_outflow;
  double loclake_area, loclake_stor_prev, loclake_temp_prev, loclake_evapo, loclake_rf, local_runoff,
         local_gw_runoff;
  double locwetl_area, locwetl_stor_prev, locwetl_temp_prev, locwetl_evapo, locwetl_rf, locwetl_inflow,
         locwetl_outflow;
  double glolake_area, glolake_stor_prev, glolake_temp_prev, glolake_evapo, glolake_inflow;
  double res_inflow, res_area, res_stor_prev, res_temp_prev, res_evapo;
  double glowetl_inflow, glowetl_area, glowetl_stor_prev, glowetl_temp_prev, glowetl_evapo, glowetl_rf;
} wgo_wt_in;

#define WGO_WT_NIN 73   /* doubles in wgo_wt_in */

/* calcWaterTempClass::calcWTemp (source/calcWaterTemp.cpp:48-240): out[0..5]
 * temperatures [degC] of river/outflow, local lake, local wetland, global lake,
 * reservoir, global wetland (-9999 where none), out[6..11] their ice
 * thickness [km]. */
void wgo_wtemp(const wgo_wt_in *t, double out[12]);
/* wgo_wtemp over n records of WGO_WT_NIN doubles each; out [n*12] */
void wgo_wtemp_batch(const double *records, int n, double *out);

/* Water temperature inputs and state of wgo_run_wt (caller-owned). */
typedef struct {
  const float *longwave;        /* [ndays*ncell] downward longwave [W/m2]              */
  const float *gw_temp;         /* [ncell] climate.G_GW_Temperature_y [degC]           */
  const int32_t *inflow_cells;  /* [ncell*9] G_inflow_cells, 0-based, -1 = none        */
  const double *river_length_check;  /* [ncell] G_riverLengthCheck (as read, 55 = none) */
  double *temp;                 /* [6*ncell] swb-major: previous day's temperatures    */
  double *ice;                  /* [6*ncell] swb-major: ice thickness [km]             */
  double *river_avail;          /* [ncell] G_RiverAvailPreStep                         */
  double *daily_temp;           /* optional [ndays*ncell]: out[0] of each cell and day */
} wgo_wt_io;

/* The reference's start values (routing.cpp:172-198): 15 degC, no ice, no flow. */
void wgo_wt_init(int ncell, wgo_wt_io *wt);

/* wgo_run with the water temperature of every cell after its routing
 * (routing.cpp:4241-4513). */
int wgo_run_wt(const wgo_static *s, wgo_state *st, int doy0, int ndays,
               const float *prec, const float *temp, const float *swrad,
               double *discharge, double *balance, int nthreads, wgo_wt_io *wt);

/* ---- water use (options.subtract_use = 2, use_alloc = 0,
 * delayedUseSatisfaction 0 or 1, aggrNUsGloLakResOpt 0 or 1) -----------------
 * Net abstractions satisfied in the cell itself: NUg from groundwater (adapted
 * by updateNetAbstractionGW, routing.cpp:5503-5572, when the previous day left
 * demand unsatisfied), NUs from the global lake and reservoir (routing.cpp:
 * 2676-2789, 2866-2946, 3066-3105), the river (routing.cpp:3465-3514) and the
 * local lake (routing.cpp:3590-3630), the bookkeeping of the end of the cell
 * (routing.cpp:3736, 3906-3919), the year start (annualInit, routing.cpp:
 * 994-1010) and end (annualWaterUsePostProcessing, routing.cpp:5246-5296).
 * Irrigation reservoirs' release reads the cell's own NUs (the downstream
 * allocation coefficients of routing.cpp:3001-3007 are zero).
 * With nus_agg (aggrNUsGloLakResOpt = 1): the outflow cell of a global lake or
 * reservoir meets the positive NUs of its GLWD unit's riparian cells
 * (aggregated by wgo_aggregate_nus, routing.cpp:926-965) and hands what it could
 * not meet back to each of them, in proportion to their NUs, as demand of
 * their next routing (routing.cpp:2199-2222, 3083-3165); every outflow cell
 * has a unit > 0, one outflow cell per unit. */
#define WGO_WU_NSTATE 13
/* state rows: 0 G_dailyRemainingUse, 1 G_unsatisfiedNAsFromIrrig,
 * 2 G_unsatisfiedNAsFromOtherSectors, 3 G_reducedReturnFlow,
 * 4 G_withdrawalIrrigFromSwb, 5 G_consumptiveUseIrrigFromSwb,
 * 6 G_totalUnsatisfiedUse, 7 G_UnsatisfiedUsePrevYear,
 * 8 G_unsatisfiedNAsFromIrrigPrevYear, 9 G_unsatisfiedNAsFromOtherSectorsPrevYear,
 * 10 G_reducedReturnFlowPrevYear, 11 G_actualUse, 12 G_unsatUseRiparian */
typedef struct {
  const double *nus, *nug, *wdr, *cons;  /* [nrow*ncell] daily values [km3/d] (dailyNUInit) */
  const int32_t *row_of_day;             /* [ndays] table row of each simulated day         */
  const double *frgi;                    /* [ncell] G_fractreturngw_irrig                   */
  double *state;                         /* [WGO_WU_NSTATE*ncell]                           */
  double *daily_actual;                  /* optional [ndays*ncell]: actual NUs + NUg        */
  int32_t delayed;                       /* 1: options.delayedUseSatisfaction (unmet demand
                                            adds to the next day's, routing.cpp:2236-2244,
                                            3900-3905)                                      */
  const double *nus_agg;                 /* NULL, or [nrow*ncell] daily NUs aggregated over
                                            the GLWD units (aggrNUsGloLakResOpt = 1)        */
  const int32_t *glwd_unit;              /* [ncell] G_glwdUnit (0: none) with nus_agg       */
} wgo_wu_io;

/* dailyNUInit's aggregation of NUs over GLWD units (routing.cpp:926-965), on one
 * month's values [ncell] in m3 (in place: out starts as a copy of nus): each
 * outflow cell of a global lake or reservoir (lake_area or res_area > 0) takes,
 * in cell order, the aggregated value of every other cell of its unit whose own
 * NUs is positive, which drops to 0.  Returns 0, or -1 where an outflow cell has
 * unit 0 or a unit has two outflow cells. */
int wgo_aggregate_nus(int ncell, const double *lake_area, const double *res_area, const int32_t *glwd_unit,
                      const double *nus, double *out);

/* wgo_run with water use. */
int wgo_run_wu(const wgo_static *s, wgo_state *st, int doy0, int ndays,
               const float *prec, const float *temp, const float *swrad,
               double *discharge, double *balance, int nthreads, wgo_wu_io *wu);
/* wgo_run with water use and the water temperature. */
int wgo_run_wt_wu(const wgo_static *s, wgo_state *st, int doy0, int ndays,
                  const float *prec, const float *temp, const float *swrad,
                  double *discharge, double *balance, int nthreads, wgo_wt_io *wt, wgo_wu_io *wu);

/* Wall time [s] of the vertical pass and of the routing pass of the last run
 * (out[0], out[1]): the CPU baseline's split. */
void wgo_last_timing(double out[2]);

#ifdef __cplusplus
}
#endif
#endif
