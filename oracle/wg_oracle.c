/*
 * wg_oracle.c -- CPU restatement of the WaterGAP2 daily step (oracle).
 *
 * TEST INFRASTRUCTURE ONLY (see wg_oracle.h).  Each block cites the reference
 * lines it restates; expression order follows the reference so that the
 * results agree bit for bit with the reference's own object code where the
 * same libm is used.  Snow bands: the reference divides band sums by its fixed
 * band count 100 (daily.cpp:1047-1061); here the divisor is nband.
 */
#include "wg_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MIN_STOR_VOL 1.e-15              /* routing.h:24                       */
static const double pi = 3.141592653589793; /* daily.cpp:73                    */
static const short first_day_in_month[12] = {1, 32, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335};

/* dailyWaterBalanceClass::setParameters (daily.cpp:1866-1880) */
#define CANOPY_EVAPO_EXP 0.66666666
#define RUNOFF_FRAC_BUILTUP 0.5
#define OPEN_WATER_ALBEDO 0.08
#define A_S 0.25
#define B_S 0.5
#define A_C_ARID 1.35
#define B_C_ARID (-0.35)
#define A_C_HUMID 1.00
#define B_C_HUMID 0.00
/* routingClass::setParameters (routing.cpp:124-129) */
#define LAKE_OUTFLOW_EXP 1.5
#define WETL_OUTFLOW_EXP 2.5
#define EVAPO_RED_EXP 3.32193
#define EVAPO_RED_EXP_RES 2.81383

#define PAR(s, k, n) ((s)->param[(size_t)(k) * (size_t)(s)->ncell + (size_t)(n)])

double wgo_bottom_width(double bf) {
  /* routing.cpp:488-495 */
  if (bf < 0.05) bf = 0.05;
  double w = 2.71 * pow(bf, 0.557);
  double d = 0.349 * pow(bf, 0.341);
  return w - 2.0 * 2.0 * d;
}

/* calc_ext_rad (daily.cpp:2398-2449), latitude given per cell. */
static double calc_ext_rad(short day, double lat_deg) {
  double declination_angle = asin(0.39795 * cos(0.2163108 + 2. * atan(0.9671396 * tan(0.00860 * (day - 186)))));
  const double pi_180 = pi / 180.0;
  double theta = lat_deg * pi_180;
  double omega_s = (sin(theta) * sin(declination_angle)) / (cos(theta) * cos(declination_angle));
  if ((omega_s) < -1.) omega_s = -1;
  if ((omega_s) > 1.) omega_s = 1;
  omega_s = pi - acos(omega_s);
  const double pi2_365 = 2. * pi / 365.0;
  double dist_es = 1. + 0.033 * cos(pi2_365 * day);
  return (15.392 * dist_es * (omega_s * sin(theta) * sin(declination_angle)
          + cos(theta) * cos(declination_angle) * sin(omega_s)));
}

/* laiClass::dailyLai_growing (lai.cpp:179-241) */
static double lai_growing(int *days, short init, int *status, char lct, int arid, double lmin,
                          double lmax, double *psum, double prec) {
  if (*status == 0) {
    if (*days >= init) {
      (*days)++;
      (*psum) += prec;
      if (*psum > 40.) {
        if (*days >= init + 30) { *days = init + 30; *status = 1; }
        return (lmin + (lmax - lmin) * (*days - init) / 30.);
      } else {
        *days = init;
        return (lmin);
      }
    } else {
      (*days)++;
      (*psum) += prec;
      return (lmin);
    }
  } else {
    if (*days <= 30) {
      (*days)--;
      if (lct <= 2) *status = 0;
      if (*days <= 0) { *days = 0; *status = 0; *psum = 0.; }
      return (lmax - (lmax - lmin) * (30 - *days) / 30.);
    } else {
      if ((arid) && (prec < 0.5)) (*days)--;
      else *days = 30 + init;
      return (lmax);
    }
  }
}

/* laiClass::dailyLai_nogrowing (lai.cpp:243-293) */
static double lai_nogrowing(int *days, short init, int *status, char lct, int arid, double lmin,
                            double lmax, double *psum, double prec) {
  (void)lct; (void)arid;
  if (*status == 0) {
    if (*days > init) {
      (*days)++;
      (*psum) += prec;
      if (*psum > 40.) {
        if (*days >= init + 30) { *days = init + 30; *status = 1; }
        return (lmin + (lmax - lmin) * (*days - init) / 30.);
      } else {
        *days = init;
        return (lmin);
      }
    } else {
      (*psum) += prec;
      return (lmin);
    }
  } else {
    if (*days <= 30) {
      (*days)--;
      if (*days <= 0) { *days = 0; *status = 0; *psum = 0.; }
      return (lmax - (lmax - lmin) * (30 - *days) / 30.);
    } else {
      (*days)--;
      return (lmax);
    }
  }
}

/* The continental share as geo.init leaves it (geo.cpp:25-45): at least the cell's
   share of local lakes, global lakes, local reservoirs (none here) and reservoirs,
   summed in that order. */
static double cont_share(const wgo_static *s, int n) {
  double fw = 0.;
  fw += s->loc_lake[n];
  fw += s->glo_lake[n];
  fw += 0.;
  fw += s->glo_res[n];
  return fw > s->contfreq[n] ? fw : s->contfreq[n];
}

int wgo_init_state(const wgo_static *s, wgo_state *st) {
  const int N = s->ncell, B = s->nband;
  for (int n = 0; n < N; n++) {
    double area = s->area_km2[n];
    double lakedepth = PAR(s, WGO_P_LAK_D, n) * 0.001;   /* initLakeDepthActive, routing.cpp:5621-5631 */
    double wetldepth = PAR(s, WGO_P_WET_D, n) * 0.001;   /* initWetlDepthActive, routing.cpp:5635-5643 */
    /* setStoragesToZero (daily.cpp:1882-1894, routing.cpp:790-848) */
    st->canopy[n] = 0.; st->soil[n] = 0.; st->snow[n] = 0.;
    for (int b = 0; b < B; b++) st->snow_band[(size_t)n * B + b] = 0.;
    st->lai_days[n] = 0; st->lai_status[n] = 0; st->lai_precsum[n] = 0.;   /* lai.cpp:55-59 */
    st->gw[n] = 0.; st->river[n] = 0.;
    if (s->river_velo_opt == 2) st->river[n] = 0.;  /* storage-based velocity starts at 0 here too */
    /* setLakeWetlToMaximum (routing.cpp:5647-5716) with resYearOpt=0 */
    st->loclake[n] = (s->loc_lake[n] / 100.) * area * lakedepth;
    st->locwetl[n] = (s->loc_wetl[n] / 100.) * area * wetldepth;
    st->glolake[n] = s->lake_area[n] * lakedepth;
    st->glowetl[n] = (s->glo_wetl[n] / 100.) * area * wetldepth;
    st->res[n] = (s->res_area[n] > 0.) ? s->stor_cap[n] : 0.;
    st->rf_res[n] = 0.;        /* second if/else of routing.cpp:5674-5679 resets it */
    st->rf_loclake[n] = 1.; st->rf_locwetl[n] = 1.; st->rf_glolake[n] = 1.; st->rf_glowetl[n] = 1.;
    st->k_release[n] = 0.1;    /* routing.cpp:443-446 */
    /* initFractionStatus (routing.cpp:748-765) */
    st->fswb_next[n] = s->loc_lake[n] / 100. + s->loc_wetl[n] / 100. + s->glo_wetl[n] / 100.;
    st->laf_started[n] = 0;
    /* annualInit, first year (routing.cpp:1174-1205) */
    double laf = (cont_share(s, n) - (s->glo_lake[n] + s->glo_wetl[n] + s->loc_lake[n] + s->loc_wetl[n] + s->glo_res[n]));
    if (laf < 0.) laf = 0.;
    st->laf[n] = laf;
    st->laf_prev[n] = 0.;
  }
  if (s->river_velo_opt == 2) {
    /* setStoragesToZero: riverveloOpt 2 starts from G_riverStorageMax (routing.cpp:807-812, 488-500) */
    for (int n = 0; n < N; n++) {
      double bf = s->bankfull[n] < 0.05 ? 0.05 : s->bankfull[n];
      double wbf = 2.71 * pow(bf, 0.557);
      double dbf = 0.349 * pow(bf, 0.341);
      double bw = wbf - 2.0 * 2.0 * dbf;
      st->river[n] = s->river_length[n] * 0.5 * dbf / 1000. * (bw / 1000. + wbf / 1000.);
    }
  }
  return 0;
}

/* Per-cell vertical outputs handed to routing (the reference's
 * G_dailyLocalSurfaceRunoff, G_dailyGwRecharge, G_dailyStorageTransfer,
 * G_openWaterPrec, G_openWaterPET) plus the terms of the closure check. */
typedef struct {
  double rs, gwr, transfer, owp, owpet;
  double land_in, land_evap;   /* mm, over the land fraction */
  double land_leak;            /* mm created (+) or lost (-) by the reference's clamps */
} vout;

/* dailyWaterBalanceClass::calcNewDay (daily.cpp:94-1257) for one cell. */
static void vertical_cell(const wgo_static *s, wgo_state *st, int n, short day,
                          double pf, double tf, double swf, vout *o) {
  const int B = s->nband;
  const double landAreaFrac = st->laf[n];
  double prevLAF;
  if (1 == st->laf_started[n]) prevLAF = st->laf_prev[n];       /* daily.cpp:159-169 */
  else prevLAF = landAreaFrac;
  const double cfa = PAR(s, WGO_P_CFA, n);
  const int lct = s->lct[n];
  int arid_gw = 0;
  double dailyPrec = pf, dailyTempC = tf, dailyShortWave = swf;  /* daily.cpp:222-235 */
  double transfer = 0.;   /* G_dailyStorageTransfer: only meaningful when LAF <= 0 */

  dailyPrec = PAR(s, WGO_M_PREC, n) * dailyPrec;                  /* daily.cpp:248 */
  double temp2 = dailyTempC + 237.3;                               /* daily.cpp:250-251 */
  double e_s = 0.6108 * exp(17.27 * dailyTempC / temp2);

  double alpha, a_c, b_c, maxDailyPET;                             /* daily.cpp:322-343 */
  if (s->aindex[n] == 1) {
    alpha = PAR(s, WGO_P_PTC_ARI, n); maxDailyPET = PAR(s, WGO_P_PET_MXDY, n);
    a_c = A_C_ARID; b_c = B_C_ARID; arid_gw = 1;
  } else {
    alpha = PAR(s, WGO_P_PTC_HUM, n); maxDailyPET = PAR(s, WGO_P_PET_MXDY, n);
    a_c = A_C_HUMID; b_c = B_C_HUMID;
  }

  /* LAI (lai.cpp:152-177); LAImin evaluated in float as the reference does */
  float lmin_f = s->lct_lai_a[lct - 1] + s->lct_lai_b[lct - 1] * s->lai_max[n];
  double LAImin = lmin_f, LAImax = s->lai_max[n];
  double dailyLai;
  if (dailyTempC > 8.)
    dailyLai = lai_growing(&st->lai_days[n], s->lct_initial_days[lct - 1], &st->lai_status[n], (char)lct,
                           arid_gw, LAImin, LAImax, &st->lai_precsum[n], dailyPrec);
  else
    dailyLai = lai_nogrowing(&st->lai_days[n], s->lct_initial_days[lct - 1], &st->lai_status[n], (char)lct,
                             arid_gw, LAImin, LAImax, &st->lai_precsum[n], dailyPrec);

  double albedo;                                                   /* daily.cpp:366-379 */
  if (st->snow[n] > 3.) albedo = s->lct_albedo_snow[lct - 1];
  else albedo = s->lct_albedo[lct - 1];

  double lat_heat;                                                 /* daily.cpp:382-387 */
  if (dailyTempC > 0) lat_heat = 2.501 - 0.002361 * dailyTempC;
  else lat_heat = 2.835;

  double ext_rad = calc_ext_rad(day, s->lat_deg[n]);               /* daily.cpp:390 */
  double solar_rad_0 = (A_S + B_S) * ext_rad;
  double conv_Wm2_to_mmd = 0.0864 / lat_heat;
  double solar_rad = conv_Wm2_to_mmd * dailyShortWave;
  double net_long_wave_rad;                                        /* cloud == 2, daily.cpp:430-448 */
  {
    double solar_fraction;
    if (ext_rad == 0.) solar_fraction = 0.;
    else solar_fraction = solar_rad / solar_rad_0;
    if (solar_fraction > 1.) solar_fraction = 1.;
    double ff = a_c * solar_fraction + b_c;
    double net_emissivity = -0.02 + 0.261 * exp(-0.000777 * dailyTempC * dailyTempC);
    double temp_K = dailyTempC + 273.2;
    const double stefan_boltz_const = 0.000000004903;
    net_long_wave_rad = (-ff * net_emissivity * stefan_boltz_const * pow(temp_K, 4.)) / lat_heat;
  }
  double net_short_wave_rad = solar_rad * (1. - albedo);           /* daily.cpp:451-465 */
  double net_rad = PAR(s, WGO_M_NETRAD, n) * (net_short_wave_rad + net_long_wave_rad);
  double openWaterNetShortWaveRad = solar_rad * (1. - OPEN_WATER_ALBEDO);
  double openWaterNetRad = openWaterNetShortWaveRad + net_long_wave_rad;

  double dailyPET = 0., dailyOpenWaterPET = 0.;                    /* daily.cpp:484-532 */
  double atmos_pres = 101.3;
  double inc_svp = 4098. * e_s / (temp2 * temp2);
  double c3 = 0.0016286 * atmos_pres;
  double gamma = c3 / lat_heat;
  if (net_rad <= 0.) dailyPET = 0.;
  else dailyPET = alpha * (inc_svp * net_rad) / (inc_svp + gamma);
  if (openWaterNetRad <= 0.) dailyOpenWaterPET = 0.;
  else dailyOpenWaterPET = alpha * (inc_svp * openWaterNetRad) / (inc_svp + gamma);

  o->owp = dailyPrec;                                              /* daily.cpp:776-777 */
  o->owpet = dailyOpenWaterPET;

  double landStorageChangeSum = 0., initialStorage = 0.;
  double max_canopy_storage = 0., dailyCanopyEvapo = 0., daily_prec_to_soil = 0., dailySoilPET = 0.;
  double canopy_water_content = 0., snowmelt = 0., dailySnowEvapo = 0., dailyEffPrec = 0.;
  double immediate_runoff = 0., surface_runoff = 0., dailyAET = 0., daily_runoff = 0.;
  double total_daily_runoff = 0., daily_gw_recharge = 0., pot_gw_recharge = 0.;
  double soil_saturation = 0., soil_water_overflow = 0., neg_land_aet = 0., neg_runoff = 0.;
  double cellLandAET = 0.;
  double gwr_to_routing = 0.;
  double leak = 0.;

  const double t_snowfz = PAR(s, WGO_P_T_SNOWFZ, n), t_snowmt = PAR(s, WGO_P_T_SNOWMT, n);
  const double t_gradnt = PAR(s, WGO_P_T_GRADNT, n), mdegday = PAR(s, WGO_M_DEGDAY_F, n);

  /* interception, daily.cpp:825-895 */
  if (landAreaFrac <= 0.) {
    transfer = st->canopy[n];
    st->canopy[n] = 0.;
    dailyCanopyEvapo = 0.;
  } else {
    st->canopy[n] *= prevLAF / landAreaFrac;
    if (fabs(st->canopy[n]) <= MIN_STOR_VOL) st->canopy[n] = 0.;
    initialStorage = st->canopy[n];
    if (dailyLai > 0.00001) {
      max_canopy_storage = PAR(s, WGO_P_MCWH, n) * dailyLai;
      double canopy_deficiency = max_canopy_storage - st->canopy[n];
      if (dailyPrec < canopy_deficiency) {
        st->canopy[n] += dailyPrec;
        daily_prec_to_soil = 0.;
      } else {
        st->canopy[n] = max_canopy_storage;
        daily_prec_to_soil = dailyPrec - canopy_deficiency;
      }
      canopy_water_content = st->canopy[n];
      dailyCanopyEvapo = dailyPET * pow((canopy_water_content / max_canopy_storage), CANOPY_EVAPO_EXP);
      if (dailyCanopyEvapo > canopy_water_content) {
        dailyCanopyEvapo = canopy_water_content;
        dailySoilPET = dailyPET - canopy_water_content;
        st->canopy[n] = 0.0;
      } else {
        st->canopy[n] -= dailyCanopyEvapo;
        dailySoilPET = dailyPET - dailyCanopyEvapo;
      }
    } else {
      daily_prec_to_soil = dailyPrec;
      dailySoilPET = dailyPET;
      dailyCanopyEvapo = 0.0;
    }
    landStorageChangeSum += st->canopy[n] - initialStorage;
  }
  if (dailySoilPET < 0.) dailySoilPET = 0.0;

  /* snow in elevation bands, daily.cpp:897-1062 */
  {
    const int16_t *el = s->elev + (size_t)n * (B + 1);
    double *band = st->snow_band + (size_t)n * B;
    double TempElevMax_ = 0.;
    double snowStorageChange = 0.;
    int thresh_elev = 0;
    double gsnow = 0.;
    for (int e = 1; e <= B; e++) {
      double temp_elev, dailyEffPrecBeforeSnowMelt_elev = 0., snowmelt_elev = 0.;
      temp_elev = dailyTempC - ((el[e] - el[0]) * t_gradnt);
      double *sb = &band[e - 1];
      if (landAreaFrac <= 0.) {
        transfer += *sb / (double)B;
        *sb = 0.;
        gsnow = 0.;
      } else {
        *sb = *sb * prevLAF / landAreaFrac;
        if (fabs(*sb) <= MIN_STOR_VOL) *sb = 0.;
        initialStorage = *sb;
        if (*sb > 1000.) {
          if (thresh_elev == 0.) thresh_elev = el[e];
          else if (thresh_elev > 0.) temp_elev = dailyTempC - ((thresh_elev - el[0]) * t_gradnt);
        }
        if (temp_elev <= t_snowfz) {
          dailyEffPrecBeforeSnowMelt_elev = 0.;
          *sb += daily_prec_to_soil;
          if (*sb > dailySoilPET) {
            *sb -= dailySoilPET;
            dailySnowEvapo += dailySoilPET;
          } else {
            dailySnowEvapo += *sb;
            *sb = 0.;
          }
        } else {
          dailyEffPrecBeforeSnowMelt_elev = daily_prec_to_soil;
        }
        if (temp_elev > t_snowmt) {
          if (!(*sb < 0.)) {
            snowmelt_elev = mdegday * s->lct_ddf[lct - 1] * (temp_elev - t_snowmt);
            if (snowmelt_elev > *sb) {
              snowmelt_elev = *sb;
              *sb = 0.;
            } else {
              *sb -= snowmelt_elev;
            }
          }
        }
        double dailyEffPrec_elev = dailyEffPrecBeforeSnowMelt_elev + snowmelt_elev;
        snowStorageChange += *sb - initialStorage;
        if (e == 1) TempElevMax_ = temp_elev;
        gsnow += *sb;
        dailyEffPrec += dailyEffPrec_elev;
        snowmelt += snowmelt_elev;
      }
    }
    if (landAreaFrac > 0.) {
      gsnow /= (double)B;
      dailyEffPrec /= (double)B;
      snowmelt /= (double)B;
      dailySnowEvapo /= (double)B;
      snowStorageChange /= (double)B;
      landStorageChangeSum += snowStorageChange;
    }
    st->snow[n] = gsnow;

    /* immediate runoff, daily.cpp:1068-1071 */
    if (s->built_up[n] > 0.) {
      immediate_runoff = RUNOFF_FRAC_BUILTUP * dailyEffPrec * s->built_up[n];
      dailyEffPrec -= immediate_runoff;
    }

    /* soil and AET, daily.cpp:1080-1239 */
    if (landAreaFrac <= 0.) {
      transfer += st->soil[n];
      transfer *= cfa;
      st->soil[n] = 0.;
      daily_gw_recharge = 0.;
      total_daily_runoff = 0.;
      gwr_to_routing = 0.;
      cellLandAET = 0.;
    } else {
      const double Smax = s->smax[n];
      st->soil[n] *= prevLAF / landAreaFrac;
      initialStorage = st->soil[n];
      soil_water_overflow = 0;
      if (st->soil[n] > Smax) {
        soil_water_overflow = st->soil[n] - Smax;
        st->soil[n] = Smax;
      }
      if (TempElevMax_ > t_snowfz) {
        if (Smax > 0.) {
          soil_saturation = st->soil[n] / Smax;
          daily_runoff = dailyEffPrec * pow(soil_saturation, (double)PAR(s, WGO_P_GAMRUN_C, n));
          if (dailySoilPET > (maxDailyPET - dailyCanopyEvapo) * soil_saturation)
            dailyAET = (maxDailyPET - dailyCanopyEvapo) * soil_saturation;
          else
            dailyAET = dailySoilPET;
          st->soil[n] += dailyEffPrec - dailyAET - daily_runoff;
          if (fabs(st->soil[n]) <= MIN_STOR_VOL) st->soil[n] = 0.;
          dailyEffPrec = 0.;
          if (st->soil[n] < 0.) {
            dailyAET += st->soil[n];
            st->soil[n] = 0.;
          }
          daily_runoff *= cfa;
          immediate_runoff *= cfa;
          const double rgmax = s->rg_max[n] / 100.;
          const float fg = s->gw_factor[n];
          /* daily.cpp:1165 tests the global G_LDD (globals.cpp:8), which no code path of the
           * reference fills (routing.cpp:545 reads routingClass::G_LDD, a different grid), so
           * its "G_LDD[n] >= 0" is true for every cell, inland sinks included. */
          if ((arid_gw) && (s->texture[n] < 21)) {
            pot_gw_recharge = 0.;
            if (rgmax < (fg * daily_runoff)) daily_gw_recharge = rgmax;
            else daily_gw_recharge = fg * daily_runoff;
            if (dailyPrec <= PAR(s, WGO_P_PCRITGWA, n)) {
              pot_gw_recharge = daily_gw_recharge;
              daily_gw_recharge = 0.;
            }
          } else {
            pot_gw_recharge = 0.;
            if (rgmax < (fg * daily_runoff)) daily_gw_recharge = rgmax;
            else daily_gw_recharge = fg * daily_runoff;
          }
          daily_runoff -= pot_gw_recharge;
          pot_gw_recharge /= cfa;
          st->soil[n] += pot_gw_recharge;
          if (st->soil[n] > Smax) {
            soil_water_overflow += st->soil[n] - Smax;
            st->soil[n] = Smax;
          }
          soil_water_overflow *= cfa;
          total_daily_runoff = daily_runoff + immediate_runoff + soil_water_overflow;
        } else {
          total_daily_runoff = 0.;
          daily_gw_recharge = 0.;
        }
      } else {
        soil_water_overflow *= cfa;
        dailyEffPrec *= cfa;
        total_daily_runoff += soil_water_overflow + dailyEffPrec;
        leak -= cfa * immediate_runoff;   /* built-up runoff is dropped in this branch */
        daily_gw_recharge = 0.;
        dailyAET = 0.;
      }
      gwr_to_routing = daily_gw_recharge;              /* daily.cpp:1232 */
      landStorageChangeSum += st->soil[n] - initialStorage;
      cellLandAET = landStorageChangeSum * (cfa - 1.0) - dailyPrec * (cfa - 1.0)
                    + (dailyAET + dailyCanopyEvapo + dailySnowEvapo) * cfa;
      if (cellLandAET < 0.) {
        neg_land_aet = cellLandAET;
        cellLandAET = 0.;
      }
    }
  }
  /* surface runoff, daily.cpp:1244-1257 */
  if (neg_land_aet < 0.) total_daily_runoff = total_daily_runoff + neg_land_aet;
  if (total_daily_runoff < 0.) { leak -= total_daily_runoff; total_daily_runoff = 0.; }
  if ((total_daily_runoff - daily_gw_recharge) < 0.) {
    neg_runoff = total_daily_runoff - daily_gw_recharge;
    daily_gw_recharge = total_daily_runoff;
    st->soil[n] += neg_runoff;
    neg_runoff = 0.;
  }
  surface_runoff = total_daily_runoff - daily_gw_recharge;
  o->rs = surface_runoff;
  o->gwr = gwr_to_routing;
  o->transfer = transfer;
  o->land_in = dailyPrec;
  o->land_evap = cellLandAET;
  o->land_leak = leak;
  (void)snowmelt; (void)canopy_water_content; (void)max_canopy_storage; (void)soil_saturation;
}

/* getRiverVelocity / getNewRiverVelocity (routing.cpp:7274-7341) */
static double river_velocity(const wgo_static *s, const wgo_state *st, int n, double riverInflow, double bw) {
  const double slope = s->river_slope[n], rough = s->roughness[n];
  const double m = PAR(s, WGO_M_RIVRGH_C, n);
  double v;
  if (s->river_velo_opt == 1) {
    double incoming_discharge = (riverInflow * 1000. * 1000. * 1000.) / (60. * 60. * 24.);
    double riverDepth = 0.349 * pow(incoming_discharge, 0.341);
    double crossSectionalArea = riverDepth * (2.0 * riverDepth + bw);
    double wettedPerimeter = bw + 2.0 * riverDepth * sqrt(5.0);
    double hydraulicRad = crossSectionalArea / wettedPerimeter;
    v = 1. / (m * rough) * pow(hydraulicRad, (2. / 3.)) * pow(slope, 0.5);
  } else {
    double crossSectionalArea = (st->river[n] / s->river_length[n]) * 1000000.;
    double riverDepth = -bw / 4.0 + sqrt(bw * bw / 16.0 + 0.5 * crossSectionalArea);
    double wettedPerimeter = bw + 2.0 * riverDepth * sqrt(5.0);
    double hydraulicRad = crossSectionalArea / wettedPerimeter;
    v = 1. / (m * rough) * pow(hydraulicRad, (2. / 3.)) * pow(slope, 0.5);
  }
  v = v * 86.4;
  if (v < 0.00001) return 0.00001;
  return v;
}

static double storage_km3(const wgo_static *s, const wgo_state *st, int n, double laf) {
  const int B = s->nband;
  /* land storages in mm over the land fraction; snow as the band mean */
  double snow = 0.;
  for (int b = 0; b < B; b++) snow += st->snow_band[(size_t)n * B + b];
  snow /= (double)B;
  double f = s->area_km2[n] * (laf / 100.) / 1000000.;
  return (st->canopy[n] + snow + st->soil[n]) * f + st->gw[n] + st->river[n] + st->loclake[n] +
         st->locwetl[n] + st->glolake[n] + st->glowetl[n] + st->res[n];
}

static double state_volume(const wgo_static *s, const wgo_state *st, int n) {
  /* land storage is held in mm of the land fraction it was last rescaled to */
  return storage_km3(s, st, n, st->laf_started[n] ? st->laf_prev[n] : st->laf[n]);
}

/* one day's inputs of the water temperature that routing produces for a cell
 * (routing.cpp:4287-4356): the water bodies' storages before the day, their
 * evaporation [mm] after any reduction, the area reduction factors the day
 * started with, and the outflows of each water body */
typedef struct {
  double loclake_prev, loclake_max, loclake_evapo, loclake_rf, loclake_out;
  double locwetl_prev, locwetl_evapo, locwetl_rf, locwetl_out;
  double glolake_prev, glolake_max, glolake_evapo, glolake_out;
  double res_prev, res_evapo, res_out;
  double glowetl_prev, glowetl_evapo, glowetl_rf, glowetl_out;
} wt_route;

/* wall time of the passes of the last run (the CPU baseline's split) */
static double g_time_vertical, g_time_routing;

void wgo_last_timing(double out[2]) {
  out[0] = g_time_vertical;
  out[1] = g_time_routing;
}

static double wall_now(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0.;
#endif
}

static int run_impl(const wgo_static *s, wgo_state *st, int doy0, int ndays, const float *prec,
                    const float *temp, const float *swrad, double *discharge, double *balance, int nthreads,
                    wgo_wt_io *wt, wgo_wu_io *wu);

int wgo_run(const wgo_static *s, wgo_state *st, int doy0, int ndays, const float *prec,
            const float *temp, const float *swrad, double *discharge, double *balance, int nthreads) {
  return run_impl(s, st, doy0, ndays, prec, temp, swrad, discharge, balance, nthreads, NULL, NULL);
}

int wgo_run_wu(const wgo_static *s, wgo_state *st, int doy0, int ndays, const float *prec,
               const float *temp, const float *swrad, double *discharge, double *balance, int nthreads,
               wgo_wu_io *wu) {
  if (!wu || !wu->nus || !wu->nug || !wu->wdr || !wu->cons || !wu->row_of_day || !wu->frgi || !wu->state)
    return -1;
  return run_impl(s, st, doy0, ndays, prec, temp, swrad, discharge, balance, nthreads, NULL, wu);
}

int wgo_run_wt_wu(const wgo_static *s, wgo_state *st, int doy0, int ndays, const float *prec,
                  const float *temp, const float *swrad, double *discharge, double *balance, int nthreads,
                  wgo_wt_io *wt, wgo_wu_io *wu) {
  if (!wt || !wt->longwave || !wt->gw_temp || !wt->inflow_cells || !wt->river_length_check || !wt->temp ||
      !wt->ice || !wt->river_avail)
    return -1;
  if (!wu || !wu->nus || !wu->nug || !wu->wdr || !wu->cons || !wu->row_of_day || !wu->frgi || !wu->state)
    return -1;
  return run_impl(s, st, doy0, ndays, prec, temp, swrad, discharge, balance, nthreads, wt, wu);
}

/* routingClass::updateNetAbstractionGW (routing.cpp:5503-5572): the day's NAg
 * after the previous day's unsatisfied surface-water demand (w: the water-use
 * state rows of the cell, stride N) */
static double update_nag(double *w, size_t N, double nug, double frgi) {
  double *rem = &w[0], *ui = &w[1 * N], *uo = &w[2 * N], *rrf = &w[3 * N];
  const double wdr = w[4 * N], cons = w[5 * N];
  if (*rem > 1.e-12) {
    if (wdr > 0.) {
      double eff = cons / wdr;
      double factor = 1 - (1 - frgi) * (1 - eff);
      double WUsiNew = 1 / factor * (wdr * factor - *rem);
      if (WUsiNew < 0.) {
        WUsiNew = 0.;
        *ui += wdr * factor;
        *uo += *rem - (wdr * factor);
      } else {
        *ui += *rem;
      }
      double returnflowChange = (frgi * (1 - eff) * (WUsiNew - wdr));
      *rrf += returnflowChange;
      *rem = 0.;
      return nug - returnflowChange;
    }
    *uo += *rem;
    return nug;
  } else if (*rem < -1.e-12) {
    double fromIrrig = *rem + *uo;
    if (fromIrrig < 0.) {
      *uo = 0.;
    } else {
      *uo += *rem;
      *rem = 0.;
      return nug;
    }
    if (*ui == 0.) {
      *rem = 0.;
      return nug;
    }
    double ratio = (fromIrrig / *ui);
    if (ratio < -1.) {
      ratio = -1.;
      fromIrrig = *ui * -1.;
    }
    double returnflowChange = (ratio * *rrf);
    *ui += fromIrrig;
    *rrf += returnflowChange;
    *rem = 0.;
    return nug - returnflowChange;
  }
  return nug;
}

int wgo_run_wt(const wgo_static *s, wgo_state *st, int doy0, int ndays, const float *prec,
               const float *temp, const float *swrad, double *discharge, double *balance, int nthreads,
               wgo_wt_io *wt) {
  if (!wt || !wt->longwave || !wt->gw_temp || !wt->inflow_cells || !wt->river_length_check || !wt->temp ||
      !wt->ice || !wt->river_avail)
    return -1;
  return run_impl(s, st, doy0, ndays, prec, temp, swrad, discharge, balance, nthreads, wt, NULL);
}

void wgo_wt_init(int ncell, wgo_wt_io *wt) {
  for (int k = 0; k < 6 * ncell; k++) {
    wt->temp[k] = 15.;
    wt->ice[k] = 0.;
  }
  for (int n = 0; n < ncell; n++) wt->river_avail[n] = 0.;
}

/* the water temperature of cell n after its routing (routing.cpp:4241-4513) */
static void cell_water_temp(const wgo_static *s, const wgo_state *st, int n, int d, double cellArea, double cfa,
                            const vout *vo, double localRunoff, double gw_runoff, double into_river,
                            double gw_into_river, const wt_route *r, double transportedVolume, double bw, float Tair,
                            float SWin, wgo_wt_io *wt) {
  const int N = s->ncell;
  wgo_wt_in t;
  t.calc_temp_pp = 0.; t.pp_withdrawal = 0.; t.pp_consumption = 0.;
  for (int i = 0; i < 9; i++) {
    const int m = wt->inflow_cells[(size_t)n * 9 + i];
    if (m >= 0) {
      t.inflow[i] = wt->river_avail[m];
      t.inflow_temp[i] = wt->temp[m];
    } else if (i == 4) {
      t.inflow[i] = 0.;
      t.inflow_temp[i] = wt->temp[n];
    } else {
      t.inflow[i] = 0.;
      t.inflow_temp[i] = 15.;
    }
  }
  for (int k = 0; k < 6; k++) t.ice[k] = wt->ice[(size_t)k * N + n];
  t.short_rad = (double)SWin;
  t.long_rad = (double)wt->longwave[(size_t)d * N + n];
  t.air_temp = (double)Tair;
  t.gw_temp = wt->gw_temp[n] < 0.f ? 0. : (double)wt->gw_temp[n];
  t.cfa = cfa;
  t.ow_pet = vo->owpet;
  t.ow_prec = vo->owp;
  t.cell_area = cellArea;
  t.loclake_area = s->loc_lake[n];
  t.loclake_stor_prev = r->loclake_prev + r->loclake_max;
  t.loclake_temp_prev = wt->temp[(size_t)1 * N + n];
  t.loclake_evapo = r->loclake_evapo;
  t.loclake_rf = r->loclake_rf;
  t.local_runoff = localRunoff;
  t.local_gw_runoff = gw_runoff;
  t.locwetl_area = s->loc_wetl[n];
  t.locwetl_stor_prev = r->locwetl_prev;
  t.locwetl_temp_prev = wt->temp[(size_t)2 * N + n];
  t.locwetl_evapo = r->locwetl_evapo;
  t.locwetl_rf = r->locwetl_rf;
  t.locwetl_inflow = r->loclake_out;
  t.locwetl_outflow = r->locwetl_out;
  t.glolake_area = s->lake_area[n];
  t.glolake_stor_prev = r->glolake_prev + r->glolake_max;
  t.glolake_temp_prev = wt->temp[(size_t)3 * N + n];
  t.glolake_evapo = r->glolake_evapo;
  t.glolake_inflow = 0.;
  for (int i = 0; i < 9; i++) t.glolake_inflow += t.inflow[i];
  if (s->loc_wetl[n] > 0.) t.glolake_inflow += r->locwetl_out;
  else if (s->loc_lake[n] > 0.) t.glolake_inflow += r->loclake_out;
  t.res_inflow = s->lake_area[n] > 0. ? r->glolake_out : t.glolake_inflow;
  t.res_area = s->res_area[n];
  t.res_stor_prev = r->res_prev;
  t.res_temp_prev = wt->temp[(size_t)4 * N + n];
  t.res_evapo = r->res_evapo;
  if (s->res_area[n] > 0.) t.glowetl_inflow = r->res_out;
  else if (s->lake_area[n] > 0.) t.glowetl_inflow = r->glolake_out;
  else t.glowetl_inflow = t.glolake_inflow;
  t.glowetl_area = s->glo_wetl[n];
  t.glowetl_stor_prev = r->glowetl_prev;
  t.glowetl_temp_prev = wt->temp[(size_t)5 * N + n];
  t.glowetl_evapo = r->glowetl_evapo;
  t.glowetl_rf = r->glowetl_rf;
  if (s->glo_wetl[n] > 0.) t.river_inflow = r->glowetl_out;
  else if (s->res_area[n] > 0.) t.river_inflow = r->res_out;
  else if (s->lake_area[n] > 0.) t.river_inflow = r->glolake_out;
  else t.river_inflow = t.glolake_inflow;
  t.river_stor = st->river[n];
  t.gw_runoff_into_river = gw_into_river;   /* zero without fractional routing */
  t.runoff_into_river = into_river;
  t.river_bottom_width = bw;
  t.river_length = s->river_length[n];
  t.river_length_check = wt->river_length_check[n];
  t.has_outflow = s->downstream[n] >= 0 ? 1. : 0.;
  double out[12];
  wgo_wtemp(&t, out);
  for (int k = 0; k < 6; k++) wt->ice[(size_t)k * N + n] = out[6 + k];
  if (wt->daily_temp) wt->daily_temp[(size_t)d * N + n] = out[0];
  for (int k = 0; k < 6; k++)
    wt->temp[(size_t)k * N + n] = out[k] == -9999. ? (t.air_temp < 0. ? 0. : t.air_temp) : out[k];
  wt->river_avail[n] = transportedVolume;
}

static const int days_in_month[12] = {31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31};   /* routing.cpp:107 */

/* GLWD units (aggrNUsGloLakResOpt): the cells of every unit > 0 in cell order;
 * per cell its unit's range [lo, hi) in cells.  Returns 0, or -1 where an
 * outflow cell (lake_area or res_area > 0) has unit 0 or a unit has two outflow
 * cells (the reference's loops would then aggregate over every cell without a
 * unit, or twice). */
typedef struct {
  int *cells, *lo, *hi;
} glwd_lists;

static const int32_t *g_unit_key;
static int cmp_unit_cell(const void *a, const void *b) {
  const int i = *(const int *)a, j = *(const int *)b;
  if (g_unit_key[i] != g_unit_key[j]) return g_unit_key[i] < g_unit_key[j] ? -1 : 1;
  return i < j ? -1 : (i > j);
}

static int glwd_build(int N, const double *lake_area, const double *res_area, const int32_t *unit, glwd_lists *g) {
  const size_t cap = (size_t)(N > 0 ? N : 1);
  g->cells = (int *)malloc(sizeof(int) * cap);
  g->lo = (int *)malloc(sizeof(int) * cap);
  g->hi = (int *)malloc(sizeof(int) * cap);
  if (!g->cells || !g->lo || !g->hi) return -2;
  int m = 0;
  for (int i = 0; i < N; i++) {
    g->lo[i] = g->hi[i] = 0;
    if (unit[i] > 0) g->cells[m++] = i;
  }
  g_unit_key = unit;
  qsort(g->cells, (size_t)m, sizeof(int), cmp_unit_cell);
  for (int k = 0; k < m;) {
    int e = k, outflows = 0;
    while (e < m && unit[g->cells[e]] == unit[g->cells[k]]) {
      const int c = g->cells[e];
      if (lake_area[c] > 0. || res_area[c] > 0.) outflows++;
      e++;
    }
    if (outflows > 1) return -1;
    for (int j = k; j < e; j++) {
      g->lo[g->cells[j]] = k;
      g->hi[g->cells[j]] = e;
    }
    k = e;
  }
  for (int i = 0; i < N; i++)
    if ((lake_area[i] > 0. || res_area[i] > 0.) && unit[i] <= 0) return -1;
  return 0;
}

static void glwd_free(glwd_lists *g) {
  free(g->cells); free(g->lo); free(g->hi);
  g->cells = g->lo = g->hi = NULL;
}

/* routing.cpp:926-965, one month */
int wgo_aggregate_nus(int ncell, const double *lake_area, const double *res_area, const int32_t *glwd_unit,
                      const double *nus, double *out) {
  glwd_lists g = {NULL, NULL, NULL};
  const int rc = glwd_build(ncell, lake_area, res_area, glwd_unit, &g);
  if (rc == 0) {
    for (int n = 0; n < ncell; n++) out[n] = nus[n];
    for (int n = 0; n < ncell; n++) {
      if (!(lake_area[n] > 0. || res_area[n] > 0.)) continue;   /* an outflow cell */
      for (int k = g.lo[n]; k < g.hi[n]; k++) {
        const int i = g.cells[k];
        if (i == n) continue;
        if (nus[i] > 0.) {
          out[n] += out[i];
          out[i] = 0.;
        }
      }
    }
  }
  glwd_free(&g);
  return rc;
}

static int run_impl(const wgo_static *s, wgo_state *st, int doy0, int ndays, const float *prec,
                    const float *temp, const float *swrad, double *discharge, double *balance, int nthreads,
                    wgo_wt_io *wt, wgo_wu_io *wu) {
  const int N = s->ncell;
  if (s->nband <= 0 || N <= 0) return -1;
  /* zero: the terms of cells without continental area, which the vertical pass
     never writes (the reference's zero-initialised grids, daily.cpp:1670-1676) */
  vout *vo = (vout *)calloc((size_t)N, sizeof(vout));
  double *inflow_up = (double *)calloc((size_t)N, sizeof(double));
  double *bw = (double *)malloc(sizeof(double) * (size_t)N);
  if (!vo || !inflow_up || !bw) return -2;
  for (int n = 0; n < N; n++) bw[n] = wgo_bottom_width(s->bankfull[n]);
  glwd_lists glwd = {NULL, NULL, NULL};
  if (wu && wu->nus_agg) {
    const int rc = wu->glwd_unit ? glwd_build(N, s->lake_area, s->res_area, wu->glwd_unit, &glwd) : -1;
    if (rc) {
      glwd_free(&glwd);
      free(vo); free(inflow_up); free(bw);
      return -3;
    }
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  g_time_vertical = g_time_routing = 0.;
  double s_prev = 0.;
  if (balance)
    for (int n = 0; n < N; n++) s_prev += state_volume(s, st, n);
  int doy = doy0;
  for (int d = 0; d < ndays; d++) {
    short day = (short)doy;
    int month = 0;
    while (month < 11 && day >= first_day_in_month[month + 1]) month++;
    const float *P = prec + (size_t)d * N, *T = temp + (size_t)d * N, *SW = swrad + (size_t)d * N;
    /* vertical pass: the reference's OpenMP cell loop over continental cells
       (integrateWGHM.cpp:767-783; G_contcell, geo.cpp:50-60) */
    const double w0 = wall_now();
#pragma omp parallel for schedule(static) if (nthreads > 1)
    for (int n = 0; n < N; n++)
      if (!(cont_share(s, n) < WGO_LIMIT_CONTCELL_PCT))
        vertical_cell(s, st, n, day, (double)P[n], (double)T[n], (double)SW[n], &vo[n]);
    const double w1 = wall_now();
    g_time_vertical += w1 - w0;

    double b_in = 0., b_evap = 0., b_out = 0., b_leak = 0.;
    double *W = wu ? wu->state : NULL;
    const size_t wo = wu ? (size_t)wu->row_of_day[d] * (size_t)N : 0;
#define WU(k) W[(size_t)(k) * (size_t)N + (size_t)n]
    if (wu && day == 1)   /* annualInit (routing.cpp:994-1010) */
      for (int n = 0; n < N; n++) {
        WU(7) = WU(6); WU(8) = WU(1); WU(9) = WU(2); WU(10) = WU(3);
        WU(11) = 0.;
      }
    /* routing sweep in routing order (routing.cpp:1830-4520) */
    for (int n = 0; n < N; n++) inflow_up[n] = 0.;
    for (int rc = 0; rc < N; rc++) {
      const int n = s->rout_order[rc];
      if (cont_share(s, n) < WGO_LIMIT_CONTCELL_PCT) {
        /* only continental cells are routed (routing.cpp:1878-4518): the storages
           stay, nothing flows on, the inflow stays behind in G_riverInflow and so
           leaves the system (a negative leak); the water temperature keeps its
           start value */
        if (discharge) discharge[(size_t)d * N + n] = 0.;
        if (wt && wt->daily_temp) wt->daily_temp[(size_t)d * N + n] = wt->temp[n];
        if (balance) b_leak -= inflow_up[n];
        continue;
      }
      const double cellArea = s->area_km2[n];
      const double cfa = PAR(s, WGO_P_CFA, n);
      const double laf = st->laf[n];
      double p_ow = 0., e_ow = 0.;
      double dailyLocalSurfaceRunoff;
      if (laf <= 0.)
        dailyLocalSurfaceRunoff = vo[n].transfer * cellArea / 1000000. * st->laf_prev[n] / 100.;
      else
        dailyLocalSurfaceRunoff = vo[n].rs * cellArea / 1000000. * laf / 100.;
      /* groundwater (routing.cpp:2091-2146 non-sink, 2148-2200 sink) */
      const double kg = PAR(s, WGO_P_GWOUTF_C, n);
      double gwPrev = st->gw[n];
      double netGWin = vo[n].gwr * cellArea * (laf / 100.) / 1000000.;
      double remainingUse = 0., dailyActualUse = 0., nug = 0., prevTotalUnsat = 0., totalDesiredUse = 0.;
      if (wu) {   /* routing.cpp:1926-1933 and the other groundwater variants */
        nug = wu->nug[wo + n];
        if (WU(0) != 0.) nug = update_nag(&WU(0), (size_t)N, nug, wu->frgi[n]);
        netGWin -= nug;
        e_ow += nug;
        remainingUse = wu->nus[wo + n];   /* routing.cpp:2225-2290 */
        if (wu->nus_agg) {                /* routing.cpp:2199-2222 */
          if (s->res_area[n] > 0. || s->lake_area[n] > 0.) remainingUse = wu->nus_agg[wo + n];
          else if (wu->glwd_unit[n] > 0) remainingUse = wu->nus_agg[wo + n] + WU(12);
        }
        if (wu->delayed) {                /* routing.cpp:2236-2244 */
          remainingUse += WU(6);
          prevTotalUnsat = WU(6);
          WU(6) = 0.;
        }
        totalDesiredUse = remainingUse;
      }
      st->gw[n] = gwPrev * exp(-1. * kg) + (1. / kg) * netGWin * (1. - exp(-1. * kg));
      if (fabs(st->gw[n]) <= MIN_STOR_VOL) st->gw[n] = 0.;
      double gw_runoff = gwPrev - st->gw[n] + netGWin;
      if (gw_runoff <= 0.) {
        gw_runoff = 0.;
        st->gw[n] = gwPrev + netGWin;
        if (fabs(st->gw[n]) <= MIN_STOR_VOL) st->gw[n] = 0.;
      }
      double localRunoff;
      double into_river = 0., gw_into_river = 0., local_gw = gw_runoff;
      if (s->frac_routing && s->ldd[n] >= 0) {
        /* fractional routing, routing.cpp:1897-1907, 1911-1915 (arid), 2024-2033 (humid):
         * the part of the runoff from outside the water bodies' catchment (20 times
         * their initial area) flows directly into the river; arid cells send all
         * their groundwater runoff there */
        double fc = (s->loc_lake[n] / 100. + s->loc_wetl[n] / 100. + s->glo_wetl[n] / 100.) * 20.;
        if (fc > 1.) fc = 1.;
        into_river = (1. - fc) * dailyLocalSurfaceRunoff;
        if (s->aindex[n] == 1) {
          local_gw = 0.;
          localRunoff = fc * dailyLocalSurfaceRunoff;
          gw_into_river = gw_runoff;
        } else {
          gw_into_river = (1. - fc) * gw_runoff;
          local_gw = fc * gw_runoff;
          localRunoff = (fc * dailyLocalSurfaceRunoff) + local_gw;
        }
      } else if (s->ldd[n] >= 0) {
        localRunoff = dailyLocalSurfaceRunoff;
        localRunoff += gw_runoff;
      } else {
        if (laf == 0.)
          dailyLocalSurfaceRunoff = vo[n].transfer * cellArea / 1000000. * st->laf_prev[n] / 100.;
        else
          dailyLocalSurfaceRunoff = vo[n].rs * cellArea / 1000000. * laf / 100.;
        localRunoff = dailyLocalSurfaceRunoff + gw_runoff;
      }
      const double swoutf = PAR(s, WGO_P_SWOUTF_C, n);
      const double evaredex = PAR(s, WGO_M_EVAREDEX, n);
      const double lakeDepth = PAR(s, WGO_P_LAK_D, n) * 0.001;
      const double wetlDepth = PAR(s, WGO_P_WET_D, n) * 0.001;
      const double owp = vo[n].owp, owpet = vo[n].owpet;
      double inflow = localRunoff, outflow = 0., maxStorage, totalInflow, PETgwr, PETgwrMax;
      wt_route wr;
      memset(&wr, 0, sizeof wr);

      /* local lake, routing.cpp:2318-2490 */
      if (s->loc_lake[n] > 0.) {
        double S0 = st->loclake[n];
        maxStorage = ((s->loc_lake[n]) / 100.) * cellArea * lakeDepth;
        double rf = st->rf_loclake[n];
        double evapo = ((1.0 - cfa) * owp * rf) + (cfa * (owpet * rf));
        if (evapo < 0.) evapo = 0.;
        double pin = (owp * rf) * (cellArea / 1000000.) * (s->loc_lake[n] / 100.);
        totalInflow = inflow + pin;
        PETgwr = evapo * (cellArea / 1000000.) * (s->loc_lake[n] / 100.);
        PETgwrMax = S0 + maxStorage + totalInflow;
        const double avail = PETgwrMax;
        if (PETgwrMax < 0.) PETgwrMax = 0.;
        wr.loclake_prev = S0; wr.loclake_max = maxStorage; wr.loclake_rf = rf;
        if (PETgwr > PETgwrMax) {
          st->loclake[n] = (-1.) * maxStorage;
          e_ow += avail;
          evapo *= PETgwrMax / PETgwr;
        } else {
          st->loclake[n] = S0 + totalInflow - PETgwr;
          e_ow += PETgwr;
        }
        p_ow += pin;
        if (S0 > 0.) {
          outflow = swoutf * S0 * pow((S0 / maxStorage), LAKE_OUTFLOW_EXP);
          if (st->loclake[n] <= 0.) outflow = 0;
          else if (outflow > st->loclake[n]) outflow = st->loclake[n];
        } else outflow = 0.;
        st->loclake[n] -= outflow;
        if (fabs(st->loclake[n]) <= MIN_STOR_VOL) st->loclake[n] = 0.;
        if (st->loclake[n] > maxStorage) {
          outflow += (st->loclake[n] - maxStorage);
          st->loclake[n] = maxStorage;
        }
        inflow = outflow;
        wr.loclake_evapo = evapo; wr.loclake_out = outflow;
        st->rf_loclake[n] = 1. - pow(fabs(st->loclake[n] - maxStorage) / (2. * maxStorage), (evaredex * EVAPO_RED_EXP));
        if (st->rf_loclake[n] < 0.) st->rf_loclake[n] = 0.;
        if (st->rf_loclake[n] > 1.) st->rf_loclake[n] = 1.;
      }
      /* local wetland, routing.cpp:2495-2617 */
      if (s->loc_wetl[n] > 0.) {
        double S0 = st->locwetl[n];
        maxStorage = ((s->loc_wetl[n]) / 100.) * cellArea * wetlDepth;
        double rf = st->rf_locwetl[n];
        double evapo = ((1.0 - cfa) * owp * rf) + (cfa * (owpet * rf));
        if (evapo < 0.) evapo = 0.;
        double pin = (owp * rf * (cellArea / 1000000.) * (s->loc_wetl[n] / 100.));
        totalInflow = inflow + pin;
        PETgwr = evapo * (cellArea / 1000000.) * (s->loc_wetl[n] / 100.);
        PETgwrMax = S0 + totalInflow;
        wr.locwetl_prev = S0; wr.locwetl_rf = rf;
        if (PETgwr > PETgwrMax) {
          st->locwetl[n] = 0.;
          e_ow += PETgwrMax;
          evapo *= PETgwrMax / PETgwr;
        } else {
          st->locwetl[n] = S0 + totalInflow - PETgwr;
          e_ow += PETgwr;
        }
        p_ow += pin;
        if (fabs(st->locwetl[n]) <= MIN_STOR_VOL) st->locwetl[n] = 0.;
        if (st->locwetl[n] > 0.) {
          outflow = swoutf * st->locwetl[n] * pow((st->locwetl[n] / maxStorage), WETL_OUTFLOW_EXP);
          if (outflow > st->locwetl[n]) outflow = st->locwetl[n];
        } else outflow = 0.;
        st->locwetl[n] -= outflow;
        if (st->locwetl[n] > maxStorage) {
          outflow += (st->locwetl[n] - maxStorage);
          st->locwetl[n] = maxStorage;
        }
        inflow = outflow;
        wr.locwetl_evapo = evapo; wr.locwetl_out = outflow;
        st->rf_locwetl[n] = 1. - pow(fabs(st->locwetl[n] - maxStorage) / (maxStorage), (evaredex * EVAPO_RED_EXP));
        if (st->rf_locwetl[n] < 0.) st->rf_locwetl[n] = 0.;
        if (st->rf_locwetl[n] > 1.) st->rf_locwetl[n] = 1.;
      }
      /* upstream inflow, routing.cpp:2623-2624 */
      inflow += inflow_up[n];
      const double inflowUpstream = inflow_up[n];
      (void)inflowUpstream;   /* CellRunoff output only (routing.cpp:3941-3946) */
      double remUseGloLake = 0., remUseRes = 0.;
      /* global lake, routing.cpp:2630-2804 */
      if (s->lake_area[n] > 0.) {
        double S0 = st->glolake[n];
        maxStorage = (s->lake_area[n]) * lakeDepth;
        double rf = st->rf_glolake[n];
        double evapo = ((1.0 - cfa) * owp) + (cfa * owpet * rf);
        if (evapo < 0.) evapo = 0.;
        double pin = (owp * (s->lake_area[n] / 1000000.));
        totalInflow = inflow + pin;
        double PETgwrRemUse = evapo * (s->lake_area[n] / 1000000.);
        double remUseStart = 0.;
        if (wu) {   /* routing.cpp:2676-2692 */
          remUseGloLake = (s->res_area[n] > 0.) ? 0.5 * remainingUse : remainingUse;
          remUseStart = remUseGloLake;
          PETgwrRemUse += remUseGloLake;
        }
        double PETgwrRemUseMax = totalInflow + maxStorage + S0;
        p_ow += pin;
        wr.glolake_prev = S0; wr.glolake_max = maxStorage;
        if (PETgwrRemUse > PETgwrRemUseMax) {
          st->glolake[n] = (-1.) * maxStorage;
          outflow = 0.;
          e_ow += PETgwrRemUseMax;
          evapo *= PETgwrRemUseMax / PETgwrRemUse;
          if (remUseGloLake > 0.) remUseGloLake -= remUseGloLake * PETgwrRemUseMax / PETgwrRemUse;
          else remUseGloLake = 0.;
        } else {
          remUseGloLake = 0.;
          st->glolake[n] = S0 * exp(-1. * swoutf) + (1. / swoutf) * (totalInflow - PETgwrRemUse) * (1. - exp(-1. * swoutf));
          outflow = totalInflow + S0 - st->glolake[n] - PETgwrRemUse;
          if (st->glolake[n] > maxStorage) {
            outflow += (st->glolake[n] - maxStorage);
            st->glolake[n] = maxStorage;
          }
          if (outflow < 0.) {
            outflow = 0.;
            st->glolake[n] = S0 + totalInflow - PETgwrRemUse;
          }
          e_ow += PETgwrRemUse;
        }
        if (fabs(st->glolake[n]) <= MIN_STOR_VOL) st->glolake[n] = 0.;
        inflow = outflow;
        dailyActualUse = remUseStart - remUseGloLake;   /* routing.cpp:2788 */
        wr.glolake_evapo = evapo; wr.glolake_out = outflow;
        st->rf_glolake[n] = 1. - pow(fabs(st->glolake[n] - maxStorage) / (2. * maxStorage), (evaredex * EVAPO_RED_EXP));
        if (st->rf_glolake[n] < 0.) st->rf_glolake[n] = 0.;
        if (st->rf_glolake[n] > 1.) st->rf_glolake[n] = 1.;
      }
      /* reservoir, routing.cpp:2807-3082 */
      if (s->res_area[n] > 0.) {
        double c_ratio = s->stor_cap[n] / (s->mean_outflow[n] * 31536000. / 1000000000.);
        maxStorage = s->stor_cap[n];
        double S0 = st->res[n];
        double rf = st->rf_res[n];
        double evapo = ((1.0 - cfa) * owp) + (cfa * (owpet * rf));
        if (evapo < 0.) evapo = 0.;
        double pin = (owp * (s->res_area[n] / 1000000.));
        totalInflow = inflow + pin;
        PETgwr = evapo * (s->res_area[n] / 1000000.);
        PETgwrMax = S0 + totalInflow;
        p_ow += pin;
        wr.res_prev = S0;
        double remUseResStart = 0.;
        if (wu) {   /* routing.cpp:2869-2877 */
          if (s->lake_area[n] > 0.) remUseRes = 0.5 * remainingUse + remUseGloLake;
          else remUseRes = remainingUse;
          remUseResStart = remUseRes;
        }
        if (PETgwr > PETgwrMax) {
          st->res[n] = S0 + totalInflow - PETgwrMax;
          e_ow += PETgwrMax;
          evapo *= PETgwrMax / PETgwr;
        } else {
          st->res[n] = S0 + totalInflow - PETgwr;
          e_ow += PETgwr;
        }
        if (wu) {   /* routing.cpp:2922-2946 */
          if (remUseRes < 0.) {
            st->res[n] -= remUseRes;
            e_ow += remUseRes;
            remUseRes = 0.;
          } else if (st->res[n] > (s->stor_cap[n] * 0.1)) {
            if (remUseRes < (st->res[n] - (s->stor_cap[n] * 0.1))) {
              st->res[n] -= remUseRes;
              e_ow += remUseRes;
              remUseRes = 0.;
            } else {
              const double used = (st->res[n] - (s->stor_cap[n] * 0.1));
              remUseRes -= used;
              st->res[n] = s->stor_cap[n] * 0.1;
              e_ow += used;
            }
          }
        }
        if (fabs(st->res[n]) <= MIN_STOR_VOL) st->res[n] = 0.;
        if (month == s->start_month[n] - 1) {
          if (day == first_day_in_month[month]) {
            if (st->res[n] < (s->stor_cap[n] * 0.1)) st->k_release[n] = 0.1;
            else st->k_release[n] = st->res[n] / (maxStorage * 0.85);
          }
        }
        double prov_rel;
        if (s->res_type[n] == 1) {
          /* routing.cpp:2974-2988; the downstream allocation coefficients are zero */
          double dailyUse = wu ? wu->nus[wo + n] : 0.0;
          double monthlyUse = dailyUse * days_in_month[month];
          monthlyUse = monthlyUse * 1000000000. / (days_in_month[month] * 86400.);
          if (s->mean_demand[n] >= 0.5 * s->mean_outflow[n])
            prov_rel = s->mean_outflow[n] / 2. * (1. + monthlyUse / s->mean_demand[n]);
          else
            prov_rel = s->mean_outflow[n] + monthlyUse - s->mean_demand[n];
        } else {
          prov_rel = s->mean_outflow[n];
        }
        double release;
        if (c_ratio >= 0.5) release = st->k_release[n] * prov_rel;
        else
          release = ((4. * c_ratio * c_ratio) * st->k_release[n] * prov_rel) +
                    ((1.0 - ((4. * c_ratio * c_ratio))) * inflow * 1000000000. / (24. * 3600.));
        if (st->res[n] >= (s->stor_cap[n] * 0.1)) outflow = release * (24. * 3600.) / 1000000000.;
        else outflow = 0.1 * release * (24. * 3600.) / 1000000000.;
        if (outflow < 0.) outflow = 0.;
        st->res[n] -= outflow;
        if (st->res[n] > maxStorage) {
          outflow += (st->res[n] - maxStorage);
          st->res[n] = maxStorage;
        }
        if (st->res[n] < 0.) {
          outflow += st->res[n];
          st->res[n] = 0.;
        }
        inflow = outflow;
        dailyActualUse += remUseResStart - remUseRes;   /* routing.cpp:3068 */
        wr.res_evapo = evapo; wr.res_out = outflow;
        st->rf_res[n] = 1. - pow(fabs(st->res[n] - maxStorage) / maxStorage, EVAPO_RED_EXP_RES);
        if (st->rf_res[n] < 0.) st->rf_res[n] = 0.;
        if (st->rf_res[n] > 1.) st->rf_res[n] = 1.;
      }
      if (wu && (s->res_area[n] > 0. || s->lake_area[n] > 0.)) {
        const double remAfter = (s->res_area[n] > 0.) ? remUseRes : remUseGloLake;
        if (!wu->nus_agg) {   /* routing.cpp:3166-3172 */
          remainingUse = remAfter;
        } else {   /* routing.cpp:3083-3165: what the lake or reservoir left of the unit's NUs */
          const double agg = wu->nus_agg[wo + n], own = wu->nus[wo + n];
          const double rUseAllocUnsat = totalDesiredUse - agg;
          for (int k = glwd.lo[n]; k < glwd.hi[n]; k++) {
            const int i = glwd.cells[k];
            double *rip_i = &W[(size_t)12 * (size_t)N + (size_t)i];
            if ((remAfter - rUseAllocUnsat) > 0.) {
              if (own <= 0.) {
                if (n == i) {
                  remainingUse = (agg < 0) ? remAfter : rUseAllocUnsat;
                  WU(12) = 0.;
                } else if (wu->nus[wo + i] <= 0.) {
                  *rip_i = 0.;
                } else {
                  *rip_i = (wu->nus[wo + i] / (agg - own)) * (remAfter - rUseAllocUnsat);
                }
              } else {
                if (n == i) {
                  remainingUse = (own / agg) * (remAfter - rUseAllocUnsat) + rUseAllocUnsat;
                  WU(12) = 0.;
                } else if (wu->nus[wo + i] < 0.) {
                  *rip_i = 0.;
                } else {
                  *rip_i = wu->nus[wo + i] / agg * (remAfter - rUseAllocUnsat);
                }
              }
            } else {
              *rip_i = 0.;
              WU(12) = 0.;
              remainingUse = remAfter;
            }
          }
        }
      }

      /* global wetland, routing.cpp:3178-3297 */
      if (s->glo_wetl[n] > 0) {
        double S0 = st->glowetl[n];
        maxStorage = ((s->glo_wetl[n]) / 100.) * cellArea * wetlDepth;
        double rf = st->rf_glowetl[n];
        double evapo = ((1.0 - cfa) * (owp * rf)) + (cfa * (owpet * rf));
        if (evapo < 0.) evapo = 0.;
        double pin = (owp * rf * (cellArea / 1000000.) * (s->glo_wetl[n] / 100.));
        totalInflow = inflow + pin;
        PETgwr = evapo * (cellArea / 1000000.) * ((s->glo_wetl[n]) / 100.);
        PETgwrMax = totalInflow + S0;
        p_ow += pin;
        wr.glowetl_prev = S0; wr.glowetl_rf = rf;
        if (PETgwr > PETgwrMax) {
          st->glowetl[n] = 0.;
          outflow = 0.;
          e_ow += PETgwrMax;
          evapo *= PETgwrMax / PETgwr;
        } else {
          st->glowetl[n] = S0 * exp(-1. * swoutf) + (1. / swoutf) * (totalInflow - PETgwr) * (1. - exp(-1. * swoutf));
          outflow = totalInflow + S0 - st->glowetl[n] - PETgwr;
          e_ow += PETgwr;
        }
        if (st->glowetl[n] > maxStorage) {
          outflow += (st->glowetl[n] - maxStorage);
          st->glowetl[n] = maxStorage;
        }
        if (fabs(st->glowetl[n]) <= MIN_STOR_VOL) st->glowetl[n] = 0.;
        inflow = outflow;
        wr.glowetl_evapo = evapo; wr.glowetl_out = outflow;
        st->rf_glowetl[n] = 1. - pow(fabs(st->glowetl[n] - maxStorage) / maxStorage, (evaredex * EVAPO_RED_EXP));
        if (st->rf_glowetl[n] < 0.) st->rf_glowetl[n] = 0.;
        if (st->rf_glowetl[n] > 1.) st->rf_glowetl[n] = 1.;
      }
      /* river, routing.cpp:3385-3514 */
      double riverInflow = inflow;
      if (s->frac_routing && s->ldd[n] >= 0) {   /* routing.cpp:3408-3412 */
        riverInflow += into_river;
        riverInflow += gw_into_river;
      }
      double riverVelocity;
      if (s->river_velo_opt == 0) riverVelocity = s->default_velocity;
      else riverVelocity = river_velocity(s, st, n, riverInflow, bw[n]);
      double K = riverVelocity / s->river_length[n];
      double S0 = st->river[n];
      riverInflow += 0.;   /* G_dailyRiverPrecip = 0 without river evaporation */
      double RiverEvapoRemUse = remainingUse + 0.;   /* routing.cpp:3466-3468 */
      const double remUseRiverStart = remainingUse;
      double RivEvapoRemUseMax = riverInflow + (K * S0 * exp(-1. * K)) / (1. - exp(-1. * K));
      double transportedVolume;
      double leak = 0.;
      if (RiverEvapoRemUse > RivEvapoRemUseMax) {
        st->river[n] = 0.;
        transportedVolume = riverInflow + S0 - RivEvapoRemUseMax;
        if (transportedVolume < 0.) { leak -= transportedVolume; transportedVolume = 0.; }
        if (wu) {
          e_ow += RivEvapoRemUseMax;
          if (remainingUse > 0.) remainingUse -= remainingUse * RivEvapoRemUseMax / RiverEvapoRemUse;
          else remainingUse = 0.;
        }
      } else {
        st->river[n] = S0 * exp(-1. * K) + (1. / K) * (riverInflow - RiverEvapoRemUse) * (1. - exp(-1. * K));
        if (fabs(st->river[n]) <= MIN_STOR_VOL) st->river[n] = 0.;
        transportedVolume = riverInflow + S0 - st->river[n] - RiverEvapoRemUse;
        if (transportedVolume < 0.) { leak -= transportedVolume; transportedVolume = 0.; }
        if (wu) e_ow += RiverEvapoRemUse;
        remainingUse = 0.;
      }
      if (wu) {
        /* what is left comes from the local lake, down to -maxStorage (routing.cpp:3590-3625) */
        if ((s->loc_lake[n] > 0.) && (remainingUse > 0.)) {
          const double maxLL = ((s->loc_lake[n]) / 100.) * cellArea * lakeDepth;
          if (st->loclake[n] > (-1.) * maxLL) {
            if (remainingUse < (maxLL + st->loclake[n])) {
              st->loclake[n] -= remainingUse;
              e_ow += remainingUse;
              remainingUse = 0.;
            } else {
              const double used = (maxLL + st->loclake[n]);
              remainingUse -= used;
              st->loclake[n] = (-1.) * maxLL;
              e_ow += used;
            }
          }
          st->rf_loclake[n] = 1. - pow(fabs(st->loclake[n] - maxLL) / (2. * maxLL), (evaredex * EVAPO_RED_EXP));
          if (st->rf_loclake[n] < 0.) st->rf_loclake[n] = 0.;
          if (st->rf_loclake[n] > 1.) st->rf_loclake[n] = 1.;
        }
        dailyActualUse += remUseRiverStart - remainingUse;
        /* bookkeeping of the cell's day (routing.cpp:3736, 3906-3919) */
        WU(11) += dailyActualUse;
        if (wu->delayed) {   /* routing.cpp:3900-3905 */
          WU(0) = remainingUse - prevTotalUnsat;
          WU(6) = remainingUse;
        } else {
          WU(6) += remainingUse;
          WU(0) = remainingUse;
        }
        WU(4) = wu->wdr[wo + n];
        WU(5) = wu->cons[wo + n];
        if (wu->daily_actual) wu->daily_actual[(size_t)d * N + n] = dailyActualUse + nug;
      }
      if (s->statcorr_opt == 1) {   /* station correction, routing.cpp:3929-3931 */
        const double before = transportedVolume;
        transportedVolume *= PAR(s, WGO_P_CFS, n);
        leak += transportedVolume - before;   /* water the correction adds (removes) */
      }
      /* push downstream, routing.cpp:3955-3958 */
      const int down = s->downstream[n];
      if (down >= 0) inflow_up[down] += transportedVolume;
      if (discharge) discharge[(size_t)d * N + n] = transportedVolume;
      if (wt)
        cell_water_temp(s, st, n, d, cellArea, cfa, &vo[n], localRunoff, local_gw, into_river, gw_into_river, &wr,
                        transportedVolume, bw[n], T[n], SW[n], wt);

      if (balance) {
        const double fl = cellArea * (laf / 100.) / 1000000.;
        b_in += vo[n].land_in * fl + p_ow;
        b_evap += vo[n].land_evap * fl + e_ow;
        b_leak += vo[n].land_leak * fl + leak;
        if (down < 0) b_out += transportedVolume;
      }
    }
    /* fractions for the next day, routing.cpp:5034-5188 and updateLandAreaFrac 5343-5352 */
    for (int n = 0; n < N; n++) {
      double fLocLake, fLocWet, fGloWet;
      if ((s->loc_lake[n] > 0.) && (st->rf_loclake[n] > 0.)) fLocLake = (st->rf_loclake[n] * s->loc_lake[n] / 100.);
      else fLocLake = 0.;
      if ((s->loc_wetl[n] > 0.) && (st->rf_locwetl[n] > 0.)) fLocWet = (st->rf_locwetl[n] * s->loc_wetl[n] / 100.);
      else fLocWet = 0.;
      if ((s->glo_wetl[n] > 0.) && (st->rf_glowetl[n] > 0.)) fGloWet = (st->rf_glowetl[n] * s->glo_wetl[n] / 100.);
      else fGloWet = 0.;
      double fswb = st->fswb_next[n];
      st->fswb_next[n] = fLocLake + fLocWet + fGloWet;
      double changePct = st->fswb_next[n] * 100. - fswb * 100.0;
      st->laf_started[n] = 1;
      double lafNext = st->laf[n] - (changePct + (0. * 100.));
      if (lafNext < 0.) lafNext = 0.;
      st->laf_prev[n] = st->laf[n];
      st->laf[n] = lafNext;
    }
    if (wu && day == 365)   /* annualWaterUsePostProcessing (routing.cpp:5246-5296) */
      for (int n = 0; n < N; n++) {
        if (WU(6) < WU(7)) {
          WU(7) = WU(6); WU(8) = WU(1); WU(9) = WU(2); WU(10) = WU(3);
          WU(1) = 0.; WU(2) = 0.; WU(3) = 0.; WU(6) = 0.;
        } else {
          WU(6) -= WU(7); WU(1) -= WU(8); WU(2) -= WU(9); WU(3) -= WU(10);
          if ((WU(1) + WU(2)) < 0) {
            WU(1) = 0; WU(2) = 0; WU(3) = 0;
          } else if (WU(2) < 0) {
            WU(1) += WU(2); WU(2) = 0;
          } else if (WU(1) < 0) {
            WU(2) += WU(1); WU(1) = 0; WU(3) = 0;
          }
          if (WU(3) > 0) { WU(3) = 0; WU(1) = 0; }
        }
      }
#undef WU
    g_time_routing += wall_now() - w1;
    if (balance) {
      double stot = 0.;
      for (int n = 0; n < N; n++) stot += state_volume(s, st, n);
      double *b = balance + (size_t)d * 6;
      b[0] = stot; b[1] = b_in; b[2] = b_evap; b[3] = b_out; b[4] = b_leak;
      b[5] = (stot - s_prev) - (b_in - b_evap - b_out + b_leak);
      s_prev = stot;
    }
    doy = (doy % 365) + 1;
  }
  glwd_free(&glwd);
  free(vo); free(inflow_up); free(bw);
  return 0;
}
