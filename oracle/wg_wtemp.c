/*
 * wg_wtemp.c -- CPU restatement of the reference's water temperature
 * (calcWaterTempClass, source/calcWaterTemp.cpp:23-1324; energy balance of
 * Beek et al. 2012 with the thermocline depth of Wanders et al. 2019).
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the GPU library, see wg_oracle.h).
 * Each surface water body keeps the reference's expression order, branch for
 * branch, so that the restatement reproduces the reference bit for bit when
 * both are compiled without floating-point contraction; the pin is
 * tests/golden/wtemp_cases.npz (the reference's calcWTemp on random records).
 */
#include <math.h>
#include <stddef.h>

#include "wg_oracle.h"

/* constants, calcWaterTemp.cpp:24-32 (the two exchange coefficients are ints there) */
#define CONV_K 273.15
#define HEAT_CAP_W 4180.
#define RHO_W (1000. * 1.e9)
#define K_H 20
#define K_H_ICE 8
#define PRECIP_T_CORR 1.5
#define LAMBDA_F (333.4 * 1.e3)
#define ALBEDO_W 0.08
#define ALBEDO_I 0.6
#define NO_TEMP (-9999.)

static double dmax(double a, double b) { return a < b ? b : a; }   /* std::max(a, b) */
static double dmin(double a, double b) { return b < a ? b : a; }   /* std::min(a, b) */

/* temperature of precipitation and surface runoff [K] */
static double rain_k(const wgo_wt_in *t) { return dmax(t->air_temp - PRECIP_T_CORR, 0.) + CONV_K; }

/* growth of the ice cover over one day [km] (same expression in every water body;
 * the river passes its storage where the others pass their temperature) */
static double ice_growth(double prev, const wgo_wt_in *t, double net_rad_ice) {
  return ((-(K_H_ICE * prev) + (K_H * (-t->air_temp)) - net_rad_ice) / (LAMBDA_F * RHO_W / 1.e9) * 86400.) / 1000.;
}

/* the clamps every water body ends with (calcWaterTemp.cpp:400-411 and the others) */
static void finish(const wgo_wt_in *t, double *temp, double *ice, double ice_floor) {
  if (*temp > 60.) *temp = t->air_temp;
  if (*temp < 1.e-10 && *temp != NO_TEMP) *temp = 0.;
  if (*ice < ice_floor) *ice = 0.;
}

/* the energy balance of an open water body once its total energy (without the
 * sensible heat flux) and volume are known: the sensible heat flux may only
 * bring the temperature to the air temperature (calcWaterTemp.cpp:376-395) */
static double open_water_temp(const wgo_wt_in *t, double energy, double sens, double vol) {
  if (!(vol > 0.)) return NO_TEMP;
  double temp = (energy / (vol * RHO_W * HEAT_CAP_W)) - CONV_K;
  energy -= sens;
  if (temp >= t->air_temp) {
    temp = (energy / (vol * RHO_W * HEAT_CAP_W)) - CONV_K;
    if (temp < t->air_temp) temp = t->air_temp;
  } else {
    temp = (energy / (vol * RHO_W * HEAT_CAP_W)) - CONV_K;
    if (temp > t->air_temp) temp = t->air_temp;
  }
  return temp;
}

/* the water under an ice cover: stored energy minus the heat to the ice, mixed
 * with the day's inflows of temperature in_k [K] and volume in_vol */
static double under_ice_temp(double energy_stor, double sens, double vol, double ice, double area, double in_vol,
                             int has_inflow, double in_k) {
  double temp = (energy_stor - sens) / (vol * RHO_W * HEAT_CAP_W) - CONV_K;
  if (temp < 0.) temp = 0.;
  if (has_inflow) {
    if ((vol - ice * area) > 0.)
      temp = (in_k * in_vol + (vol - ice * area) * (temp + CONV_K)) / ((vol - ice * area) + in_vol) - CONV_K;
    else
      temp = in_k - CONV_K;
  }
  return temp;
}

/* local lake, calcWaterTemp.cpp:258-407 */
static void loclake_temp(const wgo_wt_in *t, double nr_ice, double nr_water, double lat_heat, double *temp_out,
                         double *ice_out) {
  double gw = t->local_gw_runoff;
  double ice = t->ice[1];
  double temp = 0.;
  int ice_max = 0;
  const double area = t->cell_area * (t->loclake_area / 100.) * t->loclake_rf;
  const double precip = t->ow_prec / 1000000. * area;
  double surf = t->local_runoff - t->local_gw_runoff;
  if (!(t->has_outflow != 0.) && t->river_length_check == 55.) {
    surf += t->runoff_into_river - t->gw_runoff_into_river;
    gw += t->gw_runoff_into_river;
  }
  const double e_stor = t->loclake_stor_prev * RHO_W * HEAT_CAP_W * (t->loclake_temp_prev + CONV_K);
  if (t->air_temp <= 0. || ice > 0.) {
    ice += ice_growth(t->loclake_temp_prev, t, nr_ice);
    if (ice * area >= t->loclake_stor_prev) {
      ice = t->loclake_stor_prev / area;
      if (precip + surf + t->local_gw_runoff <= 0.) ice_max = 1;
    }
  }
  if (!ice_max) {
    if (ice > 0.) {
      const double sens = K_H_ICE * t->loclake_temp_prev * 1.e6 * 86400. * area;
      const double in_vol = precip + surf + t->local_gw_runoff;
      double in_k = 0.;
      if (in_vol > 0.)
        in_k = (precip * rain_k(t) + surf * rain_k(t) + t->local_gw_runoff * (t->gw_temp + CONV_K)) /
               (precip + surf + t->local_gw_runoff);
      temp = under_ice_temp(e_stor, sens, t->loclake_stor_prev, ice, area, precip + surf + t->local_gw_runoff,
                            in_vol > 0., in_k);
    } else {
      const double e_surf = surf * RHO_W * HEAT_CAP_W * rain_k(t);
      const double e_prec = precip * RHO_W * HEAT_CAP_W * rain_k(t);
      const double e_gw = gw * RHO_W * HEAT_CAP_W * (t->gw_temp + CONV_K);
      const double e_rad = nr_water * 1.e6 * 86400. * area;
      const double sens = K_H * (t->loclake_temp_prev - t->air_temp) * 1.e6 * 86400. * area;
      const double lat = lat_heat * RHO_W * (t->loclake_evapo / 1000000. * area);
      const double energy = e_stor + e_rad - lat + e_prec + e_surf + e_gw;
      const double vol = t->loclake_stor_prev + precip + surf + t->local_gw_runoff - (t->loclake_evapo / 1000000. * area);
      temp = open_water_temp(t, energy, sens, vol);
    }
  } else {
    temp = ice > 0. ? 0. : NO_TEMP;
  }
  finish(t, &temp, &ice, 0.);
  *temp_out = temp;
  *ice_out = ice;
}

/* local runoff into the first water body of the cell when no earlier one took it
 * (calcWaterTemp.cpp:447-457 and the same block of the others); returns the sum
 * in the order the water body adds it */
static void take_runoff(const wgo_wt_in *t, double *surf, double *gw, double *e_surf, double *e_gw) {
  if (!(t->has_outflow != 0.) && t->river_length_check == 55.) {
    *surf += t->runoff_into_river - t->gw_runoff_into_river;
    *gw += t->gw_runoff_into_river;
  }
  *surf += t->local_runoff - t->local_gw_runoff;
  *e_surf = *surf * RHO_W * HEAT_CAP_W * rain_k(t);
  *gw += t->local_gw_runoff;
  *e_gw = *gw * RHO_W * HEAT_CAP_W * (t->gw_temp + CONV_K);
}

/* local wetland, calcWaterTemp.cpp:420-568 */
static void locwetl_temp(const wgo_wt_in *t, double nr_ice, double nr_water, double lat_heat, double loclake_temp,
                         int gw_used, double *temp_out, double *ice_out) {
  double surf = 0., gw = 0., e_surf = 0., e_gw = 0., sum_runoff = 0.;
  double ice = t->ice[2];
  double temp = 0.;
  int ice_max = 0;
  const double area = t->cell_area * (t->locwetl_area / 100.) * t->locwetl_rf;
  const double precip = t->ow_prec / 1000000. * area;
  const double e_stor = t->locwetl_stor_prev * RHO_W * HEAT_CAP_W * (t->locwetl_temp_prev + CONV_K);
  if (!gw_used) {
    take_runoff(t, &surf, &gw, &e_surf, &e_gw);
    sum_runoff = gw + surf;
  }
  if (t->air_temp <= 0. || ice > 0.) {
    ice += ice_growth(t->locwetl_temp_prev, t, nr_ice);
    if (ice * area >= t->locwetl_stor_prev) {
      ice = t->locwetl_stor_prev / area;
      if (precip + sum_runoff + t->locwetl_inflow <= 0.) ice_max = 1;
    }
  }
  if (!ice_max) {
    if (ice > 0.) {
      const double sens = K_H_ICE * t->locwetl_temp_prev * 1.e6 * 86400. * area;
      const double in_vol = precip + sum_runoff + t->locwetl_inflow;
      double in_k = 0.;
      if (in_vol > 0.)
        in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t->gw_temp + CONV_K) +
                t->locwetl_inflow * (loclake_temp + CONV_K)) /
               (precip + sum_runoff + t->locwetl_inflow);
      temp = under_ice_temp(e_stor, sens, t->locwetl_stor_prev, ice, area, precip + sum_runoff + t->locwetl_inflow,
                            in_vol > 0., in_k);
    } else {
      const double e_prec = precip * RHO_W * HEAT_CAP_W * rain_k(t);
      const double e_rad = nr_water * 1.e6 * 86400. * area;
      const double sens = K_H * ((t->locwetl_temp_prev + CONV_K) - (t->air_temp + CONV_K)) * 1.e6 * 86400. * area;
      const double lat = lat_heat * RHO_W * (t->locwetl_evapo / 1000000. * area);
      double e_in = 0.;
      if (t->loclake_area > 0.) e_in = t->locwetl_inflow * RHO_W * HEAT_CAP_W * (loclake_temp + CONV_K);
      const double energy = e_stor + e_rad - lat + e_prec + e_in + e_surf + e_gw;
      double vol = t->locwetl_stor_prev + precip - (t->locwetl_evapo / 1000000. * area) + t->locwetl_inflow;
      if (!gw_used) vol += surf + gw;
      temp = open_water_temp(t, energy, sens, vol);
    }
  } else {
    temp = ice > 0. ? 0. : NO_TEMP;
  }
  finish(t, &temp, &ice, 0.);
  *temp_out = temp;
  *ice_out = ice;
}

/* volume above the thermocline [km3], calcWaterTemp.cpp:1313-1324 (0 global lake,
 * 1 reservoir) */
static double thermocline(double area, int type) {
  double f = 0.;
  if (type == 0) f = sqrt(2 * area);
  else if (type == 1) f = sqrt(3 * area / sqrt(3));
  return area * (9.52 * pow(f, 0.425));
}

/* global lake, reservoir and global wetland share one scheme
 * (calcWaterTemp.cpp:585-745, 761-915, 931-1081) and differ in their area, the
 * storage that exchanges heat, and their inflow; `type` 3/4/5 as the out index */
static void lake_temp(const wgo_wt_in *t, int type, double nr_ice, double nr_water, double lat_heat, double mix_temp,
                      int gw_used, double *temp_out, double *ice_out) {
  double area, stor_prev, temp_prev, evapo, inflow;
  if (type == 3) {
    area = t->glolake_area; temp_prev = t->glolake_temp_prev; evapo = t->glolake_evapo; inflow = t->glolake_inflow;
    stor_prev = dmin(t->glolake_stor_prev, thermocline(t->glolake_area, 0));
  } else if (type == 4) {
    area = t->res_area; temp_prev = t->res_temp_prev; evapo = t->res_evapo; inflow = t->res_inflow;
    stor_prev = dmin(t->res_stor_prev, thermocline(t->res_area, 1));
  } else {
    area = t->cell_area * (t->glowetl_area / 100.) * t->glowetl_rf;
    temp_prev = t->glowetl_temp_prev; evapo = t->glowetl_evapo; inflow = t->glowetl_inflow;
    stor_prev = t->glowetl_stor_prev;
  }
  double surf = 0., gw = 0., e_surf = 0., e_gw = 0., sum_runoff = 0.;
  double ice = t->ice[type];
  double temp = 0.;
  int ice_max = 0;
  const double precip = t->ow_prec / 1000000. * area;
  const double e_stor = stor_prev * RHO_W * HEAT_CAP_W * (temp_prev + CONV_K);
  if (!gw_used) {
    take_runoff(t, &surf, &gw, &e_surf, &e_gw);
    sum_runoff = surf + gw;
  }
  if (t->air_temp <= 0. || ice > 0.) {
    ice += ice_growth(temp_prev, t, nr_ice);
    if (ice * area >= stor_prev) {
      ice = stor_prev / area;
      if (precip + sum_runoff + inflow <= 0.) ice_max = 1;
    }
  }
  if (!ice_max) {
    if (ice > 0.) {
      const double sens = K_H_ICE * temp_prev * 1.e6 * 86400. * area;
      const double in_vol = precip + sum_runoff + inflow;
      double in_k = 0.;
      if (in_vol > 0.) {
        if (mix_temp < 0.)
          in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t->gw_temp + CONV_K)) / (precip + sum_runoff);
        else
          in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t->gw_temp + CONV_K) + inflow * (mix_temp + CONV_K)) /
                 (precip + sum_runoff + inflow);
      }
      temp = under_ice_temp(e_stor, sens, stor_prev, ice, area, precip + sum_runoff + inflow, in_vol > 0., in_k);
    } else {
      const double e_prec = precip * RHO_W * HEAT_CAP_W * rain_k(t);
      const double e_rad = nr_water * 1.e6 * 86400. * area;
      const double sens = K_H * ((temp_prev + CONV_K) - (t->air_temp + CONV_K)) * 1.e6 * 86400. * area;
      const double lat = lat_heat * RHO_W * (evapo / 1000000. * area);
      double e_in = 0.;
      if (mix_temp >= 0.) e_in = ((mix_temp + CONV_K) * inflow * RHO_W * HEAT_CAP_W);
      const double energy = e_stor + e_rad - lat + e_prec + e_in + e_surf + e_gw;
      double vol = stor_prev + precip - (evapo / 1000000. * area) + inflow;
      if (!gw_used) vol += surf + gw;
      temp = open_water_temp(t, energy, sens, vol);
    }
  } else {
    temp = ice > 0. ? 0. : NO_TEMP;
  }
  finish(t, &temp, &ice, 0.);
  *temp_out = temp;
  *ice_out = ice;
}

/* river, calcWaterTemp.cpp:1097-1298 */
static void river_temp(const wgo_wt_in *t, double nr_ice, double nr_water, double lat_heat, double mix_temp,
                       int gw_used, double *temp_out, double *ice_out) {
  double area = 0., depth = 0.;
  double gw = t->runoff_into_river;   /* the reference starts its groundwater term from this field */
  double ice = t->ice[0];
  int ice_max = 0;
  double temp = 0., vol = 0.;
  const double csa = t->river_stor / t->river_length;
  if (csa > 0.) {
    depth = -t->river_bottom_width / (4. * 1000.) +
            sqrt(t->river_bottom_width / 1000. * t->river_bottom_width / (16. * 1000.) + 0.5 * csa);
    area = t->river_stor / depth;
  }
  const double e_stor = t->river_stor * RHO_W * HEAT_CAP_W * (t->inflow_temp[4] + CONV_K);
  const double precip = t->ow_prec * area / 1000000.;
  double surf = t->runoff_into_river - t->gw_runoff_into_river;
  if (!gw_used) {
    surf += (t->local_runoff - t->local_gw_runoff);
    gw += t->local_gw_runoff;
  }
  if (t->air_temp <= 0. || ice >= 5.e-6) {
    if (area > 0.) {
      ice += ice_growth(t->river_stor, t, nr_ice);
      if (ice * area >= t->river_stor) {
        ice = t->river_stor / area;
        if (precip + surf + gw + t->river_inflow <= 0.) ice_max = 1;
      }
    } else {
      ice = 0.;
    }
  }
  if (!ice_max) {
    if (ice >= 5.e-6) {
      const double sens = K_H_ICE * t->inflow_temp[4] * 1.e6 * 86400. * area;
      vol = t->river_stor;
      const double in_vol = precip + surf + gw + t->river_inflow;
      double in_k = 0.;
      if (in_vol > 0.) {
        if (mix_temp < 0.)
          in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t->gw_temp + CONV_K)) / (precip + surf + gw);
        else
          in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t->gw_temp + CONV_K) +
                  t->river_inflow * (mix_temp + CONV_K)) /
                 (precip + surf + gw + t->river_inflow);
      }
      temp = under_ice_temp(e_stor, sens, vol, ice, area, precip + surf + gw + t->river_inflow, in_vol > 0., in_k);
    } else {
      const double e_surf = surf * RHO_W * HEAT_CAP_W * rain_k(t);
      const double e_gw = gw * RHO_W * HEAT_CAP_W * (t->gw_temp + CONV_K);
      const double evapo = ((1.0 - t->cfa) * t->ow_prec + (t->cfa * t->ow_pet)) * area / 1000000.;
      if (evapo >= t->river_stor + t->river_inflow + precip + surf + gw) {
        *temp_out = NO_TEMP;   /* everything evaporates; the ice record is reset */
        *ice_out = 0.;
        return;
      }
      const double e_prec = precip * RHO_W * HEAT_CAP_W * rain_k(t);
      const double e_rad = nr_water * 1.e6 * 86400. * area;
      const double sens = K_H * ((t->inflow_temp[4] + CONV_K) - (t->air_temp + CONV_K)) * 1.e6 * 86400. * area;
      const double lat = lat_heat * RHO_W * evapo;
      double e_in = 0.;
      if (mix_temp >= 0.) e_in = t->river_inflow * RHO_W * HEAT_CAP_W * (mix_temp + CONV_K);
      const double energy = e_stor + e_rad - lat + e_in + e_prec + e_surf + e_gw;
      vol = t->river_stor + t->river_inflow + precip + surf + gw - evapo;
      temp = open_water_temp(t, energy, sens, vol);
    }
    /* power-plant cooling (options.calc_wtemp = 2), calcWaterTemp.cpp:1263-1285 */
    if (temp >= 0. && t->pp_withdrawal > 0. && t->calc_temp_pp != 0.) {
      if (ice >= 5.e-6) vol -= ice * area;
      if (vol > 0.) {
        const double wd = vol < t->pp_withdrawal ? vol : t->pp_withdrawal;
        const double ret = wd > t->pp_consumption ? wd - t->pp_consumption : 0.;
        if (ret > 0.)
          temp = (((vol - wd) * (temp + CONV_K) + ret * (temp + 3. + CONV_K)) / (vol - wd + ret)) - CONV_K;
      }
    }
  } else {
    temp = ice > 0. ? 0. : NO_TEMP;
  }
  finish(t, &temp, &ice, 5.e-6);
  *temp_out = temp;
  *ice_out = ice;
}

/* mixing temperature of the cell's river inflow and its local wetland (or local
 * lake) outflow: the block calcWTemp repeats before each global water body */
static double local_mix(const wgo_wt_in *t, double tot_in, double in_temp, double loclake_temp, double locwetl_temp) {
  double mix;
  if ((tot_in >= 0.) && (t->locwetl_outflow > 0.)) {
    mix = ((in_temp + CONV_K) * tot_in + (locwetl_temp + CONV_K) * t->locwetl_outflow) / (tot_in + t->locwetl_outflow) -
          CONV_K;
    if (mix < 0.) mix = 0.;
  } else if (tot_in > 0.) {
    mix = ((in_temp + CONV_K) * tot_in + (loclake_temp + CONV_K) * t->locwetl_inflow) / (tot_in + t->locwetl_inflow) -
          CONV_K;
    if (mix < 0.) mix = 0.;
  } else if (t->locwetl_inflow > 0.) {
    mix = loclake_temp;
  } else {
    mix = NO_TEMP;
  }
  return mix;
}

void wgo_wtemp(const wgo_wt_in *t, double out[12]) {
  for (int k = 0; k < 12; k++) out[k] = NO_TEMP;
  double loclake = 0., locwetl = 0., glolake = 0., res = 0., glowetl = 0.;
  double mix = NO_TEMP;
  double tot_in = 0., e_in = 0., in_temp = 0.;
  int gw_used = 0;
  double tmp, ice;
  for (int i = 0; i < 9; i++) tot_in += t->inflow[i];
  for (int i = 0; i < 9; i++) e_in += t->inflow[i] * RHO_W * HEAT_CAP_W * (t->inflow_temp[i] + CONV_K);
  if (tot_in > 0.) in_temp = e_in / (tot_in * RHO_W * HEAT_CAP_W) - CONV_K;
  const double lat_heat = t->air_temp > 0. ? (2.501 - 0.002361 * t->air_temp) * 1.e6 : 0.;
  const double net_long = t->long_rad - 1. * 0.00000005670374419 * pow((t->air_temp + CONV_K), 4.);
  const double nr_water = (t->short_rad * (1. - ALBEDO_W) + net_long);
  const double nr_ice = (t->short_rad * (1. - ALBEDO_I) + net_long);
  if (t->loclake_area > 0.) {
    loclake_temp(t, nr_ice, nr_water, lat_heat, &tmp, &ice);
    gw_used = 1;
    loclake = tmp;
    out[1] = out[0] = loclake;
    out[7] = ice;
  }
  if (t->locwetl_area > 0.) {
    locwetl_temp(t, nr_ice, nr_water, lat_heat, loclake, gw_used, &tmp, &ice);
    gw_used = 1;
    locwetl = tmp;
    out[2] = out[0] = locwetl;
    out[8] = ice;
  }
  if (t->glolake_area > 0.) {
    mix = local_mix(t, tot_in, in_temp, loclake, locwetl);
    lake_temp(t, 3, nr_ice, nr_water, lat_heat, mix, gw_used, &tmp, &ice);
    gw_used = 1;
    glolake = tmp;
    out[3] = out[0] = glolake;
    out[9] = ice;
  }
  if (t->res_area > 0.) {
    mix = t->glolake_area <= 0. ? local_mix(t, tot_in, in_temp, loclake, locwetl) : glolake;
    lake_temp(t, 4, nr_ice, nr_water, lat_heat, mix, gw_used, &tmp, &ice);
    gw_used = 1;
    res = tmp;
    out[4] = out[0] = res;
    out[10] = ice;
  }
  if (t->glowetl_area > 0.) {
    if (t->res_area > 0.) mix = res;
    else if (t->glolake_area <= 0.) mix = local_mix(t, tot_in, in_temp, loclake, locwetl);
    else if (t->glolake_area > 0.) mix = glolake;
    lake_temp(t, 5, nr_ice, nr_water, lat_heat, mix, gw_used, &tmp, &ice);
    gw_used = 1;
    glowetl = tmp;
    out[5] = out[0] = glowetl;
    out[11] = ice;
  }
  if (t->has_outflow != 0. || t->river_length_check != 55.) {
    if (t->glowetl_area > 0.) mix = glowetl;
    else if (t->res_area > 0.) mix = res;
    else if (t->glolake_area > 0.) mix = glolake;
    else if (t->glolake_area <= 0.) mix = local_mix(t, tot_in, in_temp, loclake, locwetl);
    river_temp(t, nr_ice, nr_water, lat_heat, mix, gw_used, &tmp, &ice);
    out[0] = tmp;
    out[6] = ice;
  }
}

void wgo_wtemp_batch(const double *records, int n, double *out) {
  for (int k = 0; k < n; k++) wgo_wtemp((const wgo_wt_in *)(records + (size_t)k * WGO_WT_NIN), out + (size_t)k * 12);
}
