// wg_wtemp.cuh -- water temperature of one cell and day on the GPU: the
// reference's calcWaterTempClass::calcWTemp (source/calcWaterTemp.cpp:48-1324),
// the energy balance of Beek et al. (2012) with the thermocline depth of
// Wanders et al. (2019), for the river and the five kinds of surface water
// body, with ice cover.  FP64, branch for branch as the reference; the
// arithmetic folds the constant factors (rho c, the ice growth per W/m2),
// multiplies by 1e-6 and by one refined reciprocal of the volume's heat
// capacity instead of dividing, takes pow(T, 4) as two squarings and the
// thermocline's pow from fm::pow -- a few ulp of rounding against the oracle,
// which keeps the reference's expression order.  The caller assembles the
// inputs from routing_cell's terms (routing.cpp:4241-4356) and keeps the state
// (temperatures, ice thickness).
#pragma once
#include "wg_fastmath.cuh"

namespace wg {
namespace wt {

// Inputs of one cell and day: calcWaterTempClass::transfer (calcWaterTemp.h:23-95);
// swb index [0] river, [1] local lake, [2] local wetland, [3] global lake,
// [4] reservoir, [5] global wetland.
struct WtIn {
  double calc_temp_pp, pp_withdrawal, pp_consumption;
  double short_rad, long_rad, air_temp, cfa, ow_pet, ow_prec, cell_area, gw_temp;
  // the upstream cells' river outflow of the day, summed, and the energy it
  // carries (sum of volume x rho c (T + 273.15)); the cell's own river
  // temperature of the previous day (the reference's inflow entry [4])
  double inflow_sum, inflow_energy, own_temp_prev;
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
};

__device__ __forceinline__ double wt_max(double a, double b) { return a < b ? b : a; }   // std::max
__device__ __forceinline__ double wt_min(double a, double b) { return b < a ? b : a; }   // std::min
__device__ __forceinline__ double pow4(double x) { const double x2 = x * x; return x2 * x2; }

/* constants, calcWaterTemp.cpp:24-32 (the two exchange coefficients are ints there) */
#define WT_CONV_K 273.15
#define WT_HEAT_CAP_W 4180.
#define WT_RHO_W (1000. * 1.e9)
#define WT_K_H 20
#define WT_K_H_ICE 8
#define WT_PRECIP_T_CORR 1.5
#define WT_LAMBDA_F (333.4 * 1.e3)
#define WT_ALBEDO_W 0.08
#define WT_ALBEDO_I 0.6
#define WT_NO_TEMP (-9999.)
// folded constants of the device version (the oracle keeps the reference's
// separate factors): rho c [J/(km3 K)], and the day's ice growth per W/m2
#define WT_RC (WT_RHO_W * WT_HEAT_CAP_W)
#define WT_ICE_PER_FLUX (86400. / 1000. / (WT_LAMBDA_F * WT_RHO_W / 1.e9))


/* temperature of precipitation and surface runoff [K] */
__device__ __forceinline__ double rain_k(const WtIn &t) { return wt_max(t.air_temp - WT_PRECIP_T_CORR, 0.) + WT_CONV_K; }

/* growth of the ice cover over one day [km] (same expression in every water body;
 * the river passes its storage where the others pass their temperature) */
__device__ __forceinline__ double ice_growth(double prev, const WtIn &t, double net_rad_ice) {
  return (-(WT_K_H_ICE * prev) + (WT_K_H * (-t.air_temp)) - net_rad_ice) * WT_ICE_PER_FLUX;
}

/* the clamps every water body ends with (calcWaterTemp.cpp:400-411 and the others) */
__device__ __forceinline__ void finish(const WtIn &t, double *temp, double *ice, double ice_floor) {
  if (*temp > 60.) *temp = t.air_temp;
  if (*temp < 1.e-10 && *temp != WT_NO_TEMP) *temp = 0.;
  if (*ice < ice_floor) *ice = 0.;
}

/* the energy balance of an open water body once its total energy (without the
 * sensible heat flux) and volume are known: the sensible heat flux may only
 * bring the temperature to the air temperature (calcWaterTemp.cpp:376-395) */
__device__ __forceinline__ double open_water_temp(const WtIn &t, double energy, double sens, double vol) {
  if (!(vol > 0.)) return WT_NO_TEMP;
  const double inv = fm::rcp_pos(vol * WT_RC);   // vol > 0
  double temp = energy * inv - WT_CONV_K;
  energy -= sens;
  if (temp >= t.air_temp) {
    temp = energy * inv - WT_CONV_K;
    if (temp < t.air_temp) temp = t.air_temp;
  } else {
    temp = energy * inv - WT_CONV_K;
    if (temp > t.air_temp) temp = t.air_temp;
  }
  return temp;
}

/* the water under an ice cover: stored energy minus the heat to the ice, mixed
 * with the day's inflows of temperature in_k [K] and volume in_vol */
__device__ __forceinline__ double under_ice_temp(double energy_stor, double sens, double vol, double ice, double area, double in_vol,
                             int has_inflow, double in_k) {
  double temp = (energy_stor - sens) / (vol * WT_RC) - WT_CONV_K;
  if (temp < 0.) temp = 0.;
  if (has_inflow) {
    if ((vol - ice * area) > 0.)
      temp = (in_k * in_vol + (vol - ice * area) * (temp + WT_CONV_K)) / ((vol - ice * area) + in_vol) - WT_CONV_K;
    else
      temp = in_k - WT_CONV_K;
  }
  return temp;
}

/* local lake, calcWaterTemp.cpp:258-407 */
__device__ __forceinline__ void loclake_temp(const WtIn &t, double nr_ice, double nr_water, double lat_heat, double *temp_out,
                         double *ice_out) {
  double gw = t.local_gw_runoff;
  double ice = t.ice[1];
  double temp = 0.;
  int ice_max = 0;
  const double area = t.cell_area * (t.loclake_area / 100.) * t.loclake_rf;
  const double precip = t.ow_prec * 1.e-6 * area;
  double surf = t.local_runoff - t.local_gw_runoff;
  if (!(t.has_outflow != 0.) && t.river_length_check == 55.) {
    surf += t.runoff_into_river - t.gw_runoff_into_river;
    gw += t.gw_runoff_into_river;
  }
  const double e_stor = t.loclake_stor_prev * WT_RC * (t.loclake_temp_prev + WT_CONV_K);
  if (t.air_temp <= 0. || ice > 0.) {
    ice += ice_growth(t.loclake_temp_prev, t, nr_ice);
    if (ice * area >= t.loclake_stor_prev) {
      ice = t.loclake_stor_prev / area;
      if (precip + surf + t.local_gw_runoff <= 0.) ice_max = 1;
    }
  }
  if (!ice_max) {
    if (ice > 0.) {
      const double sens = WT_K_H_ICE * t.loclake_temp_prev * 1.e6 * 86400. * area;
      const double in_vol = precip + surf + t.local_gw_runoff;
      double in_k = 0.;
      if (in_vol > 0.)
        in_k = (precip * rain_k(t) + surf * rain_k(t) + t.local_gw_runoff * (t.gw_temp + WT_CONV_K)) /
               (precip + surf + t.local_gw_runoff);
      temp = under_ice_temp(e_stor, sens, t.loclake_stor_prev, ice, area, precip + surf + t.local_gw_runoff,
                            in_vol > 0., in_k);
    } else {
      const double e_surf = surf * WT_RC * rain_k(t);
      const double e_prec = precip * WT_RC * rain_k(t);
      const double e_gw = gw * WT_RC * (t.gw_temp + WT_CONV_K);
      const double e_rad = nr_water * 1.e6 * 86400. * area;
      const double sens = WT_K_H * (t.loclake_temp_prev - t.air_temp) * 1.e6 * 86400. * area;
      const double lat = lat_heat * WT_RHO_W * (t.loclake_evapo * 1.e-6 * area);
      const double energy = e_stor + e_rad - lat + e_prec + e_surf + e_gw;
      const double vol = t.loclake_stor_prev + precip + surf + t.local_gw_runoff - (t.loclake_evapo * 1.e-6 * area);
      temp = open_water_temp(t, energy, sens, vol);
    }
  } else {
    temp = ice > 0. ? 0. : WT_NO_TEMP;
  }
  finish(t, &temp, &ice, 0.);
  *temp_out = temp;
  *ice_out = ice;
}

/* local runoff into the first water body of the cell when no earlier one took it
 * (calcWaterTemp.cpp:447-457 and the same block of the others); returns the sum
 * in the order the water body adds it */
__device__ __forceinline__ void take_runoff(const WtIn &t, double *surf, double *gw, double *e_surf, double *e_gw) {
  if (!(t.has_outflow != 0.) && t.river_length_check == 55.) {
    *surf += t.runoff_into_river - t.gw_runoff_into_river;
    *gw += t.gw_runoff_into_river;
  }
  *surf += t.local_runoff - t.local_gw_runoff;
  *e_surf = *surf * WT_RC * rain_k(t);
  *gw += t.local_gw_runoff;
  *e_gw = *gw * WT_RC * (t.gw_temp + WT_CONV_K);
}

/* local wetland, calcWaterTemp.cpp:420-568 */
__device__ __forceinline__ void locwetl_temp(const WtIn &t, double nr_ice, double nr_water, double lat_heat, double loclake_temp,
                         int gw_used, double *temp_out, double *ice_out) {
  double surf = 0., gw = 0., e_surf = 0., e_gw = 0., sum_runoff = 0.;
  double ice = t.ice[2];
  double temp = 0.;
  int ice_max = 0;
  const double area = t.cell_area * (t.locwetl_area / 100.) * t.locwetl_rf;
  const double precip = t.ow_prec * 1.e-6 * area;
  const double e_stor = t.locwetl_stor_prev * WT_RC * (t.locwetl_temp_prev + WT_CONV_K);
  if (!gw_used) {
    take_runoff(t, &surf, &gw, &e_surf, &e_gw);
    sum_runoff = gw + surf;
  }
  if (t.air_temp <= 0. || ice > 0.) {
    ice += ice_growth(t.locwetl_temp_prev, t, nr_ice);
    if (ice * area >= t.locwetl_stor_prev) {
      ice = t.locwetl_stor_prev / area;
      if (precip + sum_runoff + t.locwetl_inflow <= 0.) ice_max = 1;
    }
  }
  if (!ice_max) {
    if (ice > 0.) {
      const double sens = WT_K_H_ICE * t.locwetl_temp_prev * 1.e6 * 86400. * area;
      const double in_vol = precip + sum_runoff + t.locwetl_inflow;
      double in_k = 0.;
      if (in_vol > 0.)
        in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t.gw_temp + WT_CONV_K) +
                t.locwetl_inflow * (loclake_temp + WT_CONV_K)) /
               (precip + sum_runoff + t.locwetl_inflow);
      temp = under_ice_temp(e_stor, sens, t.locwetl_stor_prev, ice, area, precip + sum_runoff + t.locwetl_inflow,
                            in_vol > 0., in_k);
    } else {
      const double e_prec = precip * WT_RC * rain_k(t);
      const double e_rad = nr_water * 1.e6 * 86400. * area;
      const double sens = WT_K_H * ((t.locwetl_temp_prev + WT_CONV_K) - (t.air_temp + WT_CONV_K)) * 1.e6 * 86400. * area;
      const double lat = lat_heat * WT_RHO_W * (t.locwetl_evapo * 1.e-6 * area);
      double e_in = 0.;
      if (t.loclake_area > 0.) e_in = t.locwetl_inflow * WT_RC * (loclake_temp + WT_CONV_K);
      const double energy = e_stor + e_rad - lat + e_prec + e_in + e_surf + e_gw;
      double vol = t.locwetl_stor_prev + precip - (t.locwetl_evapo * 1.e-6 * area) + t.locwetl_inflow;
      if (!gw_used) vol += surf + gw;
      temp = open_water_temp(t, energy, sens, vol);
    }
  } else {
    temp = ice > 0. ? 0. : WT_NO_TEMP;
  }
  finish(t, &temp, &ice, 0.);
  *temp_out = temp;
  *ice_out = ice;
}

/* volume above the thermocline [km3], calcWaterTemp.cpp:1313-1324 (0 global lake,
 * 1 reservoir) */
__device__ __forceinline__ double thermocline(double area, int type) {
  double f = 0.;
  if (type == 0) f = sqrt(2 * area);
  else if (type == 1) f = sqrt(3 * area / sqrt(3.));
  return area * (9.52 * fm::pow(f, 0.425));
}

/* global lake, reservoir and global wetland share one scheme
 * (calcWaterTemp.cpp:585-745, 761-915, 931-1081) and differ in their area, the
 * storage that exchanges heat, and their inflow; `type` 3/4/5 as the out index */
__device__ __forceinline__ void lake_temp(const WtIn &t, int type, double nr_ice, double nr_water, double lat_heat, double mix_temp,
                      int gw_used, double *temp_out, double *ice_out) {
  double area, stor_prev, temp_prev, evapo, inflow;
  if (type == 3) {
    area = t.glolake_area; temp_prev = t.glolake_temp_prev; evapo = t.glolake_evapo; inflow = t.glolake_inflow;
    stor_prev = wt_min(t.glolake_stor_prev, thermocline(t.glolake_area, 0));
  } else if (type == 4) {
    area = t.res_area; temp_prev = t.res_temp_prev; evapo = t.res_evapo; inflow = t.res_inflow;
    stor_prev = wt_min(t.res_stor_prev, thermocline(t.res_area, 1));
  } else {
    area = t.cell_area * (t.glowetl_area / 100.) * t.glowetl_rf;
    temp_prev = t.glowetl_temp_prev; evapo = t.glowetl_evapo; inflow = t.glowetl_inflow;
    stor_prev = t.glowetl_stor_prev;
  }
  double surf = 0., gw = 0., e_surf = 0., e_gw = 0., sum_runoff = 0.;
  double ice = t.ice[type];
  double temp = 0.;
  int ice_max = 0;
  const double precip = t.ow_prec * 1.e-6 * area;
  const double e_stor = stor_prev * WT_RC * (temp_prev + WT_CONV_K);
  if (!gw_used) {
    take_runoff(t, &surf, &gw, &e_surf, &e_gw);
    sum_runoff = surf + gw;
  }
  if (t.air_temp <= 0. || ice > 0.) {
    ice += ice_growth(temp_prev, t, nr_ice);
    if (ice * area >= stor_prev) {
      ice = stor_prev / area;
      if (precip + sum_runoff + inflow <= 0.) ice_max = 1;
    }
  }
  if (!ice_max) {
    if (ice > 0.) {
      const double sens = WT_K_H_ICE * temp_prev * 1.e6 * 86400. * area;
      const double in_vol = precip + sum_runoff + inflow;
      double in_k = 0.;
      if (in_vol > 0.) {
        if (mix_temp < 0.)
          in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t.gw_temp + WT_CONV_K)) / (precip + sum_runoff);
        else
          in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t.gw_temp + WT_CONV_K) + inflow * (mix_temp + WT_CONV_K)) /
                 (precip + sum_runoff + inflow);
      }
      temp = under_ice_temp(e_stor, sens, stor_prev, ice, area, precip + sum_runoff + inflow, in_vol > 0., in_k);
    } else {
      const double e_prec = precip * WT_RC * rain_k(t);
      const double e_rad = nr_water * 1.e6 * 86400. * area;
      const double sens = WT_K_H * ((temp_prev + WT_CONV_K) - (t.air_temp + WT_CONV_K)) * 1.e6 * 86400. * area;
      const double lat = lat_heat * WT_RHO_W * (evapo * 1.e-6 * area);
      double e_in = 0.;
      if (mix_temp >= 0.) e_in = ((mix_temp + WT_CONV_K) * inflow * WT_RC);
      const double energy = e_stor + e_rad - lat + e_prec + e_in + e_surf + e_gw;
      double vol = stor_prev + precip - (evapo * 1.e-6 * area) + inflow;
      if (!gw_used) vol += surf + gw;
      temp = open_water_temp(t, energy, sens, vol);
    }
  } else {
    temp = ice > 0. ? 0. : WT_NO_TEMP;
  }
  finish(t, &temp, &ice, 0.);
  *temp_out = temp;
  *ice_out = ice;
}

/* river, calcWaterTemp.cpp:1097-1298 */
__device__ __forceinline__ void river_temp(const WtIn &t, double nr_ice, double nr_water, double lat_heat, double mix_temp,
                       int gw_used, double *temp_out, double *ice_out) {
  double area = 0., depth = 0.;
  double gw = t.runoff_into_river;   /* the reference starts its groundwater term from this field */
  double ice = t.ice[0];
  int ice_max = 0;
  double temp = 0., vol = 0.;
  const double csa = t.river_stor / t.river_length;
  if (csa > 0.) {
    depth = -t.river_bottom_width / (4. * 1000.) +
            sqrt(t.river_bottom_width / 1000. * t.river_bottom_width / (16. * 1000.) + 0.5 * csa);
    area = t.river_stor / depth;
  }
  const double e_stor = t.river_stor * WT_RC * (t.own_temp_prev + WT_CONV_K);
  const double precip = t.ow_prec * area * 1.e-6;
  double surf = t.runoff_into_river - t.gw_runoff_into_river;
  if (!gw_used) {
    surf += (t.local_runoff - t.local_gw_runoff);
    gw += t.local_gw_runoff;
  }
  if (t.air_temp <= 0. || ice >= 5.e-6) {
    if (area > 0.) {
      ice += ice_growth(t.river_stor, t, nr_ice);
      if (ice * area >= t.river_stor) {
        ice = t.river_stor / area;
        if (precip + surf + gw + t.river_inflow <= 0.) ice_max = 1;
      }
    } else {
      ice = 0.;
    }
  }
  if (!ice_max) {
    if (ice >= 5.e-6) {
      const double sens = WT_K_H_ICE * t.own_temp_prev * 1.e6 * 86400. * area;
      vol = t.river_stor;
      const double in_vol = precip + surf + gw + t.river_inflow;
      double in_k = 0.;
      if (in_vol > 0.) {
        if (mix_temp < 0.)
          in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t.gw_temp + WT_CONV_K)) / (precip + surf + gw);
        else
          in_k = (precip * rain_k(t) + surf * rain_k(t) + gw * (t.gw_temp + WT_CONV_K) +
                  t.river_inflow * (mix_temp + WT_CONV_K)) /
                 (precip + surf + gw + t.river_inflow);
      }
      temp = under_ice_temp(e_stor, sens, vol, ice, area, precip + surf + gw + t.river_inflow, in_vol > 0., in_k);
    } else {
      const double e_surf = surf * WT_RC * rain_k(t);
      const double e_gw = gw * WT_RC * (t.gw_temp + WT_CONV_K);
      const double evapo = ((1.0 - t.cfa) * t.ow_prec + (t.cfa * t.ow_pet)) * area * 1.e-6;
      if (evapo >= t.river_stor + t.river_inflow + precip + surf + gw) {
        *temp_out = WT_NO_TEMP;   /* everything evaporates; the ice record is reset */
        *ice_out = 0.;
        return;
      }
      const double e_prec = precip * WT_RC * rain_k(t);
      const double e_rad = nr_water * 1.e6 * 86400. * area;
      const double sens = WT_K_H * ((t.own_temp_prev + WT_CONV_K) - (t.air_temp + WT_CONV_K)) * 1.e6 * 86400. * area;
      const double lat = lat_heat * WT_RHO_W * evapo;
      double e_in = 0.;
      if (mix_temp >= 0.) e_in = t.river_inflow * WT_RC * (mix_temp + WT_CONV_K);
      const double energy = e_stor + e_rad - lat + e_in + e_prec + e_surf + e_gw;
      vol = t.river_stor + t.river_inflow + precip + surf + gw - evapo;
      temp = open_water_temp(t, energy, sens, vol);
    }
    /* power-plant cooling (options.calc_wtemp = 2), calcWaterTemp.cpp:1263-1285 */
    if (temp >= 0. && t.pp_withdrawal > 0. && t.calc_temp_pp != 0.) {
      if (ice >= 5.e-6) vol -= ice * area;
      if (vol > 0.) {
        const double wd = vol < t.pp_withdrawal ? vol : t.pp_withdrawal;
        const double ret = wd > t.pp_consumption ? wd - t.pp_consumption : 0.;
        if (ret > 0.)
          temp = (((vol - wd) * (temp + WT_CONV_K) + ret * (temp + 3. + WT_CONV_K)) / (vol - wd + ret)) - WT_CONV_K;
      }
    }
  } else {
    temp = ice > 0. ? 0. : WT_NO_TEMP;
  }
  finish(t, &temp, &ice, 5.e-6);
  *temp_out = temp;
  *ice_out = ice;
}

/* mixing temperature of the cell's river inflow and its local wetland (or local
 * lake) outflow: the block calcWTemp repeats before each global water body */
__device__ __forceinline__ double local_mix(const WtIn &t, double tot_in, double in_temp, double loclake_temp, double locwetl_temp) {
  double mix;
  if ((tot_in >= 0.) && (t.locwetl_outflow > 0.)) {
    mix = ((in_temp + WT_CONV_K) * tot_in + (locwetl_temp + WT_CONV_K) * t.locwetl_outflow) / (tot_in + t.locwetl_outflow) -
          WT_CONV_K;
    if (mix < 0.) mix = 0.;
  } else if (tot_in > 0.) {
    mix = ((in_temp + WT_CONV_K) * tot_in + (loclake_temp + WT_CONV_K) * t.locwetl_inflow) / (tot_in + t.locwetl_inflow) -
          WT_CONV_K;
    if (mix < 0.) mix = 0.;
  } else if (t.locwetl_inflow > 0.) {
    mix = loclake_temp;
  } else {
    mix = WT_NO_TEMP;
  }
  return mix;
}

__device__ __forceinline__ void water_temp_cell(const WtIn &t, double out[12]) {
  for (int k = 0; k < 12; k++) out[k] = WT_NO_TEMP;
  double loclake = 0., locwetl = 0., glolake = 0., res = 0., glowetl = 0.;
  double mix = WT_NO_TEMP;
  double tot_in = 0., e_in = 0., in_temp = 0.;
  int gw_used = 0;
  double tmp, ice;
  tot_in = t.inflow_sum;
  e_in = t.inflow_energy;
  if (tot_in > 0.) in_temp = e_in / (tot_in * WT_RC) - WT_CONV_K;
  const double lat_heat = t.air_temp > 0. ? (2.501 - 0.002361 * t.air_temp) * 1.e6 : 0.;
  const double net_long = t.long_rad - 1. * 0.00000005670374419 * pow4(t.air_temp + WT_CONV_K);
  const double nr_water = (t.short_rad * (1. - WT_ALBEDO_W) + net_long);
  const double nr_ice = (t.short_rad * (1. - WT_ALBEDO_I) + net_long);
  if (t.loclake_area > 0.) {
    loclake_temp(t, nr_ice, nr_water, lat_heat, &tmp, &ice);
    gw_used = 1;
    loclake = tmp;
    out[1] = out[0] = loclake;
    out[7] = ice;
  }
  if (t.locwetl_area > 0.) {
    locwetl_temp(t, nr_ice, nr_water, lat_heat, loclake, gw_used, &tmp, &ice);
    gw_used = 1;
    locwetl = tmp;
    out[2] = out[0] = locwetl;
    out[8] = ice;
  }
  if (t.glolake_area > 0.) {
    mix = local_mix(t, tot_in, in_temp, loclake, locwetl);
    lake_temp(t, 3, nr_ice, nr_water, lat_heat, mix, gw_used, &tmp, &ice);
    gw_used = 1;
    glolake = tmp;
    out[3] = out[0] = glolake;
    out[9] = ice;
  }
  if (t.res_area > 0.) {
    mix = t.glolake_area <= 0. ? local_mix(t, tot_in, in_temp, loclake, locwetl) : glolake;
    lake_temp(t, 4, nr_ice, nr_water, lat_heat, mix, gw_used, &tmp, &ice);
    gw_used = 1;
    res = tmp;
    out[4] = out[0] = res;
    out[10] = ice;
  }
  if (t.glowetl_area > 0.) {
    if (t.res_area > 0.) mix = res;
    else if (t.glolake_area <= 0.) mix = local_mix(t, tot_in, in_temp, loclake, locwetl);
    else if (t.glolake_area > 0.) mix = glolake;
    lake_temp(t, 5, nr_ice, nr_water, lat_heat, mix, gw_used, &tmp, &ice);
    gw_used = 1;
    glowetl = tmp;
    out[5] = out[0] = glowetl;
    out[11] = ice;
  }
  if (t.has_outflow != 0. || t.river_length_check != 55.) {
    if (t.glowetl_area > 0.) mix = glowetl;
    else if (t.res_area > 0.) mix = res;
    else if (t.glolake_area > 0.) mix = glolake;
    else if (t.glolake_area <= 0.) mix = local_mix(t, tot_in, in_temp, loclake, locwetl);
    river_temp(t, nr_ice, nr_water, lat_heat, mix, gw_used, &tmp, &ice);
    out[0] = tmp;
    out[6] = ice;
  }
}


}  // namespace wt
}  // namespace wg
