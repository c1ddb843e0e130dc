// wg_wtemp.cuh -- water temperature of one cell and day on the GPU: the
// reference's calcWaterTempClass::calcWTemp (source/calcWaterTemp.cpp:48-1324),
// the energy balance of Beek et al. (2012) with the thermocline depth of
// Wanders et al. (2019), for the river and the five kinds of surface water
// body, with ice cover.  FP64, branch for branch as the reference; the
// arithmetic folds the constant factors (rho c, the ice growth per W/m2),
// multiplies by 1e-6 and by one refined reciprocal of the volume's heat
// capacity instead of dividing, takes pow(T, 4) as two squarings and the
// thermocline's pow from fm::pow -- a few ulp of rounding against the oracle,
// which keeps the reference's expression order.
//
// calcWTemp runs after a cell's routing (routing.cpp:4241-4513) and visits the
// water bodies in routing's own order (local lake, local wetland, global lake,
// reservoir, global wetland, river), each reading what its own routing left
// and what the bodies before it computed.  WtDay therefore runs each body as
// soon as routing_cell has finished it: the body's temperature and ice are
// written to the state at once, and only what the later bodies read (the
// local runoff, the temperature and volume of the next body's inflow) is
// carried on -- a few values instead of calcWTemp's sixty-odd arguments, so
// that the routing kernel holds them in registers.
#pragma once
#include "wg_device.h"
#include "wg_fastmath.cuh"

namespace wg {
namespace wt {

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

// What every water body of the cell reads on the day (calcWaterTempClass::transfer,
// calcWaterTemp.h:23-95, without the per-body entries).
struct WtCommon {
  double air;       // air temperature [degC]
  double prec;      // open-water precipitation [mm/d]
  double area;      // cell area [km2]
  double rain_k;    // temperature of precipitation and surface runoff [K]
  double gw_k;      // groundwater temperature [K]
  double nr_ice, nr_water, lat_heat;   // net radiation over ice / water, latent heat of evaporation
  // runoff into the cell's water bodies, and past them into the river (fractional routing)
  double local_runoff, local_gw_runoff, runoff_into_river, gw_runoff_into_river;
  bool keep_runoff;   // no outflow and no river (river length 55): the runoff stays in the water bodies
  int gw_used;        // an earlier water body took the local runoff
};

/* growth of the ice cover over one day [km] (same expression in every water body;
 * the river passes its storage where the others pass their temperature) */
__device__ __forceinline__ double ice_growth(double prev, const WtCommon &t, double net_rad_ice) {
  return (-(WT_K_H_ICE * prev) + (WT_K_H * (-t.air)) - net_rad_ice) * WT_ICE_PER_FLUX;
}

/* the clamps every water body ends with (calcWaterTemp.cpp:400-411 and the others) */
__device__ __forceinline__ void finish(const WtCommon &t, double *temp, double *ice, double ice_floor) {
  if (*temp > 60.) *temp = t.air;
  if (*temp < 1.e-10 && *temp != WT_NO_TEMP) *temp = 0.;
  if (*ice < ice_floor) *ice = 0.;
}

/* the energy balance of an open water body once its total energy (without the
 * sensible heat flux) and volume are known: the sensible heat flux may only
 * bring the temperature to the air temperature (calcWaterTemp.cpp:376-395) */
__device__ __forceinline__ double open_water_temp(const WtCommon &t, double energy, double sens, double vol) {
  if (!(vol > 0.)) return WT_NO_TEMP;
  const double inv = fm::rcp_pos(vol * WT_RC);   // vol > 0
  double temp = energy * inv - WT_CONV_K;
  energy -= sens;
  if (temp >= t.air) {
    temp = energy * inv - WT_CONV_K;
    if (temp < t.air) temp = t.air;
  } else {
    temp = energy * inv - WT_CONV_K;
    if (temp > t.air) temp = t.air;
  }
  return temp;
}

/* the water under an ice cover: stored energy minus the heat to the ice, mixed
 * with the day's inflows of temperature in_k [K] and volume in_vol */
__device__ __forceinline__ double under_ice_temp(double energy_stor, double sens, double vol, double ice, double area,
                                                 double in_vol, int has_inflow, double in_k) {
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

/* local lake, calcWaterTemp.cpp:258-407: pct its share of the cell [%], stor_prev
 * its storage before the day plus its capacity, evapo [mm] after any reduction,
 * rf its reduction factor; ice in *ice (in and out) */
__device__ __forceinline__ double loclake_temp(const WtCommon &t, double pct, double stor_prev, double temp_prev,
                                               double evapo, double rf, double *ice_io) {
  double gw = t.local_gw_runoff;
  double ice = *ice_io;
  double temp = 0.;
  int ice_max = 0;
  const double area = t.area * (pct / 100.) * rf;
  const double precip = t.prec * 1.e-6 * area;
  double surf = t.local_runoff - t.local_gw_runoff;
  if (t.keep_runoff) {
    surf += t.runoff_into_river - t.gw_runoff_into_river;
    gw += t.gw_runoff_into_river;
  }
  const double e_stor = stor_prev * WT_RC * (temp_prev + WT_CONV_K);
  if (t.air <= 0. || ice > 0.) {
    ice += ice_growth(temp_prev, t, t.nr_ice);
    if (ice * area >= stor_prev) {
      ice = stor_prev / area;
      if (precip + surf + t.local_gw_runoff <= 0.) ice_max = 1;
    }
  }
  if (!ice_max) {
    if (ice > 0.) {
      const double sens = WT_K_H_ICE * temp_prev * 1.e6 * 86400. * area;
      const double in_vol = precip + surf + t.local_gw_runoff;
      double in_k = 0.;
      if (in_vol > 0.)
        in_k = (precip * t.rain_k + surf * t.rain_k + t.local_gw_runoff * t.gw_k) / (precip + surf + t.local_gw_runoff);
      temp = under_ice_temp(e_stor, sens, stor_prev, ice, area, precip + surf + t.local_gw_runoff, in_vol > 0., in_k);
    } else {
      const double e_surf = surf * WT_RC * t.rain_k;
      const double e_prec = precip * WT_RC * t.rain_k;
      const double e_gw = gw * WT_RC * t.gw_k;
      const double e_rad = t.nr_water * 1.e6 * 86400. * area;
      const double sens = WT_K_H * (temp_prev - t.air) * 1.e6 * 86400. * area;
      const double lat = t.lat_heat * WT_RHO_W * (evapo * 1.e-6 * area);
      const double energy = e_stor + e_rad - lat + e_prec + e_surf + e_gw;
      const double vol = stor_prev + precip + surf + t.local_gw_runoff - (evapo * 1.e-6 * area);
      temp = open_water_temp(t, energy, sens, vol);
    }
  } else {
    temp = ice > 0. ? 0. : WT_NO_TEMP;
  }
  finish(t, &temp, &ice, 0.);
  *ice_io = ice;
  return temp;
}

/* local runoff into the first water body of the cell when no earlier one took it
 * (calcWaterTemp.cpp:447-457 and the same block of the others) */
__device__ __forceinline__ void take_runoff(const WtCommon &t, double *surf, double *gw, double *e_surf, double *e_gw) {
  if (t.keep_runoff) {
    *surf += t.runoff_into_river - t.gw_runoff_into_river;
    *gw += t.gw_runoff_into_river;
  }
  *surf += t.local_runoff - t.local_gw_runoff;
  *e_surf = *surf * WT_RC * t.rain_k;
  *gw += t.local_gw_runoff;
  *e_gw = *gw * WT_RC * t.gw_k;
}

/* local wetland, calcWaterTemp.cpp:420-568: inflow the local lake's outflow,
 * loclake_t the local lake's temperature of the day (used where the cell has one) */
__device__ __forceinline__ double locwetl_temp(const WtCommon &t, double pct, double stor_prev, double temp_prev,
                                               double evapo, double rf, double inflow, bool has_loclake,
                                               double loclake_t, double *ice_io) {
  double surf = 0., gw = 0., e_surf = 0., e_gw = 0., sum_runoff = 0.;
  double ice = *ice_io;
  double temp = 0.;
  int ice_max = 0;
  const double area = t.area * (pct / 100.) * rf;
  const double precip = t.prec * 1.e-6 * area;
  const double e_stor = stor_prev * WT_RC * (temp_prev + WT_CONV_K);
  if (!t.gw_used) {
    take_runoff(t, &surf, &gw, &e_surf, &e_gw);
    sum_runoff = gw + surf;
  }
  if (t.air <= 0. || ice > 0.) {
    ice += ice_growth(temp_prev, t, t.nr_ice);
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
      if (in_vol > 0.)
        in_k = (precip * t.rain_k + surf * t.rain_k + gw * t.gw_k + inflow * (loclake_t + WT_CONV_K)) /
               (precip + sum_runoff + inflow);
      temp = under_ice_temp(e_stor, sens, stor_prev, ice, area, precip + sum_runoff + inflow, in_vol > 0., in_k);
    } else {
      const double e_prec = precip * WT_RC * t.rain_k;
      const double e_rad = t.nr_water * 1.e6 * 86400. * area;
      const double sens = WT_K_H * ((temp_prev + WT_CONV_K) - (t.air + WT_CONV_K)) * 1.e6 * 86400. * area;
      const double lat = t.lat_heat * WT_RHO_W * (evapo * 1.e-6 * area);
      double e_in = 0.;
      if (has_loclake) e_in = inflow * WT_RC * (loclake_t + WT_CONV_K);
      const double energy = e_stor + e_rad - lat + e_prec + e_in + e_surf + e_gw;
      double vol = stor_prev + precip - (evapo * 1.e-6 * area) + inflow;
      if (!t.gw_used) vol += surf + gw;
      temp = open_water_temp(t, energy, sens, vol);
    }
  } else {
    temp = ice > 0. ? 0. : WT_NO_TEMP;
  }
  finish(t, &temp, &ice, 0.);
  *ice_io = ice;
  return temp;
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
 * storage that exchanges heat and their inflow, which the caller passes: area
 * [km2], stor_prev the storage that exchanges heat, inflow its volume and
 * mix_temp its temperature (negative: none) */
__device__ __forceinline__ double lake_temp(const WtCommon &t, double area, double stor_prev, double temp_prev,
                                            double evapo, double inflow, double mix_temp, double *ice_io) {
  double surf = 0., gw = 0., e_surf = 0., e_gw = 0., sum_runoff = 0.;
  double ice = *ice_io;
  double temp = 0.;
  int ice_max = 0;
  const double precip = t.prec * 1.e-6 * area;
  const double e_stor = stor_prev * WT_RC * (temp_prev + WT_CONV_K);
  if (!t.gw_used) {
    take_runoff(t, &surf, &gw, &e_surf, &e_gw);
    sum_runoff = surf + gw;
  }
  if (t.air <= 0. || ice > 0.) {
    ice += ice_growth(temp_prev, t, t.nr_ice);
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
          in_k = (precip * t.rain_k + surf * t.rain_k + gw * t.gw_k) / (precip + sum_runoff);
        else
          in_k = (precip * t.rain_k + surf * t.rain_k + gw * t.gw_k + inflow * (mix_temp + WT_CONV_K)) /
                 (precip + sum_runoff + inflow);
      }
      temp = under_ice_temp(e_stor, sens, stor_prev, ice, area, precip + sum_runoff + inflow, in_vol > 0., in_k);
    } else {
      const double e_prec = precip * WT_RC * t.rain_k;
      const double e_rad = t.nr_water * 1.e6 * 86400. * area;
      const double sens = WT_K_H * ((temp_prev + WT_CONV_K) - (t.air + WT_CONV_K)) * 1.e6 * 86400. * area;
      const double lat = t.lat_heat * WT_RHO_W * (evapo * 1.e-6 * area);
      double e_in = 0.;
      if (mix_temp >= 0.) e_in = ((mix_temp + WT_CONV_K) * inflow * WT_RC);
      const double energy = e_stor + e_rad - lat + e_prec + e_in + e_surf + e_gw;
      double vol = stor_prev + precip - (evapo * 1.e-6 * area) + inflow;
      if (!t.gw_used) vol += surf + gw;
      temp = open_water_temp(t, energy, sens, vol);
    }
  } else {
    temp = ice > 0. ? 0. : WT_NO_TEMP;
  }
  finish(t, &temp, &ice, 0.);
  *ice_io = ice;
  return temp;
}

/* river, calcWaterTemp.cpp:1097-1298: river_stor its storage after routing,
 * own_prev its temperature of the previous day, inflow the volume of the last
 * water body's outflow (or the upstream inflow) and mix_temp its temperature;
 * power-plant cooling (options.calc_wtemp = 2, calcWaterTemp.cpp:1263-1285) with
 * the day's withdrawal and consumption when calc_pp */
__device__ __forceinline__ double river_temp(const WtCommon &t, double river_stor, double bottom_width,
                                             double river_length, double cfa, double ow_pet, double own_prev,
                                             double inflow, double mix_temp, bool calc_pp, double pp_withdrawal,
                                             double pp_consumption, double *ice_io) {
  double area = 0., depth = 0.;
  double gw = t.runoff_into_river;   /* the reference starts its groundwater term from this field */
  double ice = *ice_io;
  int ice_max = 0;
  double temp = 0., vol = 0.;
  const double csa = river_stor / river_length;
  if (csa > 0.) {
    depth = -bottom_width / (4. * 1000.) + sqrt(bottom_width / 1000. * bottom_width / (16. * 1000.) + 0.5 * csa);
    area = river_stor / depth;
  }
  const double e_stor = river_stor * WT_RC * (own_prev + WT_CONV_K);
  const double precip = t.prec * area * 1.e-6;
  double surf = t.runoff_into_river - t.gw_runoff_into_river;
  if (!t.gw_used) {
    surf += (t.local_runoff - t.local_gw_runoff);
    gw += t.local_gw_runoff;
  }
  if (t.air <= 0. || ice >= 5.e-6) {
    if (area > 0.) {
      ice += ice_growth(river_stor, t, t.nr_ice);
      if (ice * area >= river_stor) {
        ice = river_stor / area;
        if (precip + surf + gw + inflow <= 0.) ice_max = 1;
      }
    } else {
      ice = 0.;
    }
  }
  if (!ice_max) {
    if (ice >= 5.e-6) {
      const double sens = WT_K_H_ICE * own_prev * 1.e6 * 86400. * area;
      vol = river_stor;
      const double in_vol = precip + surf + gw + inflow;
      double in_k = 0.;
      if (in_vol > 0.) {
        if (mix_temp < 0.)
          in_k = (precip * t.rain_k + surf * t.rain_k + gw * t.gw_k) / (precip + surf + gw);
        else
          in_k = (precip * t.rain_k + surf * t.rain_k + gw * t.gw_k + inflow * (mix_temp + WT_CONV_K)) /
                 (precip + surf + gw + inflow);
      }
      temp = under_ice_temp(e_stor, sens, vol, ice, area, precip + surf + gw + inflow, in_vol > 0., in_k);
    } else {
      const double e_surf = surf * WT_RC * t.rain_k;
      const double e_gw = gw * WT_RC * t.gw_k;
      const double evapo = ((1.0 - cfa) * t.prec + (cfa * ow_pet)) * area * 1.e-6;
      if (evapo >= river_stor + inflow + precip + surf + gw) {
        *ice_io = 0.;   /* everything evaporates; the ice record is reset */
        return WT_NO_TEMP;
      }
      const double e_prec = precip * WT_RC * t.rain_k;
      const double e_rad = t.nr_water * 1.e6 * 86400. * area;
      const double sens = WT_K_H * ((own_prev + WT_CONV_K) - (t.air + WT_CONV_K)) * 1.e6 * 86400. * area;
      const double lat = t.lat_heat * WT_RHO_W * evapo;
      double e_in = 0.;
      if (mix_temp >= 0.) e_in = inflow * WT_RC * (mix_temp + WT_CONV_K);
      const double energy = e_stor + e_rad - lat + e_in + e_prec + e_surf + e_gw;
      vol = river_stor + inflow + precip + surf + gw - evapo;
      temp = open_water_temp(t, energy, sens, vol);
    }
    if (temp >= 0. && pp_withdrawal > 0. && calc_pp) {
      if (ice >= 5.e-6) vol -= ice * area;
      if (vol > 0.) {
        const double wd = vol < pp_withdrawal ? vol : pp_withdrawal;
        const double ret = wd > pp_consumption ? wd - pp_consumption : 0.;
        if (ret > 0.)
          temp = (((vol - wd) * (temp + WT_CONV_K) + ret * (temp + 3. + WT_CONV_K)) / (vol - wd + ret)) - WT_CONV_K;
      }
    }
  } else {
    temp = ice > 0. ? 0. : WT_NO_TEMP;
  }
  finish(t, &temp, &ice, 5.e-6);
  *ice_io = ice;
  return temp;
}

/* mixing temperature of the cell's river inflow and its local wetland (or local
 * lake) outflow: the block calcWTemp repeats before each global water body and
 * the river where no global water body came before */
__device__ __forceinline__ double local_mix(double tot_in, double in_temp, double loclake_t, double locwetl_t,
                                            double locwetl_inflow, double locwetl_outflow) {
  double mix;
  if ((tot_in >= 0.) && (locwetl_outflow > 0.)) {
    mix = ((in_temp + WT_CONV_K) * tot_in + (locwetl_t + WT_CONV_K) * locwetl_outflow) / (tot_in + locwetl_outflow) -
          WT_CONV_K;
    if (mix < 0.) mix = 0.;
  } else if (tot_in > 0.) {
    mix = ((in_temp + WT_CONV_K) * tot_in + (loclake_t + WT_CONV_K) * locwetl_inflow) / (tot_in + locwetl_inflow) -
          WT_CONV_K;
    if (mix < 0.) mix = 0.;
  } else if (locwetl_inflow > 0.) {
    mix = loclake_t;
  } else {
    mix = WT_NO_TEMP;
  }
  return mix;
}

// One cell's calcWTemp on one day, driven by routing_cell: begin() with the day's
// inputs, runoff() once the runoff is split, one call per water body right after
// its routing (locals_done() between the local and the global ones), river() at
// the end.  Temperatures and ice go to the state [6][N] (index k * N + si; 0
// river, 1 local lake, 2 local wetland, 3 global lake, 4 reservoir, 5 global
// wetland); a water body without a temperature keeps the air temperature (at
// least 0), one the cell does not have gets no ice record (-9999).
struct WtDay {
  const DevWaterTemp *w;   // the state (temp/ice [k * N + si]) and the water-body areas (slot s)
  size_t si, N;
  int s;
  uint32_t fl;          // the cell's flag bits (which water bodies it has)
  WtCommon t;
  double tot_in, in_temp;   // upstream river inflow [km3] and its temperature (calcWaterTemp.cpp:76-90)
  double loclake_t, locwetl_t, ll_out, lw_out;   // the local bodies' temperatures and outflows
  double mix, chain_in;     // temperature and volume of the next global body's (or the river's) inflow
  double last;              // the temperature calcWTemp reports for the cell (its last water body's)
  // the monthly mean temperatures (routing.cpp:4375-4458): sums (k) and day
  // counts (6 + k) of the day's month at msum[k * ms], or null
  double *msum = nullptr;
  size_t ms = 0;
  __device__ __forceinline__ void file(int k, double tk) {
    if (msum && tk >= 0.) {   // a computed temperature (calcWTempReturns[k] >= 0)
      msum[k * ms] += tk;
      msum[(6 + k) * ms] += 1.;
    }
  }

  // tot_in/e_in: the upstream cells' river outflow of the day, summed, and the
  // energy it carries (sum of volume x rho c (T + 273.15))
  __device__ __forceinline__ void begin(const DevWaterTemp *w_, int s_, size_t si_, size_t N_, uint32_t fl_, double air,
                                        double sw, double lw, double prec, double area, double gw_temp,
                                        double tot_in_, double e_in) {
    w = w_; si = si_; N = N_; fl = fl_; s = s_;
    t.air = air;
    t.prec = prec;
    t.area = area;
    t.rain_k = wt_max(air - WT_PRECIP_T_CORR, 0.) + WT_CONV_K;
    t.gw_k = gw_temp + WT_CONV_K;
    t.lat_heat = air > 0. ? (2.501 - 0.002361 * air) * 1.e6 : 0.;
    const double net_long = lw - 1. * 0.00000005670374419 * pow4(air + WT_CONV_K);
    t.nr_water = (sw * (1. - WT_ALBEDO_W) + net_long);
    t.nr_ice = (sw * (1. - WT_ALBEDO_I) + net_long);
    t.keep_runoff = (fl & F_OUTLET) && w->len_check[s] == 55.;
    t.gw_used = 0;
    tot_in = tot_in_;
    in_temp = 0.;
    if (tot_in > 0.) in_temp = e_in / (tot_in * WT_RC) - WT_CONV_K;
    loclake_t = 0.; locwetl_t = 0.; ll_out = 0.; lw_out = 0.;
    last = WT_NO_TEMP;
  }
  __device__ __forceinline__ void runoff(double local_runoff, double local_gw_runoff, double into_river,
                                         double gw_into_river) {
    t.local_runoff = local_runoff;
    t.local_gw_runoff = local_gw_runoff;
    t.runoff_into_river = into_river;
    t.gw_runoff_into_river = gw_into_river;
  }
  __device__ __forceinline__ double &temp(int k) const { return w->temp[(size_t)k * N + si]; }
  __device__ __forceinline__ double &ice(int k) const { return w->ice[(size_t)k * N + si]; }
  __device__ __forceinline__ double keep() const { return t.air < 0. ? 0. : t.air; }
  __device__ __forceinline__ void absent(int k) {
    temp(k) = keep();
    ice(k) = WT_NO_TEMP;
  }
  __device__ __forceinline__ void put(int k, double temp_k, double ice_k) {
    temp(k) = temp_k == WT_NO_TEMP ? keep() : temp_k;
    ice(k) = ice_k;
    last = temp_k;
    file(k, temp_k);
  }
  // local lake: storage before the day plus capacity, evaporation after any
  // reduction, reduction factor, outflow
  __device__ __forceinline__ void loclake(double stor_prev, double evapo, double rf, double outflow) {
    double ic = ice(1);
    loclake_t = loclake_temp(t, w->ll_pct[s], stor_prev, temp(1), evapo, rf, &ic);
    t.gw_used = 1;
    ll_out = outflow;
    put(1, loclake_t, ic);
  }
  __device__ __forceinline__ void locwetl(double stor_prev, double evapo, double rf, double outflow) {
    double ic = ice(2);
    locwetl_t = locwetl_temp(t, w->lw_pct[s], stor_prev, temp(2), evapo, rf, ll_out, (fl & F_LOCLAKE) != 0, loclake_t, &ic);
    t.gw_used = 1;
    lw_out = outflow;
    put(2, locwetl_t, ic);
  }
  // after the local water bodies: the inflow of the first global one (or of the
  // river) and its temperature
  __device__ __forceinline__ void locals_done() {
    mix = local_mix(tot_in, in_temp, loclake_t, locwetl_t, ll_out, lw_out);
    chain_in = tot_in;
    if (fl & F_LOCWETL) chain_in += lw_out;
    else if (fl & F_LOCLAKE) chain_in += ll_out;
  }
  // a global lake (k 3), reservoir (4) or global wetland (5): area [km2], the
  // storage that exchanges heat, evaporation after any reduction, outflow;
  // glolake and res take their storage before the day (with the global lake's
  // capacity added), glowetl also its reduction factor
  __device__ __forceinline__ void global_body(int k, double area, double stor_prev, double evapo, double outflow) {
    double ic = ice(k);
    const double tk = lake_temp(t, area, stor_prev, temp(k), evapo, chain_in, mix, &ic);
    t.gw_used = 1;
    mix = tk;
    chain_in = outflow;
    put(k, tk, ic);
  }
  __device__ __forceinline__ void glolake(double stor_prev, double evapo, double outflow) {
    const double area = w->lake_km2[s];
    global_body(3, area, wt_min(stor_prev, thermocline(area, 0)), evapo, outflow);
  }
  __device__ __forceinline__ void res(double stor_prev, double evapo, double outflow) {
    const double area = w->res_km2[s];
    global_body(4, area, wt_min(stor_prev, thermocline(area, 1)), evapo, outflow);
  }
  __device__ __forceinline__ void glowetl(double stor_prev, double evapo, double rf, double outflow) {
    global_body(5, t.area * (w->gw_pct[s] / 100.) * rf, stor_prev, evapo, outflow);
  }
  // the river (where the cell has an outflow or a river), the water bodies the
  // cell does not have, and the river temperature the downstream cell reads
  __device__ __forceinline__ double river(double river_stor, double bottom_width, double river_length, double cfa,
                                          double ow_pet) {
    double ice0 = WT_NO_TEMP;
    if (!t.keep_runoff) {
      double ic = ice(0);
      // no power-plant cooling in this path (calc_wtemp = 1)
      last = river_temp(t, river_stor, bottom_width, river_length, cfa, ow_pet, temp(0), chain_in, mix, false, 0., 0.,
                        &ic);
      ice0 = ic;
    }
    file(0, last);   // the cell's reported temperature (calcWTempReturns[0])
    if (!(fl & F_LOCLAKE)) absent(1);
    if (!(fl & F_LOCWETL)) absent(2);
    if (!(fl & F_GLOLAKE)) absent(3);
    if (!(fl & F_RES)) absent(4);
    if (!(fl & F_GLOWETL)) absent(5);
    const double tr = last == WT_NO_TEMP ? keep() : last;
    temp(0) = tr;
    ice(0) = ice0;
    return tr;
  }
};

}  // namespace wt
}  // namespace wg
