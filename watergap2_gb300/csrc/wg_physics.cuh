// wg_physics.cuh -- per-cell physics of one day, as device functions.
//
// vertical_cell: dailyWaterBalanceClass::calcNewDay (source/daily.cpp:94-1257)
//                with laiClass::getDailyLai (source/lai.cpp:152-293);
// routing_cell:  one cell of routingClass::routing (source/routing.cpp:1835-4520)
//                with getRiverVelocity / getNewRiverVelocity (routing.cpp:7274-7341);
// fraction_update: the land-area-fraction update of routing.cpp:5034-5188 and
//                updateLandAreaFrac (routing.cpp:5343-5352).
//
// Expression order follows the reference term by term (the library is built
// with --fmad=false), so that results differ from the reference only where
// CUDA's exp/pow round differently from the host libm.
#pragma once
#include "wg_device.h"

namespace wg {

#define WG_MIN_STOR_VOL 1.e-15   // routingClass::minStorVol (routing.h:24)

__constant__ short c_first_day_in_month[12] = {1, 32, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335};

__device__ __forceinline__ int month_of(int doy) {
  int m = 0;
#pragma unroll
  for (int k = 1; k < 12; ++k) m += (doy >= c_first_day_in_month[k]) ? 1 : 0;
  return m;
}

struct VOut {
  double rs, gwr, transfer, owp, owpet;
  double land_in, land_evap, land_leak;
};

// laiClass::dailyLai_growing (lai.cpp:179-241)
__device__ __forceinline__ double lai_growing(int &days, int init, int &status, bool evergreen, bool arid,
                                              double lmin, double lmax, double &psum, double prec) {
  if (status == 0) {
    if (days >= init) {
      days++;
      psum += prec;
      if (psum > 40.) {
        if (days >= init + 30) { days = init + 30; status = 1; }
        return (lmin + (lmax - lmin) * (days - init) / 30.);
      }
      days = init;
      return lmin;
    }
    days++;
    psum += prec;
    return lmin;
  }
  if (days <= 30) {
    days--;
    if (evergreen) status = 0;
    if (days <= 0) { days = 0; status = 0; psum = 0.; }
    return (lmax - (lmax - lmin) * (30 - days) / 30.);
  }
  if (arid && (prec < 0.5)) days--;
  else days = 30 + init;
  return lmax;
}

// laiClass::dailyLai_nogrowing (lai.cpp:243-293)
__device__ __forceinline__ double lai_nogrowing(int &days, int init, int &status, double lmin, double lmax,
                                                double &psum, double prec) {
  if (status == 0) {
    if (days > init) {
      days++;
      psum += prec;
      if (psum > 40.) {
        if (days >= init + 30) { days = init + 30; status = 1; }
        return (lmin + (lmax - lmin) * (days - init) / 30.);
      }
      days = init;
      return lmin;
    }
    psum += prec;
    return lmin;
  }
  if (days <= 30) {
    days--;
    if (days <= 0) { days = 0; status = 0; psum = 0.; }
    return (lmax - (lmax - lmin) * (30 - days) / 30.);
  }
  days--;
  return lmax;
}

// dailyWaterBalanceClass::calcNewDay for slot i (daily.cpp:94-1257).
__device__ __forceinline__ void vertical_cell(const DevCells &c, const DevState &s, int i, double P, double T,
                                              double SW, double ext_rad, VOut &o) {
  const int n = c.n, B = c.nband;
  const uint32_t fl = c.flags[i];
  const double landAreaFrac = s.laf[i];
  const double prevLAF = (s.laf_started[i] == 1) ? s.laf_prev[i] : landAreaFrac;   // daily.cpp:159-169
  const double cfa = c.cfa[i];
  const bool arid = (fl & F_ARID) != 0;
  double transfer = 0.;

  double dailyPrec = c.mprec[i] * P;                           // daily.cpp:248
  const double dailyTempC = T;
  const double temp2 = dailyTempC + 237.3;
  const double e_s = 0.6108 * exp(17.27 * dailyTempC / temp2);
  const double alpha = c.alpha[i], maxDailyPET = c.pet_mxdy[i];
  const double a_c = arid ? 1.35 : 1.00, b_c = arid ? -0.35 : 0.00;

  // LAI state machine (lai.cpp:152-177)
  int days = s.lai_days[i], status = s.lai_status[i];
  double psum = s.lai_precsum[i];
  double dailyLai;
  if (dailyTempC > 8.)
    dailyLai = lai_growing(days, c.init_days[i], status, (fl & F_EVERGREEN) != 0, arid, c.lai_min[i], c.lai_max[i],
                           psum, dailyPrec);
  else
    dailyLai = lai_nogrowing(days, c.init_days[i], status, c.lai_min[i], c.lai_max[i], psum, dailyPrec);
  s.lai_days[i] = days;
  s.lai_status[i] = status;
  s.lai_precsum[i] = psum;

  const double albedo = (s.snow[i] > 3.) ? c.albedo_snow[i] : c.albedo[i];          // daily.cpp:366-379
  const double lat_heat = (dailyTempC > 0) ? 2.501 - 0.002361 * dailyTempC : 2.835;  // daily.cpp:382-387
  const double solar_rad_0 = (0.25 + 0.5) * ext_rad;
  const double conv = 0.0864 / lat_heat;
  const double solar_rad = conv * SW;
  double solar_fraction;                                                             // daily.cpp:430-448
  if (ext_rad == 0.) solar_fraction = 0.;
  else solar_fraction = solar_rad / solar_rad_0;
  if (solar_fraction > 1.) solar_fraction = 1.;
  const double ff = a_c * solar_fraction + b_c;
  const double net_emissivity = -0.02 + 0.261 * exp(-0.000777 * dailyTempC * dailyTempC);
  const double temp_K = dailyTempC + 273.2;
  const double net_lw = (-ff * net_emissivity * 0.000000004903 * pow(temp_K, 4.)) / lat_heat;
  const double net_sw = solar_rad * (1. - albedo);
  const double net_rad = c.mnetrad[i] * (net_sw + net_lw);
  const double ow_net_rad = solar_rad * (1. - 0.08) + net_lw;
  const double inc_svp = 4098. * e_s / (temp2 * temp2);                             // daily.cpp:484-532
  const double gamma = (0.0016286 * 101.3) / lat_heat;
  const double dailyPET = (net_rad <= 0.) ? 0. : alpha * (inc_svp * net_rad) / (inc_svp + gamma);
  const double owPET = (ow_net_rad <= 0.) ? 0. : alpha * (inc_svp * ow_net_rad) / (inc_svp + gamma);
  o.owp = dailyPrec;
  o.owpet = owPET;

  double lsc = 0., initialStorage = 0.;
  double canopyEvapo = 0., prec_to_soil = 0., soilPET = 0., snowEvapo = 0., effPrec = 0.;
  double immediate = 0., dailyAET = 0., runoff = 0., total = 0., gwr = 0., pot = 0.;
  double overflow = 0., neg_land_aet = 0., cellAET = 0., gwr_route = 0., leak = 0.;

  // interception (daily.cpp:825-895)
  double canopy = s.canopy[i];
  if (landAreaFrac <= 0.) {
    transfer = canopy;
    canopy = 0.;
  } else {
    canopy *= prevLAF / landAreaFrac;
    if (fabs(canopy) <= WG_MIN_STOR_VOL) canopy = 0.;
    initialStorage = canopy;
    if (dailyLai > 0.00001) {
      const double maxcs = c.mcwh[i] * dailyLai;
      const double deficiency = maxcs - canopy;
      if (dailyPrec < deficiency) {
        canopy += dailyPrec;
        prec_to_soil = 0.;
      } else {
        canopy = maxcs;
        prec_to_soil = dailyPrec - deficiency;
      }
      const double cwc = canopy;
      canopyEvapo = dailyPET * pow((cwc / maxcs), 0.66666666);
      if (canopyEvapo > cwc) {
        canopyEvapo = cwc;
        soilPET = dailyPET - cwc;
        canopy = 0.0;
      } else {
        canopy -= canopyEvapo;
        soilPET = dailyPET - canopyEvapo;
      }
    } else {
      prec_to_soil = dailyPrec;
      soilPET = dailyPET;
    }
    lsc += canopy - initialStorage;
  }
  s.canopy[i] = canopy;
  if (soilPET < 0.) soilPET = 0.0;

  // snow in elevation bands (daily.cpp:897-1062)
  double tempElevMax = 0., snowChange = 0., gsnow = 0.;
  int thresh = 0;
  const double t_snowfz = c.t_snowfz[i], t_snowmt = c.t_snowmt[i], ddf_m = c.ddf_m[i];
  for (int e = 0; e < B; ++e) {
    const size_t k = (size_t)e * n + i;
    double sb = s.snow_band[k];
    double temp_elev = dailyTempC - c.band_dt[k];
    if (landAreaFrac <= 0.) {
      transfer += sb / (double)B;
      sb = 0.;
      gsnow = 0.;
    } else {
      double effBefore, melt = 0.;
      sb = sb * prevLAF / landAreaFrac;
      if (fabs(sb) <= WG_MIN_STOR_VOL) sb = 0.;
      initialStorage = sb;
      if (sb > 1000.) {
        if (thresh == 0.) thresh = c.band_el[k];
        else if (thresh > 0.) temp_elev = dailyTempC - ((thresh - c.elev0[i]) * c.t_gradnt[i]);
      }
      if (temp_elev <= t_snowfz) {
        effBefore = 0.;
        sb += prec_to_soil;
        if (sb > soilPET) {
          sb -= soilPET;
          snowEvapo += soilPET;
        } else {
          snowEvapo += sb;
          sb = 0.;
        }
      } else {
        effBefore = prec_to_soil;
      }
      if (temp_elev > t_snowmt) {
        if (!(sb < 0.)) {
          melt = ddf_m * (temp_elev - t_snowmt);
          if (melt > sb) {
            melt = sb;
            sb = 0.;
          } else {
            sb -= melt;
          }
        }
      }
      snowChange += sb - initialStorage;
      if (e == 0) tempElevMax = temp_elev;
      gsnow += sb;
      effPrec += effBefore + melt;
    }
    s.snow_band[k] = sb;
  }
  if (landAreaFrac > 0.) {
    gsnow /= (double)B;
    effPrec /= (double)B;
    snowEvapo /= (double)B;
    snowChange /= (double)B;
    lsc += snowChange;
  }
  s.snow[i] = gsnow;

  // immediate runoff from built-up area (daily.cpp:1068-1071)
  const double bu = c.built_up[i];
  if (bu > 0.) {
    immediate = 0.5 * effPrec * bu;
    effPrec -= immediate;
  }

  // soil, AET, runoff, groundwater recharge (daily.cpp:1080-1239)
  double soil = s.soil[i];
  if (landAreaFrac <= 0.) {
    transfer += soil;
    transfer *= cfa;
    soil = 0.;
  } else {
    const double Smax = c.smax[i];
    soil *= prevLAF / landAreaFrac;
    initialStorage = soil;
    overflow = 0;
    if (soil > Smax) {
      overflow = soil - Smax;
      soil = Smax;
    }
    if (tempElevMax > t_snowfz) {
      if (Smax > 0.) {
        const double sat = soil / Smax;
        runoff = effPrec * pow(sat, c.gamma[i]);
        if (soilPET > (maxDailyPET - canopyEvapo) * sat) dailyAET = (maxDailyPET - canopyEvapo) * sat;
        else dailyAET = soilPET;
        soil += effPrec - dailyAET - runoff;
        if (fabs(soil) <= WG_MIN_STOR_VOL) soil = 0.;
        effPrec = 0.;
        if (soil < 0.) {
          dailyAET += soil;
          soil = 0.;
        }
        runoff *= cfa;
        immediate *= cfa;
        const double rgmax = c.rgmax[i], fg = c.fg[i];
        if (rgmax < (fg * runoff)) gwr = rgmax;
        else gwr = fg * runoff;
        // the reference's inland-sink test here reads a grid nothing fills (globals.cpp:8),
        // so the arid rule applies by land cover and texture alone
        if ((fl & F_ARID_GW) && (dailyPrec <= c.pcritgwa[i])) {
          pot = gwr;
          gwr = 0.;
        }
        runoff -= pot;
        pot /= cfa;
        soil += pot;
        if (soil > Smax) {
          overflow += soil - Smax;
          soil = Smax;
        }
        overflow *= cfa;
        total = runoff + immediate + overflow;
      }
    } else {
      overflow *= cfa;
      effPrec *= cfa;
      total += overflow + effPrec;
      dailyAET = 0.;
      leak -= cfa * immediate;   // built-up runoff is dropped in this branch
    }
    gwr_route = gwr;   // G_dailyGwRecharge (daily.cpp:1232)
    lsc += soil - initialStorage;
    cellAET = lsc * (cfa - 1.0) - dailyPrec * (cfa - 1.0) + (dailyAET + canopyEvapo + snowEvapo) * cfa;
    if (cellAET < 0.) {
      neg_land_aet = cellAET;
      cellAET = 0.;
    }
  }
  // surface runoff (daily.cpp:1244-1257)
  if (neg_land_aet < 0.) total = total + neg_land_aet;
  if (total < 0.) {
    leak -= total;
    total = 0.;
  }
  if ((total - gwr) < 0.) {
    soil += total - gwr;
    gwr = total;
  }
  s.soil[i] = soil;
  o.rs = total - gwr;
  o.gwr = gwr_route;
  o.transfer = transfer;
  o.land_in = dailyPrec;
  o.land_evap = cellAET;
  o.land_leak = leak;
}

struct RTerms {
  double p_ow, e_ow, leak;
};

// getRiverVelocity / getNewRiverVelocity (routing.cpp:7274-7341)
__device__ __forceinline__ double river_velocity(const DevCells &c, int i, double riverInflow, double S) {
  const double bw = c.bw[i];
  double v;
  if (c.velo_opt == 1) {
    const double Q = (riverInflow * 1000. * 1000. * 1000.) / (60. * 60. * 24.);
    const double depth = 0.349 * pow(Q, 0.341);
    const double csa = depth * (2.0 * depth + bw);
    const double wp = bw + 2.0 * depth * sqrt(5.0);
    const double hr = csa / wp;
    v = c.inv_mr[i] * pow(hr, (2. / 3.)) * c.sqrt_slope[i];
  } else {
    const double csa = (S / c.rlen[i]) * 1000000.;
    const double depth = -bw / 4.0 + sqrt(bw * bw / 16.0 + 0.5 * csa);
    const double wp = bw + 2.0 * depth * sqrt(5.0);
    const double hr = csa / wp;
    v = c.inv_mr[i] * pow(hr, (2. / 3.)) * c.sqrt_slope[i];
  }
  v = v * 86.4;
  return (v < 0.00001) ? 0.00001 : v;
}

// One cell of routingClass::routing (routing.cpp:1835-4520) given the vertical
// outputs and the summed upstream inflow; returns transportedVolume.
__device__ __forceinline__ double routing_cell(const DevCells &c, const DevState &s, int i, int doy, int month,
                                               const VOut &v, double inflow_up, RTerms &rt) {
  const uint32_t fl = c.flags[i];
  const double cellArea = c.area[i];
  const double cfa = c.cfa[i];
  const double laf = s.laf[i];
  rt.p_ow = 0.; rt.e_ow = 0.; rt.leak = 0.;
  double dlsr;
  if (laf <= 0.) dlsr = v.transfer * cellArea / 1000000. * s.laf_prev[i] / 100.;
  else dlsr = v.rs * cellArea / 1000000. * laf / 100.;
  // groundwater (routing.cpp:2061-2200)
  const double gw0 = s.gw[i];
  const double netGWin = v.gwr * cellArea * (laf / 100.) / 1000000.;
  double gw = gw0 * c.gw_e[i] + c.gw_ik[i] * netGWin * c.gw_ome[i];
  if (fabs(gw) <= WG_MIN_STOR_VOL) gw = 0.;
  double gw_runoff = gw0 - gw + netGWin;
  if (gw_runoff <= 0.) {
    gw_runoff = 0.;
    gw = gw0 + netGWin;
    if (fabs(gw) <= WG_MIN_STOR_VOL) gw = 0.;
  }
  s.gw[i] = gw;
  double inflow;
  if (!(fl & F_SINK)) {
    inflow = dlsr;
    inflow += gw_runoff;
  } else {
    if (laf == 0.) dlsr = v.transfer * cellArea / 1000000. * s.laf_prev[i] / 100.;
    else dlsr = v.rs * cellArea / 1000000. * laf / 100.;
    inflow = dlsr + gw_runoff;
  }
  const double owp = v.owp, owpet = v.owpet;
  double outflow = 0.;
  const double a6 = c.a6[i];

  if (fl & F_LOCLAKE) {  // local lake (routing.cpp:2318-2490)
    const double S0 = s.loclake[i], maxS = c.maxs_ll[i], rf = s.rf_loclake[i], p100 = c.ll100[i];
    double evapo = ((1.0 - cfa) * owp * rf) + (cfa * (owpet * rf));
    if (evapo < 0.) evapo = 0.;
    const double pin = (owp * rf) * a6 * p100;
    const double TI = inflow + pin;
    const double PETgwr = evapo * a6 * p100;
    double PETgwrMax = S0 + maxS + TI;
    const double avail = PETgwrMax;
    if (PETgwrMax < 0.) PETgwrMax = 0.;
    double S;
    if (PETgwr > PETgwrMax) {
      S = (-1.) * maxS;
      rt.e_ow += avail;
    } else {
      S = S0 + TI - PETgwr;
      rt.e_ow += PETgwr;
    }
    rt.p_ow += pin;
    if (S0 > 0.) {
      outflow = c.sw_k[i] * S0 * pow((S0 / maxS), 1.5);
      if (S <= 0.) outflow = 0;
      else if (outflow > S) outflow = S;
    } else outflow = 0.;
    S -= outflow;
    if (fabs(S) <= WG_MIN_STOR_VOL) S = 0.;
    if (S > maxS) {
      outflow += (S - maxS);
      S = maxS;
    }
    inflow = outflow;
    double r = 1. - pow(fabs(S - maxS) / (2. * maxS), c.evx[i]);
    if (r < 0.) r = 0.;
    if (r > 1.) r = 1.;
    s.loclake[i] = S;
    s.rf_loclake[i] = r;
  }
  if (fl & F_LOCWETL) {  // local wetland (routing.cpp:2495-2617)
    const double S0 = s.locwetl[i], maxS = c.maxs_lw[i], rf = s.rf_locwetl[i], p100 = c.lw100[i];
    double evapo = ((1.0 - cfa) * owp * rf) + (cfa * (owpet * rf));
    if (evapo < 0.) evapo = 0.;
    const double pin = (owp * rf * a6 * p100);
    const double TI = inflow + pin;
    const double PETgwr = evapo * a6 * p100;
    const double PETgwrMax = S0 + TI;
    double S;
    if (PETgwr > PETgwrMax) {
      S = 0.;
      rt.e_ow += PETgwrMax;
    } else {
      S = S0 + TI - PETgwr;
      rt.e_ow += PETgwr;
    }
    rt.p_ow += pin;
    if (fabs(S) <= WG_MIN_STOR_VOL) S = 0.;
    if (S > 0.) {
      outflow = c.sw_k[i] * S * pow((S / maxS), 2.5);
      if (outflow > S) outflow = S;
    } else outflow = 0.;
    S -= outflow;
    if (S > maxS) {
      outflow += (S - maxS);
      S = maxS;
    }
    inflow = outflow;
    double r = 1. - pow(fabs(S - maxS) / (maxS), c.evx[i]);
    if (r < 0.) r = 0.;
    if (r > 1.) r = 1.;
    s.locwetl[i] = S;
    s.rf_locwetl[i] = r;
  }
  inflow += inflow_up;   // routing.cpp:2623-2624
  if (fl & F_GLOLAKE) {  // global lake (routing.cpp:2630-2804)
    const double S0 = s.glolake[i], maxS = c.maxs_gl[i], rf = s.rf_glolake[i], la6 = c.la6[i];
    double evapo = ((1.0 - cfa) * owp) + (cfa * owpet * rf);
    if (evapo < 0.) evapo = 0.;
    const double pin = (owp * la6);
    const double TI = inflow + pin;
    const double PU = evapo * la6;
    const double PUmax = TI + maxS + S0;
    rt.p_ow += pin;
    double S;
    if (PU > PUmax) {
      S = (-1.) * maxS;
      outflow = 0.;
      rt.e_ow += PUmax;
    } else {
      S = S0 * c.sw_e[i] + c.sw_ik[i] * (TI - PU) * c.sw_ome[i];
      outflow = TI + S0 - S - PU;
      if (S > maxS) {
        outflow += (S - maxS);
        S = maxS;
      }
      if (outflow < 0.) {
        outflow = 0.;
        S = S0 + TI - PU;
      }
      rt.e_ow += PU;
    }
    if (fabs(S) <= WG_MIN_STOR_VOL) S = 0.;
    inflow = outflow;
    double r = 1. - pow(fabs(S - maxS) / (2. * maxS), c.evx[i]);
    if (r < 0.) r = 0.;
    if (r > 1.) r = 1.;
    s.glolake[i] = S;
    s.rf_glolake[i] = r;
  }
  if (fl & F_RES) {  // reservoir (routing.cpp:2807-3082)
    const double S0 = s.res[i], maxS = c.rcap[i], rf = s.rf_res[i], ra6 = c.ra6[i];
    double evapo = ((1.0 - cfa) * owp) + (cfa * (owpet * rf));
    if (evapo < 0.) evapo = 0.;
    const double pin = (owp * ra6);
    const double TI = inflow + pin;
    const double PETgwr = evapo * ra6;
    const double PETgwrMax = S0 + TI;
    rt.p_ow += pin;
    double S;
    if (PETgwr > PETgwrMax) {
      S = S0 + TI - PETgwrMax;
      rt.e_ow += PETgwrMax;
    } else {
      S = S0 + TI - PETgwr;
      rt.e_ow += PETgwr;
    }
    if (fabs(S) <= WG_MIN_STOR_VOL) S = 0.;
    double K = s.k_release[i];
    if (month == c.start_month[i] - 1 && doy == c_first_day_in_month[month]) {
      if (S < c.rcap01[i]) K = 0.1;
      else K = S / c.rcap085[i];
      s.k_release[i] = K;
    }
    const double prov_rel = c.prov_rel[i];
    double release;
    if (c.c_ratio[i] >= 0.5) release = K * prov_rel;
    else release = (c.c4[i] * K * prov_rel) + (c.one_m_c4[i] * inflow * 1000000000. / (24. * 3600.));
    if (S >= c.rcap01[i]) outflow = release * (24. * 3600.) / 1000000000.;
    else outflow = 0.1 * release * (24. * 3600.) / 1000000000.;
    if (outflow < 0.) outflow = 0.;
    S -= outflow;
    if (S > maxS) {
      outflow += (S - maxS);
      S = maxS;
    }
    if (S < 0.) {
      outflow += S;
      S = 0.;
    }
    inflow = outflow;
    double r = 1. - pow(fabs(S - maxS) / maxS, 2.81383);
    if (r < 0.) r = 0.;
    if (r > 1.) r = 1.;
    s.res[i] = S;
    s.rf_res[i] = r;
  }
  if (fl & F_GLOWETL) {  // global wetland (routing.cpp:3178-3297)
    const double S0 = s.glowetl[i], maxS = c.maxs_gw[i], rf = s.rf_glowetl[i], p100 = c.gw100[i];
    double evapo = ((1.0 - cfa) * (owp * rf)) + (cfa * (owpet * rf));
    if (evapo < 0.) evapo = 0.;
    const double pin = (owp * rf * a6 * p100);
    const double TI = inflow + pin;
    const double PETgwr = evapo * a6 * p100;
    const double PETgwrMax = TI + S0;
    rt.p_ow += pin;
    double S;
    if (PETgwr > PETgwrMax) {
      S = 0.;
      outflow = 0.;
      rt.e_ow += PETgwrMax;
    } else {
      S = S0 * c.sw_e[i] + c.sw_ik[i] * (TI - PETgwr) * c.sw_ome[i];
      outflow = TI + S0 - S - PETgwr;
      rt.e_ow += PETgwr;
    }
    if (S > maxS) {
      outflow += (S - maxS);
      S = maxS;
    }
    if (fabs(S) <= WG_MIN_STOR_VOL) S = 0.;
    inflow = outflow;
    double r = 1. - pow(fabs(S - maxS) / maxS, c.evx[i]);
    if (r < 0.) r = 0.;
    if (r > 1.) r = 1.;
    s.glowetl[i] = S;
    s.rf_glowetl[i] = r;
  }
  // river (routing.cpp:3385-3514)
  const double S0 = s.river[i];
  double velocity;
  if (c.velo_opt == 0) velocity = c.default_velocity;
  else velocity = river_velocity(c, i, inflow, S0);
  const double K = velocity / c.rlen[i];
  const double eK = exp(-1. * K);
  const double maxUse = inflow + (K * S0 * eK) / (1. - eK);
  double S, transported;
  if (0. > maxUse) {
    S = 0.;
    transported = inflow + S0 - maxUse;
  } else {
    S = S0 * eK + (1. / K) * (inflow - 0.) * (1. - eK);
    if (fabs(S) <= WG_MIN_STOR_VOL) S = 0.;
    transported = inflow + S0 - S - 0.;
  }
  if (transported < 0.) {
    rt.leak -= transported;
    transported = 0.;
  }
  s.river[i] = S;
  return transported;
}

// Land-area fraction for the next day (routing.cpp:5034-5188, 5343-5352).
__device__ __forceinline__ void fraction_update(const DevCells &c, const DevState &s, int i) {
  const uint32_t fl = c.flags[i];
  double fLocLake = 0., fLocWet = 0., fGloWet = 0.;
  if ((fl & F_LOCLAKE) && (s.rf_loclake[i] > 0.)) fLocLake = (s.rf_loclake[i] * c.ll[i] / 100.);
  if ((fl & F_LOCWETL) && (s.rf_locwetl[i] > 0.)) fLocWet = (s.rf_locwetl[i] * c.lw[i] / 100.);
  if ((fl & F_GLOWETL) && (s.rf_glowetl[i] > 0.)) fGloWet = (s.rf_glowetl[i] * c.gwet[i] / 100.);
  const double fswb = s.fswb_next[i];
  const double next = fLocLake + fLocWet + fGloWet;
  s.fswb_next[i] = next;
  const double changePct = next * 100. - fswb * 100.0;
  const double laf = s.laf[i];
  double lafNext = laf - (changePct + (0. * 100.));
  if (lafNext < 0.) lafNext = 0.;
  s.laf_started[i] = 1;
  s.laf_prev[i] = laf;
  s.laf[i] = lafNext;
}

}  // namespace wg
