// ref_harness.cpp -- drives the reference's own daily.cpp / routing.cpp object
// code over a synthetic region, the way integrate_wghm_ does
// (source/integrateWGHM.cpp:280-800), and dumps the resulting state.
//
// TEST INFRASTRUCTURE ONLY.  Built from the reference sources by
// oracle/Makefile (target "ref") into oracle/_ref/; it exists in the build
// container only and pins the C restatement (wg_oracle.c) to the reference.
//
// Inputs (directory argv[1], written by oracle/ref_case.py): the UNF grids
// read by geo.init and routing.init, LAI_22.DAT, LCT_22.DAT, params.json,
// config.txt, plus raw little-endian arrays for what the harness sets directly.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>
#include <array>
#include <algorithm>
#include <initializer_list>
#include <type_traits>
#include <iomanip>
#include <set>
#include <list>
#include <functional>
#include <chrono>
#include <omp.h>
// The harness needs write access to a few members the reference keeps private
// (laiClass::G_LAImax, calibParamClass::calibParamJson, LAI state for the dump).
#define private public
#define protected public
#include "globals.h"
#include "calib_param.h"
#include "json11.hpp"
#undef private
#undef protected

calibParamClass calibParam;   // defined in watergap.cpp in the reference, which the harness replaces

template <class T>
static std::vector<T> read_raw(const std::string &path, size_t count) {
  std::vector<T> v(count);
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) { fprintf(stderr, "harness: cannot open %s\n", path.c_str()); exit(2); }
  if (fread(v.data(), sizeof(T), count, f) != count) { fprintf(stderr, "harness: short read %s\n", path.c_str()); exit(2); }
  fclose(f);
  return v;
}

static void write_raw(FILE *f, const double *p, size_t n) { fwrite(p, sizeof(double), n, f); }

int main(int argc, char **argv) {
  if (argc < 3) { fprintf(stderr, "usage: %s <case dir> <out file>\n", argv[0]); return 1; }
  std::string dir = argv[1];
  int ncase, ndays, doy0, year0, resopt, velo, nstation, nsnap, wtemp = 0, frac = 0, wuse = 0, statcorr = 0;
  int outputs = 0;
  {
    std::ifstream m(dir + "/meta.txt");
    m >> ncase >> ndays >> doy0 >> year0 >> resopt >> velo >> nstation >> nsnap;
    if (!m) { fprintf(stderr, "harness: bad meta.txt\n"); return 2; }
    if (!(m >> wtemp)) wtemp = 0;   // optional: water temperature (options.calc_wtemp)
    if (!(m >> frac)) frac = 0;     // optional: options.fractionalRoutingOpt
    if (!(m >> wuse)) wuse = 0;     // optional: water use (options.subtract_use = 2); 1/2 cell-local
                                    // (2: delayed satisfaction), 3/4 the same with the NUs of global
                                    // lakes' riparian cells aggregated (aggrNUsGloLakResOpt = 1)
    if (!(m >> statcorr)) statcorr = 0;   // optional: options.statcorrOpt
    if (!(m >> outputs)) outputs = 0;     // optional: the monthly output grids (1: grid_store = 2),
                                          // and the daily 365 grids as well (2: grid_store = 6)
  }
  std::vector<int> snap_days(nsnap);
  {
    std::ifstream m(dir + "/snapshots.txt");
    for (int i = 0; i < nsnap; i++) m >> snap_days[i];
  }

  // options of the hot path (integrateWGHM.cpp / option.cpp defaults, then the configs' switches)
  options.input_dir = dir; options.output_dir = dir; options.routing_dir = dir; options.climate_dir = dir;
  options.water_use_dir = dir; options.land_cover_dir = dir;
  options.basin = 1; options.fileEndianType = 2; options.grid_store = 0; options.grid_store_TypeForStorages = 0;
  options.day_store = 0; options.cloud = 2; options.intercept = 1; options.calc_albedo = 0;
  options.rout_prepare = 0; options.timeStepCheckFlag = 0; options.riverveloOpt = velo; options.time_series = 1;
  options.subtract_use = 0; options.use_alloc = 0; options.delayedUseSatisfaction = 0; options.petOpt = 0;
  options.clclOpt = 0; options.permaOpt = 0; options.resOpt = resopt; options.landCoverOpt = 0; options.use_kc = 0;
  options.statcorrOpt = statcorr; options.aridareaOpt = 0; options.fractionalRoutingOpt = frac; options.riverEvapoOpt = 0;
  options.aggrNUsGloLakResOpt = 0; options.climate_spatial_resolution = 0; options.resYearOpt = 0;
  options.resYearReference = 2000; options.resYearFirstToUse = 1900; options.resYearLastToUse = 2010;
  options.antNatOpt = 0; options.resNUsMeanYearFirst = 1971; options.resNUsMeanYearLast = 2000;
  // calc_wtemp and fractionalRoutingOpt set directly (the option file parser
  // switches fractional routing on with calc_wtemp, option.cpp:591-593)
  // water use: net abstractions from the yearly G_NETUSE_*_m3 files, satisfied in
  // the cell itself (use_alloc, delayedUseSatisfaction and aggrNUsGloLakResOpt off)
  if (wuse) options.subtract_use = 2;
  if (wuse == 2 || wuse == 4) options.delayedUseSatisfaction = 1;   // unmet demand carried to the next day
  if (wuse >= 3) options.aggrNUsGloLakResOpt = 1;   // GLWD units from <case>/GLWDunits.UNF4
  if (outputs) {   // monthly output grids, storages at the month's end (grid_store_TypeForStorages 0)
    options.grid_store = 2;
    options.outMinMaxRiverAvail = 1;
    if (wtemp) { options.outWaterTempMonthly = 1; options.outWaterTempMonthlyAllSWB = 1; }   // routing.cpp:4375-4458
  }
  if (outputs == 2) {   // and the vertical balance's daily 365 grids (daily.cpp:1388-1399, 1472-1540)
    options.grid_store = 6;
    options.outPrecDaily = 1; options.outTemp = 1; options.outPETDaily = 1; options.outTotalPETDaily = 1;
    options.outLAIDaily = 1; options.outAlbedoDaily = 1; options.outInterceptionDaily = 1;
    options.outCanopyWaterDaily = 1; options.outmaxCanopyWaterDaily = 1; options.outSnowFallDaily = 1;
    options.outSnowMeltDaily = 1; options.outSWEDaily = 1; options.outSnowCoverDaily = 1;
    options.outSoilWaterDaily = 1; options.outSurfaceRunoffDaily = 1; options.outGWRechargeDaily = 1;
    options.outExtRadiationDaily = 1; options.outShortDownRadiationDaily = 1; options.outShortUpRadiationDaily = 1;
    options.outNetShortWaveRadiationDaily = 1; options.outNetLongWaveRadiationDaily = 1;
    options.outNetRadiationDaily = 1; options.outSingleStoragesDaily = 1;
    // and routing's daily grids (routing.cpp:4113-4210, 4620-4634)
    options.outRiverAvailDaily = 1; options.outRiverVeloDaily = 1; options.outCellRunoffDaily = 1;
    options.outCellSurfaceDaily = 1; options.outGWRunoffDaily = 1; options.outLandAreaFracDaily = 1;
    options.outCellAETDaily = 1;
  }
  options.glacierOpt = 0; options.calc_wtemp = wtemp; options.start_year = year0; options.end_year = year0;
  options.init_years = 0; options.time_step = 1; options.outLAImax = 0;

  ConfigFile cfg(dir + "/config.txt", year0, 1, "OL");

  geo.init(dir, 2);
  auto lct = read_raw<unsigned char>(dir + "/c_lct.bin", ncase);
  auto built = read_raw<float>(dir + "/c_built_up.bin", ncase);
  auto smax = read_raw<float>(dir + "/c_smax.bin", ncase);
  auto laimax = read_raw<float>(dir + "/c_lai_max.bin", ncase);
  auto fg = read_raw<float>(dir + "/c_gw_factor.bin", ncase);
  auto rg = read_raw<short>(dir + "/c_rg_max.bin", ncase);
  auto tex = read_raw<signed char>(dir + "/c_texture.bin", ncase);
  auto aind = read_raw<short>(dir + "/c_aindex.bin", ncase);
  auto elev = read_raw<short>(dir + "/c_elev.bin", (size_t)ncase * 101);
  auto stations = read_raw<int>(dir + "/c_stations.bin", nstation);
  for (int n = 0; n < ng; n++) {
    land.G_landCover[n] = n < ncase ? (char)lct[n] : 1;
    land.G_built_up[n] = n < ncase ? built[n] : 0.f;
    G_aindex[n] = n < ncase ? aind[n] : 0;
    G_toBeCalculated[n] = 1;
  }

  // cell-specific calibration parameters: the JSON object calibParamClass::getValue reads
  {
    std::ifstream f(dir + "/params.json");
    std::stringstream ss; ss << f.rdbuf();
    std::string err;
    calibParam.calibParamJson = json11::Json::parse(ss.str(), err);
    if (!err.empty()) { fprintf(stderr, "harness: json: %s\n", err.c_str()); return 2; }
  }

  WghmStateFile wghmState(ng, 31);
  AdditionalOutputInputFile additionalOutIn;
  SnowInElevationFile snowIO;

  cbasin.cellNum.clear();
  for (int i = 0; i < nstation; i++) cbasin.cellNum.push_back(stations[i] + 1);
  cbasin.numberOfCalibBasins = 0;

  lai.init(dir, dir, land.G_landCover, additionalOutIn, calibParam);
  for (int n = 0; n < ncase; n++) lai.G_LAImax[n] = laimax[n];
  dailyWaterBalance.init(dir, nstation);
  routing.init(nstation, cfg, wghmState, additionalOutIn);
  routing.initLakeDepthActive(calibParam);
  routing.initWetlDepthActive(calibParam);
  routing.initFractionStatus();
  routing.setStoragesToZero();
  routing.setLakeWetlToMaximum(options.start_year);
  for (int n = 0; n < ng; n++) {
    dailyWaterBalance.G_gammaHBV[n] = calibParam.getValue(P_GAMRUN_C, n);
    dailyWaterBalance.G_cellCorrFact[n] = calibParam.getValue(P_CFA, n);
    routing.G_statCorrFact[n] = calibParam.getValue(P_CFS, n);
  }
  dailyWaterBalance.setStoragesToZero();
  for (int n = 0; n < ng; n++) {
    maxSoilWaterCap.G_Smax[n] = n < ncase ? smax[n] : 0.f;
    GW.setgwFactor(n, n < ncase ? fg[n] : 0.f);
    GW.setRgmax(n, n < ncase ? rg[n] : 0);
    GW.G_texture[n] = n < ncase ? tex[n] : 0;
    for (int e = 0; e < 101; e++) dailyWaterBalance.G_Elevation(n, e) = n < ncase ? elev[(size_t)n * 101 + e] : 0;
  }

  FILE *out = fopen(argv[2], "wb");
  if (!out) { fprintf(stderr, "harness: cannot write %s\n", argv[2]); return 2; }
  // the LAI factors the reference derived (checked against the restatement's inputs)
  {
    std::vector<double> la(18), lb(18);
    for (int i = 0; i < 18; i++) { la[i] = lai.lai_factor_a[i]; lb[i] = lai.lai_factor_b[i]; }
    write_raw(out, la.data(), 18); write_raw(out, lb.data(), 18);
    std::vector<double> g(ncase);
    for (int n = 0; n < ncase; n++) g[n] = routing.G_riverBottomWidth[n];
    write_raw(out, g.data(), ncase);
    for (int n = 0; n < ncase; n++) g[n] = routing.G_landAreaFrac[n];
    write_raw(out, g.data(), ncase);
  }

  const short first_day_in_month[12] = {1, 32, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335};
  const short last_day_in_month[12] = {30, 58, 89, 119, 150, 180, 211, 242, 272, 303, 333, 364};
  auto P = read_raw<float>(dir + "/f_prec.bin", (size_t)ndays * ncase);
  auto T = read_raw<float>(dir + "/f_temp.bin", (size_t)ndays * ncase);
  auto S = read_raw<float>(dir + "/f_swrad.bin", (size_t)ndays * ncase);
  std::vector<float> LW;
  std::vector<double> q((size_t)ndays * nstation, 0.0);
  std::vector<double> wt_daily;   // water temperature state of the stations' cells after each day
  if (wtemp) {
    climate.init();   // allocates the month's daily grids (climate.cpp:44-56)
    LW = read_raw<float>(dir + "/f_lwrad.bin", (size_t)ndays * ncase);
    auto gwt = read_raw<float>(dir + "/c_gwtemp.bin", ncase);
    for (int n = 0; n < ng; n++) climate.G_GW_Temperature_y[n] = n < ncase ? (double)gwt[n] : 10.;
    wt_daily.assign((size_t)ndays * nstation, 0.0);
  }

  // the vertical pass runs the reference's OpenMP cell loop (integrateWGHM.cpp:767-783)
  // on WG_REF_THREADS threads (default 1); routing is serial as in the reference.
  // Wall time of each pass goes to <case dir>/timing.txt (the CPU baseline).
  int nthreads = 1;
  if (const char *e = getenv("WG_REF_THREADS")) nthreads = std::max(1, atoi(e));
  omp_set_num_threads(nthreads);
  using clk = std::chrono::steady_clock;
  double t_vert = 0., t_rout = 0.;

  int year = year0;
  int doy = doy0;
  int snap_i = 0;
  bool year_started = false;
  for (int d = 0; d < ndays; d++) {
    if (!year_started || doy == 1) {
      dailyWaterBalance.annualInit();
      routing.annualInit(year, 1, additionalOutIn);
      // the year's net uses, read as integrate_wghm_ does (integrateWGHM.cpp:645-646)
      if (wuse) routing.dailyNUInit(dir, (short)year, calibParam);
      year_started = true;
    }
    int month = 0;
    while (month < 11 && doy >= first_day_in_month[month + 1]) month++;
    short day_in_month = (short)(doy - first_day_in_month[month] + 1);
    for (int n = 0; n < ncase; n++) {
      climateYear.G_precipitation_d365(n, doy - 1) = P[(size_t)d * ncase + n];
      climateYear.G_temperature_d365(n, doy - 1) = T[(size_t)d * ncase + n];
      climateYear.G_shortwave_d365(n, doy - 1) = S[(size_t)d * ncase + n];
    }
    if (wtemp)   // the water temperature reads the month's daily grids (routing.cpp:4275-4277)
      for (int n = 0; n < ncase; n++) {
        climate.G_shortwave_d(n, day_in_month - 1) = S[(size_t)d * ncase + n];
        climate.G_longwave_d(n, day_in_month - 1) = LW[(size_t)d * ncase + n];
        climate.G_temperature_d(n, day_in_month - 1) = T[(size_t)d * ncase + n];
      }
    const auto c0 = clk::now();
#pragma omp parallel for if (nthreads > 1)
    for (int n = 0; n < ng; ++n)
      if (geo.G_contcell[n])
        dailyWaterBalance.calcNewDay((short)doy, (short)month, day_in_month, last_day_in_month[month], (short)year, n,
                                     wghmState, additionalOutIn, snowIO, 0, calibParam);
    const auto c1 = clk::now();
    if (wuse) routing.calcNextDay_M(month);   // integrateWGHM.cpp:794-796
    routing.routing((short)year, (short)doy, (short)month, day_in_month, last_day_in_month[month], wghmState,
                    additionalOutIn, 0, calibParam);
    routing.updateLandAreaFrac(additionalOutIn);
    const auto c2 = clk::now();
    t_vert += std::chrono::duration<double>(c1 - c0).count();
    t_rout += std::chrono::duration<double>(c2 - c1).count();
    // end of the year (integrateWGHM.cpp:940-944), before the day's snapshot
    if (wuse && doy == 365) routing.annualWaterUsePostProcessing((short)year, additionalOutIn);
    for (int b = 0; b < nstation; b++) q[(size_t)d * nstation + b] = routing.dailyRiverDischarge(b, doy - 1);
    if (wtemp)
      for (int b = 0; b < nstation; b++) wt_daily[(size_t)d * nstation + b] = routing.G_RiverWTempPreStep[stations[b]];
    if (snap_i < nsnap && snap_days[snap_i] == d + 1) {
      // state snapshot after day d+1, fixed field order (read by oracle/ref_case.py)
      std::vector<double> g(ncase);
#define DUMP(expr) do { for (int n = 0; n < ncase; n++) g[n] = (double)(expr); write_raw(out, g.data(), ncase); } while (0)
      DUMP(dailyWaterBalance.G_canopyWaterContent[n]);
      DUMP(dailyWaterBalance.G_soilWaterContent[n]);
      DUMP(dailyWaterBalance.G_snow[n]);
      DUMP(lai.G_days_since_start[n]);
      DUMP(lai.G_GrowingStatus[n]);
      DUMP(lai.G_PrecSum[n]);
      DUMP(routing.G_groundwaterStorage[n]);
      DUMP(routing.G_riverStorage[n]);
      DUMP(routing.G_locLakeStorage[n]);
      DUMP(routing.G_locWetlStorage[n]);
      DUMP(routing.G_gloLakeStorage[n]);
      DUMP(routing.G_gloWetlStorage[n]);
      DUMP(routing.G_gloResStorage[n]);
      DUMP(routing.G_locLakeAreaReductionFactor[n]);
      DUMP(routing.G_locWetlAreaReductionFactor[n]);
      DUMP(routing.G_gloLakeEvapoReductionFactor[n]);
      DUMP(routing.G_gloWetlAreaReductionFactor[n]);
      DUMP(routing.G_gloResEvapoReductionFactor[n]);
      DUMP(routing.K_release[n]);
      DUMP(routing.G_landAreaFrac[n]);
      DUMP(routing.G_landAreaFracPrevTimestep[n]);
      DUMP(dailyWaterBalance.G_dailyLocalSurfaceRunoff[n]);
      DUMP(dailyWaterBalance.G_dailyGwRecharge[n]);
      for (int e = 1; e <= 100; e++) DUMP(dailyWaterBalance.G_SnowInElevation(n, e));
      if (wtemp) {   // water temperature state, the oracle's swb order
        DUMP(routing.G_RiverWTempPreStep[n]);
        DUMP(routing.G_locLakeTempPrevStep[n]);
        DUMP(routing.G_locWetlTempPrevStep[n]);
        DUMP(routing.G_gloLakeTempPrevStep[n]);
        DUMP(routing.G_reservoirTempPrevStep[n]);
        DUMP(routing.G_gloWetlandTempPrevStep[n]);
        DUMP(routing.G_iceThicknessRiver[n]);
        DUMP(routing.G_iceThicknesslocLake[n]);
        DUMP(routing.G_iceThicknesslocWetland[n]);
        DUMP(routing.G_iceThicknessGloLake[n]);
        DUMP(routing.G_iceThicknessReservoir[n]);
        DUMP(routing.G_iceThicknessGloWetland[n]);
        DUMP(routing.G_RiverAvailPreStep[n]);
      }
      if (wuse) {   // water-use state, the oracle's order
        DUMP(routing.G_dailyRemainingUse[n]);
        DUMP(routing.G_unsatisfiedNAsFromIrrig[n]);
        DUMP(routing.G_unsatisfiedNAsFromOtherSectors[n]);
        DUMP(routing.G_reducedReturnFlow[n]);
        DUMP(routing.G_withdrawalIrrigFromSwb[n]);
        DUMP(routing.G_consumptiveUseIrrigFromSwb[n]);
        DUMP(routing.G_totalUnsatisfiedUse[n]);
        DUMP(routing.G_UnsatisfiedUsePrevYear[n]);
        DUMP(routing.G_unsatisfiedNAsFromIrrigPrevYear[n]);
        DUMP(routing.G_unsatisfiedNAsFromOtherSectorsPrevYear[n]);
        DUMP(routing.G_reducedReturnFlowPrevYear[n]);
        DUMP(routing.G_actualUse[n]);
        if (wuse >= 3) DUMP(routing.G_unsatUseRiparian[n]);
      }
#undef DUMP
      snap_i++;
    }
    doy = doy % 365 + 1;
    if (doy == 1) year++;
  }
  write_raw(out, q.data(), q.size());
  if (wtemp) write_raw(out, wt_daily.data(), wt_daily.size());
  if (outputs) {   // the year's monthly grids [field][month][cell]: daily.cpp:1281-1386, routing.cpp:3964-4040, 4725-4737
    auto &w = dailyWaterBalance;
    const MonthlyGrid<false> *vert[] = {
        &w.G_monthlyPrecipitation, &w.G_monthlyTemperature, &w.G_monthlyExtRad, &w.G_monthlyShortUpRad,
        &w.G_monthlyShortDownRad, &w.G_monthlyNetShortRad, &w.G_monthlyNetLongRad, &w.G_monthlyNetRadiation,
        &w.G_monthlyOpenWaterPET, &w.G_monthlyPET, &w.G_monthlyAET, &w.G_monthlyLandAET, &w.G_monthlyLandAET_uncorr,
        &w.G_monthlyLAI, &w.G_monthlyAlbedo, &w.G_monthlyInterception, &w.G_monthlycanopyWaterContent,
        &w.G_monthlymaxcanopyWaterContent, &w.G_monthlySnowFall, &w.G_monthlyRainFall, &w.G_monthlySnowMelt,
        &w.G_monthlySnowEvap, &w.G_monthlySWE, &w.G_monthlySnowCoverAvg, &w.G_monthlySoilWaterAvg,
        &w.G_monthlyRunoff, &w.G_monthlyUrbanRunoff, &w.G_monthlySurfaceRunoff, &w.G_monthlyGwRecharge};
    const MonthlyGrid<> *vstor[] = {&w.G_monthlyCanopyStorage, &w.G_monthlySnowStorage, &w.G_monthlySoilStorage};
    const MonthlyGrid<false> *vlate[] = {&w.G_monthlyTotalPET};   // daily.cpp:1303
    const MonthlyGrid<false> *rout[] = {
        &routing.G_monthlyRiverAvail, &routing.G_monthlyMinRiverAvail, &routing.G_monthlyMaxRiverAvail,
        &routing.G_monthlyCellRunoff, &routing.G_monthlyVelocity, &routing.G_monthlyLocLakeStorage,
        &routing.G_monthlyLocWetlStorage, &routing.G_monthlyGloLakeStorage, &routing.G_monthlyGloWetlStorage,
        &routing.G_monthlyResStorage, &routing.G_monthlyRiverStorage, &routing.G_monthlyGwStorage,
        // routing's further grids (routing.cpp:3964-4238, 4525-4737, 5183-5186)
        &routing.G_monthlyOpenWaterEvap, &routing.G_monthlyCellSurfaceRunoff, &routing.G_monthlyGwRunoff,
        &routing.G_monthlyLandAreaFrac, &routing.G_monthlyLocWetlExtent, &routing.G_monthlyGloWetlExtent,
        &routing.G_monthlyResInflow, &routing.G_monthlyResOutflow, &routing.G_monthlyConsistentPrecip,
        &routing.G_monthlySurfStor, &routing.G_monthlyActualUse, &routing.G_monthlyNUg, &routing.G_monthlyCellAET,
        &routing.G_monthlyCellAETWCa};
    std::vector<double> buf((size_t)12 * ncase);
    auto dump = [&](auto *g) {
      for (int m = 0; m < 12; m++)
        for (int n = 0; n < ncase; n++) buf[(size_t)m * ncase + n] = (*g)(n, m);
      write_raw(out, buf.data(), buf.size());
    };
    for (auto *g : vert) dump(g);
    for (auto *g : vstor) dump(g);
    for (auto *g : vlate) dump(g);
    for (auto *g : rout) dump(g);
    if (wtemp) {   // the monthly mean water temperatures (routing.cpp:4375-4458)
      const MonthlyGrid<false> *wt[] = {
          &routing.G_monthlyMeanWaterTempRiver, &routing.G_monthlyMeanWaterTempLocLake,
          &routing.G_monthlyMeanWaterTempLocWetl, &routing.G_monthlyMeanWaterTempGloLake,
          &routing.G_monthlyMeanWaterTempReservoir, &routing.G_monthlyMeanWaterTempGloWetl};
      for (auto *g : wt) dump(g);
    }
  }
  if (outputs == 2) {   // the year's daily grids [field][day][cell] (daily.cpp:1388-1399, 1472-1540)
    auto &w = dailyWaterBalance;
    const DailyGrid<false> *dvert[] = {
        &w.G_daily365Precip, &w.G_daily365temp, &w.G_daily365PET, &w.G_daily365TotalPET, &w.G_daily365LAI,
        &w.G_daily365Kc, &w.G_daily365Albedo, &w.G_daily365Interception, &w.G_daily365canopyWaterContent,
        &w.G_daily365maxcanopyWaterContent, &w.G_daily365SnowFall, &w.G_daily365SnowMelt, &w.G_daily365SWE,
        &w.G_daily365SnowCoverAvg, &w.G_daily365SoilWaterAvg, &w.G_daily365SurfaceRunoff, &w.G_daily365GwRecharge,
        &w.G_daily365ExtRad, &w.G_daily365ShortDownRad, &w.G_daily365ShortUpRad, &w.G_daily365NetShortRad,
        &w.G_daily365NetLongRad, &w.G_daily365NetRadiation, &w.G_daily365CanopyStorage, &w.G_daily365SnowStorage,
        &w.G_daily365SoilStorage};
    const DailyGrid<false> *drout[] = {
        &routing.G_daily365RiverAvail, &routing.G_daily365Velocity, &routing.G_daily365CellRunoff,
        &routing.G_daily365CellRunoff_mm, &routing.G_daily365CellSurfaceRunoff, &routing.G_daily365GwRunoff,
        &routing.G_daily365LandAreaFrac, &routing.G_daily365ConsistentPrecip, &routing.G_daily365CellAET};
    std::vector<double> buf((size_t)365 * ncase);
    auto dump_day = [&](const DailyGrid<false> *g) {
      for (int d = 0; d < 365; d++)
        for (int n = 0; n < ncase; n++) buf[(size_t)d * ncase + n] = (*g)(n, d);
      write_raw(out, buf.data(), buf.size());
    };
    for (auto *g : dvert) dump_day(g);
    for (auto *g : drout) dump_day(g);
  }
  fclose(out);
  if (FILE *tf = fopen((dir + "/timing.txt").c_str(), "w")) {
    fprintf(tf, "%d %.9f %.9f %d %d\n", nthreads, t_vert, t_rout, ndays, ncase);
    fclose(tf);
  }
  return 0;
}
