// The drop-in stand-ins of include/wg_gpu.hpp instantiated with the reference's
// own state-file and calibration classes (wghmStateFile.h, snowInElevationFile.h,
// additionalOutputInputFile.h, calib_param.h), exactly as integrate_wghm_ passes
// them (integrateWGHM.cpp:779, 797-798, 830-847).  Compiled with -fsyntax-only
// against the reference's headers where its sources exist; nothing runs.
#include "additionalOutputInputFile.h"
#include "calib_param.h"
#include "snowInElevationFile.h"
#include "grid.h"
#include "wghmStateFile.h"
#include "wg_gpu.hpp"

// the reference's own grid types filled from the device's output grids, for its writers
void output_grids(wg::DailyWaterBalanceGpu &dailyWaterBalance, wg::RoutingGpu &routing, MonthlyGrid<false> &mg,
                  MonthlyGrid<> &mg_storage, DailyGrid<false> &dg) {
  dailyWaterBalance.monthly_grid(6, 0, mg);            // G_monthlyPrecipitation
  dailyWaterBalance.monthly_grid(6 + 29, 0, mg_storage);   // G_monthlyCanopyStorage
  dailyWaterBalance.daily_grid(0, 0, dg);              // G_daily365Precip
  routing.monthly_grid(0, 0, mg);                      // G_monthlyRiverAvail
  routing.daily_grid(0, 0, dg);                        // G_daily365RiverAvail
}

void day_loop(wg::DailyWaterBalanceGpu &dailyWaterBalance, wg::RoutingGpu &routing, WghmStateFile &wghmState,
              AdditionalOutputInputFile &additionalOutIn, SnowInElevationFile &snow_in_elevation,
              calibParamClass &calParam, const double *contfreq, int ncell) {
  const short last_day_in_month[12] = {30, 58, 89, 119, 150, 180, 211, 242, 272, 303, 333, 364};
  short day = 1, month = 0, day_in_month = 1, year = 2000, readinstatus = 0;
  for (int n = 0; n < ncell; ++n)
    dailyWaterBalance.calcNewDay(day, month, day_in_month, last_day_in_month[month], year, n, wghmState,
                                 additionalOutIn, snow_in_elevation, readinstatus, calParam);
  routing.calcNextDay_M(month);
  routing.routing(year, day, month, day_in_month, last_day_in_month[month], wghmState, additionalOutIn,
                  readinstatus, calParam);
  routing.updateLandAreaFrac(additionalOutIn);
  for (int n = 0; n < ncell; ++n) {
    const double landAreaFrac = routing.getLandAreaFrac(n);
    for (short elev = 0; elev <= 100; elev++)
      snow_in_elevation.snowInElevation(n, elev) =
          dailyWaterBalance.G_SnowInElevation(n, elev) * landAreaFrac / contfreq[n];
    wghmState.cell(n).canopy(0) = dailyWaterBalance.G_canopyWaterContent[n] * landAreaFrac / contfreq[n];
    wghmState.cell(n).snow(0) = dailyWaterBalance.G_snow[n] * landAreaFrac / contfreq[n];
    wghmState.cell(n).soil(0) = dailyWaterBalance.G_soilWaterContent[n] * landAreaFrac / contfreq[n];
  }
  routing.annualWaterUsePostProcessing(year, additionalOutIn);
}
