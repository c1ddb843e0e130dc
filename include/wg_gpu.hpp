// wg_gpu.hpp -- C++ host side above the C ABI (include/wg_gpu.h).
//
// wg::Context owns one wg_ctx (RAII, exceptions instead of status codes).
// wg::DailyWaterBalanceGpu and wg::RoutingGpu are drop-in stand-ins for the
// reference's singletons `dailyWaterBalance` and `routing` inside
// integrate_wghm_ (source/integrateWGHM.cpp:755-799): the same method names and
// argument meaning as
//   dailyWaterBalanceClass::calcNewDay(day, month, day_in_month, last_day_in_month,
//                                      year, n, wghmState, additionalOutIn,
//                                      snow_in_elevation, readinstatus, calParam)
//                                      (source/daily.h:24)
//   routingClass::routing(year, day, month, day_in_month, last_day_in_month,
//                         wghmState, additionalOutIn, readinstatus, calParam)
//                         (source/routing.h:44-45)
//   routingClass::updateLandAreaFrac(additionalOutIn)  (source/routing.h:46)
// The reference calls calcNewDay once per cell from an OpenMP loop; here the
// first call of a day queues the whole grid and the other calls of that day
// return at once, so the loop can stay as it is; the days of a month run as one
// day-pipelined launch sequence (wg_set_deferred).  The state-file arguments are
// the reference's types (templates): at each month end the stand-ins write into
// them what the reference writes during the month.
#ifndef WG_GPU_HPP
#define WG_GPU_HPP

#include <atomic>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "wg_gpu.h"

namespace wg {

class Error : public std::runtime_error {
 public:
  Error(wg_status s, const std::string &what) : std::runtime_error(what), status(s) {}
  wg_status status;
};

class Context {
 public:
  Context(const wg_region &region, const wg_options &opt) {
    check(wg_create(&region, &opt, &ctx_), "wg_create");
  }
  ~Context() {
    if (ctx_) wg_destroy(ctx_);
  }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;

  wg_ctx *get() const { return ctx_; }
  int levels() const { return wg_num_levels(ctx_); }

  void upload_forcing(int day0, int ndays, const float *prec, const float *temp, const float *swrad) {
    check(wg_upload_forcing(ctx_, day0, ndays, prec, temp, swrad), "wg_upload_forcing");
  }
  void step_vertical(int doy, int fday) { check(wg_step_vertical(ctx_, doy, fday), "wg_step_vertical"); }
  void step_routing(int doy, int oday) { check(wg_step_routing(ctx_, doy, oday), "wg_step_routing"); }
  void run_days(int doy0, int fday0, int ndays) { check(wg_run_days(ctx_, doy0, fday0, ndays), "wg_run_days"); }
  void synchronize() { check(wg_synchronize(ctx_), "wg_synchronize"); }
  void state(wg_state_view &out) { check(wg_get_state(ctx_, &out), "wg_get_state"); }
  void set_state(const wg_state_view &in) { check(wg_set_state(ctx_, &in), "wg_set_state"); }
  void discharge(int day0, int ndays, double *out) {
    check(wg_get_discharge(ctx_, day0, ndays, out), "wg_get_discharge");
  }

  // day-pipelined run in pieces: steps [t_begin, t_end) of a run of ndays days
  int num_steps(int ndays) const { return wg_run_num_steps(ctx_, ndays); }
  void run_steps(int doy0, int fday0, int ndays, int t_begin, int t_end) {
    check(wg_run_steps(ctx_, doy0, fday0, ndays, t_begin, t_end), "wg_run_steps");
  }
  // next year's forcing on the copy stream while the current one runs
  void upload_forcing_async(int day0, int ndays, const float *prec, const float *temp, const float *swrad) {
    check(wg_upload_forcing_async(ctx_, day0, ndays, prec, temp, swrad), "wg_upload_forcing_async");
  }
  // the reference's in-memory yearly grids, cell-major [ncell][nd_file] native floats
  void upload_forcing_cells(int day0, int nd_file, int d_first, int ndays, const float *prec, const float *temp,
                            const float *swrad, bool overlap = false) {
    check(wg_upload_forcing_cells(ctx_, day0, nd_file, d_first, ndays, prec, temp, swrad, overlap ? 1 : 0),
          "wg_upload_forcing_cells");
  }
  // the reference's yearly UNF climate files as read (big-endian, cell-major)
  void upload_forcing_unf(int day0, int nd_file, int d_first, int ndays, const void *prec, const void *temp,
                          const void *swrad, bool overlap) {
    check(wg_upload_forcing_unf(ctx_, day0, nd_file, d_first, ndays, prec, temp, swrad, overlap ? 1 : 0),
          "wg_upload_forcing_unf");
  }
  // monthly aggregates of the routing outputs (river availability, min/max, storage, ...)
  void monthly_outputs(int nmonths, int doy_day0) {
    check(wg_monthly_outputs(ctx_, nmonths, doy_day0), "wg_monthly_outputs");
  }
  // the vertical balance's 33 monthly grids as well (which 6..38 of monthly())
  void monthly_outputs_vertical(bool enable) {
    check(wg_monthly_outputs_vertical(ctx_, enable ? 1 : 0), "wg_monthly_outputs_vertical");
  }
  void monthly(int which, int m0, int nm, double *out) {
    check(wg_get_monthly(ctx_, which, m0, nm, out), "wg_get_monthly");
  }
  // the vertical balance's daily grids for output days 0 .. ndays-1 (0: off)
  void daily_outputs_vertical(int ndays) {
    check(wg_daily_outputs_vertical(ctx_, ndays), "wg_daily_outputs_vertical");
  }
  void daily_vertical(int field, int day0, int nd, double *out) {
    check(wg_get_daily_vertical(ctx_, field, day0, nd, out), "wg_get_daily_vertical");
  }
  // routing's further monthly grids (which 39..52 of monthly()) and its daily grids
  void monthly_outputs_routing(bool enable) {
    check(wg_monthly_outputs_routing(ctx_, enable ? 1 : 0), "wg_monthly_outputs_routing");
  }
  void daily_outputs_routing(int ndays) { check(wg_daily_outputs_routing(ctx_, ndays), "wg_daily_outputs_routing"); }
  void daily_routing(int field, int day0, int nd, double *out) {
    check(wg_get_daily_routing(ctx_, field, day0, nd, out), "wg_get_daily_routing");
  }
  // water temperature (wg_options.water_temp = 1)
  void upload_longwave(int day0, int ndays, const float *longwave) {
    check(wg_upload_longwave(ctx_, day0, ndays, longwave), "wg_upload_longwave");
  }
  void set_water_temp_inputs(const float *gw_temp, const double *river_length_check) {
    check(wg_set_water_temp_inputs(ctx_, gw_temp, river_length_check), "wg_set_water_temp_inputs");
  }
  void water_temp(double *temp, double *ice) { check(wg_get_water_temp(ctx_, temp, ice), "wg_get_water_temp"); }
  void set_water_temp(const double *temp, const double *ice) {
    check(wg_set_water_temp(ctx_, temp, ice), "wg_set_water_temp");
  }
  void river_temp(int day0, int ndays, double *out) {
    check(wg_get_river_temp(ctx_, day0, ndays, out), "wg_get_river_temp");
  }
  // water use (wg_options.water_use = 1)
  void upload_water_use(int fday0, int ndays, int doy0, const double *nus_m3, const double *nug_m3,
                        const double *irrig_withdrawal_sw_m3, const double *irrig_consumptive_sw_m3) {
    check(wg_upload_water_use(ctx_, fday0, ndays, doy0, nus_m3, nug_m3, irrig_withdrawal_sw_m3,
                              irrig_consumptive_sw_m3),
          "wg_upload_water_use");
  }
  void set_water_use_inputs(const double *frac_return_gw_irrig) {
    check(wg_set_water_use_inputs(ctx_, frac_return_gw_irrig), "wg_set_water_use_inputs");
  }
  void water_use(double *out) { check(wg_get_water_use(ctx_, out), "wg_get_water_use"); }
  void set_water_use(const double *in) { check(wg_set_water_use(ctx_, in), "wg_set_water_use"); }

  void check(wg_status s, const char *what) const {
    if (s != WG_OK)   // without a context: why this thread's wg_create failed
      throw Error(s, std::string(what) + ": " + wg_status_string(s) + " " + wg_last_error(ctx_));
  }

 private:
  wg_ctx *ctx_ = nullptr;
};

// ---------------------------------------------------------------------------
// Drop-in stand-ins for the reference's singletons `dailyWaterBalance` and
// `routing` inside integrate_wghm_'s day loop (integrateWGHM.cpp:755-860):
//
//   for each day:   dailyWaterBalance.calcNewDay(...)  for every cell (OpenMP)
//                   routing.routing(...); routing.updateLandAreaFrac(...)
//   month end:      read routing.getLandAreaFrac(n), dailyWaterBalance.G_snow[n],
//                   .G_soilWaterContent[n], .G_canopyWaterContent[n],
//                   .G_SnowInElevation(n, elev) into the state files
//
// The context runs in deferred mode (wg_set_deferred): the first calcNewDay call
// of a day queues that day's whole-grid vertical balance, the other calls of the
// day return at once, and the routing call queues the day's routing; the days of
// a month run as one day-pipelined launch sequence when the month ends (the same
// bits as launching each day).  At the month's last day (day == last_day_in_month
// + 1, the reference's test) the shims then write what the reference writes
// during that month: the day-end routing storages of every day into the state
// file cells (routing.cpp:5001-5020), the water-use columns of the additional
// output (routing.cpp:5021-5030), the snow bands and the soil, canopy and snow
// columns (daily.cpp:1033-1035, 1258-1262).  Cell i of the region is grid cell
// n = i of the reference.  Forcing: the caller uploads each year's forcing
// (Context::upload_forcing, 365 days from slot slot_offset()) before the year's
// first day, as the reference reads its yearly .365 grids; day d of the year
// uses slot slot_offset() + d - 1, and so does its discharge record.  The
// calibration parameters gamma (P_GAMRUN_C) and the cell correction factor
// (P_CFA) are read from calParam at the first calcNewDay call and after
// reload_calib_param() (the reference changes them between runs,
// integrateWGHM.cpp:414-417).
// ---------------------------------------------------------------------------

namespace detail {
template <class T> struct first_arg;
template <class C, class R, class A, class... Rest> struct first_arg<R (C::*)(A, Rest...)> { using type = A; };
template <class C, class R, class A, class... Rest> struct first_arg<R (C::*)(A, Rest...) const> { using type = A; };
// calibParamClass::getValue(eCalibParam, n) (calib_param.h:131) for eCalibParam index k
template <class CP> double calib_value(CP &cp, int k, int n) {
  using K = typename first_arg<decltype(&CP::getValue)>::type;
  return cp.getValue(static_cast<K>(k), n);
}
}  // namespace detail

// What both stand-ins share: the context, the geometry of the state-file
// conversions, the host copies of the state read at month ends, the month's days.
class DropInCore {
 public:
  DropInCore(Context &c, const wg_region &r) : ctx(c), n(r.ncell), nband(r.nband), area(r.area_km2, r.area_km2 + r.ncell),
                                              contfreq(r.contfreq, r.contfreq + r.ncell) {
    // the continental share as geo.init leaves it (geo.cpp:25-45): at least the
    // share of local lakes, global lakes, local reservoirs (none) and reservoirs
    for (int i = 0; i < n; ++i) {
      double fw = 0.;
      fw += r.loc_lake[i];
      fw += r.glo_lake[i];
      fw += 0.;
      fw += r.glo_res[i];
      if (fw > contfreq[i]) contfreq[i] = fw;
    }
    ctx.check(wg_set_deferred(ctx.get(), 1), "wg_set_deferred");
    ctx.check(wg_record_daily_storages(ctx.get(), 1), "wg_record_daily_storages");
    canopy.resize(n); soil.resize(n); snow.resize(n); snow_band.resize((size_t)n * nband); laf.resize(n);
  }
  Context &ctx;
  const int n, nband;
  std::vector<double> area, contfreq;
  int slot_offset = 0;
  std::atomic<bool> expect_vertical{true};   // the next calcNewDay call starts a day
  bool params_loaded = false;
  std::vector<int> month_days;               // day_in_month of the month's routed days
  std::vector<int> month_slots;              // their output slots
  // host copies, valid after sync()
  std::vector<double> canopy, soil, snow, snow_band, laf;
  bool fresh = false;

  // run what is queued and copy the state the month end reads (the other
  // fields of the view stay null: wg_get_state skips them)
  void sync() {
    if (fresh) return;
    wg_state_view v{};
    v.canopy = canopy.data(); v.soil = soil.data(); v.snow = snow.data(); v.snow_band = snow_band.data();
    v.laf = laf.data();
    ctx.state(v);
    fresh = true;
  }
  // km3 -> mm over the continental area, as the reference writes its state file
  double to_mm(int i, double km3) const { return km3 / ((area[i] * (contfreq[i] / 100.)) / 1000000.); }
  // The reference's output grids (grid_store 2 and 5/6) from the device's, for its
  // own writers (daily.cpp:1969-2392, routing.cpp:6066-6834): a grid with
  // g(cell, month) of the 12 months from output month m0 (wg_get_monthly's which),
  // and with g(cell, day) of the 365 days from output day d0 (the vertical
  // balance's or routing's daily field).  The context's grids must be on
  // (Context::monthly_outputs and the others).
  template <class MonthlyGrid>
  void monthly_grid(int which, int m0, MonthlyGrid &g) {
    std::vector<double> v((size_t)12 * n);
    ctx.monthly(which, m0, 12, v.data());
    for (int m = 0; m < 12; ++m)
      for (int i = 0; i < n; ++i) g(i, m) = v[(size_t)m * n + i];
  }
  template <class DailyGrid>
  void daily_grid(bool routing, int field, int d0, DailyGrid &g) {
    std::vector<double> v((size_t)365 * n);
    if (routing) ctx.daily_routing(field, d0, 365, v.data());
    else ctx.daily_vertical(field, d0, 365, v.data());
    for (int d = 0; d < 365; ++d)
      for (int i = 0; i < n; ++i) g(i, d) = v[(size_t)d * n + i];
  }
  // band of the reference's 100 (1..100) -> this region's band
  double band_of_ref(int i, int elev) const {
    if (elev < 1 || elev > 100) return 0.;
    return snow_band[(size_t)i * nband + (size_t)(elev - 1) * nband / 100];
  }
};

// Stand-in for dailyWaterBalanceClass (daily.h:22-227) in the day loop.
class DailyWaterBalanceGpu {
 public:
  DailyWaterBalanceGpu(Context &c, const wg_region &r) : core(c, r), G_canopyWaterContent{this, 0},
                                                         G_snow{this, 1}, G_soilWaterContent{this, 2} {}

  template <class WghmStateFile, class AdditionalOutputInputFile, class SnowInElevationFile, class CalibParam>
  void calcNewDay(const short day, const short /*month*/, const short /*day_in_month*/,
                  const short last_day_in_month, const short /*year*/, const int /*n*/, WghmStateFile &,
                  AdditionalOutputInputFile &additionalOutIn, SnowInElevationFile &snow_in_elevation,
                  const short /*readinstatus*/, CalibParam &calParam) {
    // whole grid on the first call of the day (the call after the last routing
    // call); the remaining calls of the day return at once
    bool want = true;
    if (!core.expect_vertical.compare_exchange_strong(want, false)) return;
    if (!core.params_loaded) load_params(calParam);
    core.fresh = false;
    core.ctx.step_vertical(day, core.slot_offset + day - 1);
    if (day == last_day_in_month + 1) {
      // what calcNewDay writes on the month's last day, filled when the month has run
      AdditionalOutputInputFile *ao = &additionalOutIn;
      SnowInElevationFile *se = &snow_in_elevation;
      month_end = [this, ao, se]() {
        for (int i = 0; i < core.n; ++i) {
          for (int e = 1; e <= 100; ++e) se->snowInElevation(i, e) = core.band_of_ref(i, e);
          ao->additionalOutputInput(i, 20) = core.soil[i];
          ao->additionalOutputInput(i, 22) = core.canopy[i];
          ao->additionalOutputInput(i, 24) = core.snow[i];
        }
      };
    }
  }

  // the reference's monthly and daily grids of the vertical balance (DropInCore::monthly_grid)
  template <class MonthlyGrid>
  void monthly_grid(int which, int m0, MonthlyGrid &g) { core.monthly_grid(which, m0, g); }
  template <class DailyGrid>
  void daily_grid(int field, int d0, DailyGrid &g) { core.daily_grid(false, field, d0, g); }
  // the calibration parameters are read again at the next calcNewDay call
  void reload_calib_param() { core.params_loaded = false; }
  void set_slot_offset(int slot0) { core.slot_offset = slot0; }

  // the month-end reads of integrate_wghm_ (integrateWGHM.cpp:830-847)
  struct Field {
    DailyWaterBalanceGpu *self;
    int which;
    double operator[](int i) const {
      self->core.sync();
      const auto &v = which == 0 ? self->core.canopy : which == 1 ? self->core.snow : self->core.soil;
      return v[i];
    }
  };
  double G_SnowInElevation(int i, int elev) {
    core.sync();
    return core.band_of_ref(i, elev);
  }

  DropInCore core;
  Field G_canopyWaterContent, G_snow, G_soilWaterContent;
  std::function<void()> month_end;   // set on the month's last day, run by RoutingGpu

 private:
  template <class CalibParam>
  void load_params(CalibParam &cp) {
    std::vector<double> v(core.n);
    for (int k = 0; k < 2; ++k) {   // P_GAMRUN_C, P_CFA
      for (int i = 0; i < core.n; ++i) v[i] = detail::calib_value(cp, k, i);
      core.ctx.check(wg_set_calib_param(core.ctx.get(), k, v.data()), "wg_set_calib_param");
    }
    core.params_loaded = true;
  }
};

// Stand-in for routingClass (routing.h:22-594) in the day loop.
class RoutingGpu {
 public:
  explicit RoutingGpu(DailyWaterBalanceGpu &d) : dwb_(d), core_(d.core) {}

  template <class WghmStateFile, class AdditionalOutputInputFile, class CalibParam>
  void routing(const short /*year*/, short day, short /*month*/, const short day_in_month,
               const short last_day_in_month, WghmStateFile &wghmState, AdditionalOutputInputFile &additionalOutIn,
               const short /*readinstatus*/, CalibParam &) {
    const int slot = core_.slot_offset + day - 1;
    core_.fresh = false;
    core_.ctx.step_routing(day, slot);
    core_.expect_vertical.store(true);
    core_.month_days.push_back(day_in_month);
    core_.month_slots.push_back(slot);
    if (day == last_day_in_month + 1) month_end(wghmState, additionalOutIn);
  }
  // the reference's monthly and daily grids of routing (DropInCore::monthly_grid)
  template <class MonthlyGrid>
  void monthly_grid(int which, int m0, MonthlyGrid &g) { core_.monthly_grid(which, m0, g); }
  template <class DailyGrid>
  void daily_grid(int field, int d0, DailyGrid &g) { core_.daily_grid(true, field, d0, g); }
  // the land-area-fraction update is part of the queued routing (routing.cpp:5034-5188)
  template <class AdditionalOutputInputFile>
  void updateLandAreaFrac(AdditionalOutputInputFile &) {}
  double getLandAreaFrac(int i) {
    core_.sync();
    return core_.laf[i];
  }

  // Water use (wg_options.water_use): in place of dailyNUInit (routing.cpp:884-976),
  // the year's monthly net uses [12][ncell] in m3 as the yearly files hold them
  // (M_NETABSSW / M_NETABSGW applied) for forcing slots fday0.. starting on day of
  // year doy0; calcNextDay_M (routing.cpp:7405-7447) is the device's table row
  // lookup, so it is a no-op here.
  void dailyNUInit(int fday0, int ndays, int doy0, const double *nus_m3, const double *nug_m3,
                   const double *irrig_withdrawal_sw_m3, const double *irrig_consumptive_sw_m3) {
    core_.ctx.upload_water_use(fday0, ndays, doy0, nus_m3, nug_m3, irrig_withdrawal_sw_m3, irrig_consumptive_sw_m3);
  }
  void calcNextDay_M(const short /*month*/) {}
  // the year-end state change runs in the kernel on each cell's day 365; here the
  // columns the reference writes then (routing.cpp:5297-5305)
  template <class AdditionalOutputInputFile>
  void annualWaterUsePostProcessing(short /*year*/, AdditionalOutputInputFile &additionalOutIn) {
    std::vector<double> wu;
    if (!water_use(wu)) return;
    const size_t n = (size_t)core_.n;
    for (size_t i = 0; i < n; ++i) {
      additionalOutIn.additionalOutputInput((int)i, 3) = wu[6 * n + i];    // G_totalUnsatisfiedUse
      additionalOutIn.additionalOutputInput((int)i, 4) = wu[7 * n + i];    // G_UnsatisfiedUsePrevYear
      additionalOutIn.additionalOutputInput((int)i, 50) = wu[10 * n + i];  // G_reducedReturnFlowPrevYear
      additionalOutIn.additionalOutputInput((int)i, 51) = wu[8 * n + i];   // G_unsatisfiedNAsFromIrrigPrevYear
      additionalOutIn.additionalOutputInput((int)i, 52) = wu[9 * n + i];   // ...FromOtherSectorsPrevYear
      additionalOutIn.additionalOutputInput((int)i, 38) = wu[3 * n + i];   // G_reducedReturnFlow
      additionalOutIn.additionalOutputInput((int)i, 39) = wu[1 * n + i];   // G_unsatisfiedNAsFromIrrig
      additionalOutIn.additionalOutputInput((int)i, 49) = wu[2 * n + i];   // G_unsatisfiedNAsFromOtherSectors
    }
  }

 private:
  // the water-use state, false without water use
  bool water_use(std::vector<double> &wu) {
    wu.assign((size_t)WG_WU_NSTATE * core_.n, 0.);
    const wg_status s = wg_get_water_use(core_.ctx.get(), wu.data());
    if (s == WG_ERR_UNSUPPORTED) return false;
    core_.ctx.check(s, "wg_get_water_use");
    return true;
  }

  template <class WghmStateFile, class AdditionalOutputInputFile>
  void month_end(WghmStateFile &wghmState, AdditionalOutputInputFile &additionalOutIn) {
    core_.sync();   // runs the month
    const int n = core_.n, nd = (int)core_.month_slots.size();
    // the daily routing storages of the month's days (routing.cpp:5001-5020);
    // consecutive output slots are read in one call
    std::vector<double> ds;
    for (int k = 0; k < nd;) {
      int len = 1;
      while (k + len < nd && core_.month_slots[k + len] == core_.month_slots[k] + len) ++len;
      ds.resize((size_t)len * 7 * n);
      core_.ctx.check(wg_get_daily_storages(core_.ctx.get(), core_.month_slots[k], len, ds.data()),
                      "wg_get_daily_storages");
      for (int j = 0; j < len; ++j) {
        const int d = core_.month_days[k + j] - 1;
        const double *p = ds.data() + (size_t)j * 7 * n;
        for (int i = 0; i < n; ++i) {
          auto &cell = wghmState.cell(i);
          cell.locallake(d) = core_.to_mm(i, p[i]);
          cell.localwetland(d) = core_.to_mm(i, p[(size_t)n + i]);
          cell.globallake(d) = core_.to_mm(i, p[(size_t)2 * n + i]);
          cell.globalwetland(d) = core_.to_mm(i, p[(size_t)3 * n + i]);
          cell.reservoir(d) = core_.to_mm(i, p[(size_t)4 * n + i]);
          cell.river(d) = core_.to_mm(i, p[(size_t)5 * n + i]);
          cell.groundwater(d) = core_.to_mm(i, p[(size_t)6 * n + i]);
        }
      }
      k += len;
    }
    core_.month_days.clear();
    core_.month_slots.clear();
    std::vector<double> wu;   // the month's last water-use columns (routing.cpp:5021-5030)
    if (water_use(wu)) {
      const size_t N = (size_t)n;
      for (size_t i = 0; i < N; ++i) {
        additionalOutIn.additionalOutputInput((int)i, 3) = wu[6 * N + i];
        additionalOutIn.additionalOutputInput((int)i, 4) = wu[7 * N + i];
        additionalOutIn.additionalOutputInput((int)i, 50) = wu[10 * N + i];
        additionalOutIn.additionalOutputInput((int)i, 51) = wu[8 * N + i];
        additionalOutIn.additionalOutputInput((int)i, 52) = wu[9 * N + i];
        // G_unsatUseRiparian, which the outflow cell's hand-back writes on the
        // month's last day (routing.cpp:3121-3154); zero outside GLWD units
        additionalOutIn.additionalOutputInput((int)i, 42) = wu[12 * N + i];
      }
    }
    if (dwb_.month_end) {
      dwb_.month_end();
      dwb_.month_end = nullptr;
    }
  }

  DailyWaterBalanceGpu &dwb_;
  DropInCore &core_;
};

}  // namespace wg

#endif
