// The reference's day loop (integrate_wghm_, integrateWGHM.cpp:755-860) driven
// through the drop-in stand-ins of include/wg_gpu.hpp, with stand-ins for the
// reference's state-file classes that have their interfaces (wghmStateFile.h,
// additionalOutputInputFile.h, snowInElevationFile.h, calib_param.h:131).
//
//   dropin_loop <case dir> <years>
// reads region.bin (written by tests/test_gpu_dropin.py), forcing.bin (day-major
// float P, T, S of every year) and params.bin (the 26 x ncell parameters); runs
// the years; writes out.bin: the final state, every day's discharge of every
// cell, the last month's state-file cells and the additional-output and snow
// columns; prints the loop's wall time.
#include <omp.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <string>
#include <vector>

#include "wg_gpu.hpp"

struct Cell {   // wghmStateFile.h:38-47
  std::vector<double> c_, sn_, so_, ll_, lw_, gl_, gw_, rs_, ri_, g_;
  explicit Cell(size_t l = 31) : c_(l), sn_(l), so_(l), ll_(l), lw_(l), gl_(l), gw_(l), rs_(l), ri_(l), g_(l) {}
  double &canopy(int i) { return c_.at(i); }
  double &snow(int i) { return sn_.at(i); }
  double &soil(int i) { return so_.at(i); }
  double &locallake(int i) { return ll_.at(i); }
  double &localwetland(int i) { return lw_.at(i); }
  double &globallake(int i) { return gl_.at(i); }
  double &globalwetland(int i) { return gw_.at(i); }
  double &reservoir(int i) { return rs_.at(i); }
  double &river(int i) { return ri_.at(i); }
  double &groundwater(int i) { return g_.at(i); }
};
struct WghmStateFile {
  std::vector<Cell> cells;
  WghmStateFile(size_t n, size_t l) : cells(n, Cell(l)) {}
  Cell &cell(int i) { return cells.at(i); }
};
struct AdditionalOutputInputFile {
  int additionalfilestatus = 0;
  std::vector<std::vector<double>> v;
  explicit AdditionalOutputInputFile(size_t n) : v(n, std::vector<double>(53, 0.)) {}
  double &additionalOutputInput(int i, int j) { return v[i][j]; }
};
struct SnowInElevationFile {
  std::vector<std::vector<double>> v;
  explicit SnowInElevationFile(size_t n) : v(n, std::vector<double>(101, 0.)) {}
  double &snowInElevation(int i, int j) { return v[i][j]; }
};
enum eCalibParam { P_GAMRUN_C, P_CFA };
struct CalibParam {
  const double *param;
  int n;
  double getValue(eCalibParam k, int cell) { return param[(size_t)k * n + cell]; }
};

template <class T>
static std::vector<T> slurp(FILE *f, size_t count) {
  std::vector<T> v(count);
  if (count && fread(v.data(), sizeof(T), count, f) != count) {
    fprintf(stderr, "short read\n");
    exit(2);
  }
  return v;
}

static int run(int argc, char **argv);

int main(int argc, char **argv) {
  try {
    return run(argc, argv);
  } catch (const std::exception &e) {
    fprintf(stderr, "dropin_loop: %s\n", e.what());
    return 5;
  }
}

static int run(int argc, char **argv) {
  if (argc < 3) return 1;
  const std::string dir = argv[1];
  const int years = atoi(argv[2]);
  FILE *f = fopen((dir + "/region.bin").c_str(), "rb");
  if (!f) return 2;
  wg_region r{};
  int32_t hdr[4];
  if (fread(hdr, 4, 4, f) != 4 || fread(&r.default_velocity, 8, 1, f) != 1) return 2;
  r.ncell = hdr[0]; r.nband = hdr[1]; r.river_velo_opt = hdr[2]; r.frac_routing = hdr[3];
  // the pointer fields of wg_region, in declaration order: element size, count, bytes
  std::vector<std::vector<char>> keep;
  const void **ptr = reinterpret_cast<const void **>(&r.lct_albedo);
  const int nptr = (int)((reinterpret_cast<const char *>(&r.rout_order) - reinterpret_cast<const char *>(&r.lct_albedo)) /
                         sizeof(void *)) + 1;
  for (int k = 0; k < nptr; ++k) {
    int64_t bytes = 0;
    if (fread(&bytes, 8, 1, f) != 1) return 2;
    keep.push_back(slurp<char>(f, (size_t)bytes));
    ptr[k] = keep.back().data();
  }
  fclose(f);
  const int n = r.ncell;
  f = fopen((dir + "/forcing.bin").c_str(), "rb");
  if (!f) return 3;
  const size_t per = (size_t)365 * n;
  auto P = slurp<float>(f, per * years), T = slurp<float>(f, per * years), S = slurp<float>(f, per * years);
  fclose(f);

  wg_options o{};
  o.max_days = 365;
  o.members = 1;
  std::vector<int32_t> stations(n);
  for (int i = 0; i < n; ++i) stations[i] = i;
  o.nstation = n;
  o.stations = stations.data();
  wg::Context ctx(r, o);
  wg::DailyWaterBalanceGpu dailyWaterBalance(ctx, r);
  wg::RoutingGpu routing(dailyWaterBalance);
  WghmStateFile wghmState(n, 31);
  AdditionalOutputInputFile additionalOutIn(n);
  SnowInElevationFile snow_in_elevation(n), snow_state(n);
  CalibParam calParam{r.param, n};

  const short number_of_days_in_month[12] = {31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31};
  const short last_day_in_month[12] = {30, 58, 89, 119, 150, 180, 211, 242, 272, 303, 333, 364};
  std::vector<double> q((size_t)years * 365 * n);
  const auto t0 = std::chrono::steady_clock::now();
  for (int y = 0; y < years; ++y) {
    const short year = (short)(2000 + y);
    ctx.upload_forcing(0, 365, P.data() + y * per, T.data() + y * per, S.data() + y * per);
    short day = 0;
    for (short month = 0; month < 12; ++month) {
      for (short day_in_month = 1; day_in_month <= number_of_days_in_month[month]; ++day_in_month) {
        day++;
#pragma omp parallel for
        for (int cell = 0; cell < n; ++cell)
          dailyWaterBalance.calcNewDay(day, month, day_in_month, last_day_in_month[month], year, cell, wghmState,
                                       additionalOutIn, snow_in_elevation, 0, calParam);
        routing.routing(year, day, month, day_in_month, last_day_in_month[month], wghmState, additionalOutIn, 0,
                        calParam);
        routing.updateLandAreaFrac(additionalOutIn);
      }
      // the month end (integrateWGHM.cpp:830-847)
      for (int cell = 0; cell < n; ++cell) {
        const double landAreaFrac = routing.getLandAreaFrac(cell);
        const double cf = r.contfreq[cell];
        for (short elev = 0; elev <= 100; elev++)
          snow_state.snowInElevation(cell, elev) =
              landAreaFrac == 0. ? 0. : dailyWaterBalance.G_SnowInElevation(cell, elev) * landAreaFrac / cf;
        for (short dm = 1; dm <= number_of_days_in_month[month]; dm++) {
          wghmState.cell(cell).canopy(dm - 1) = dailyWaterBalance.G_canopyWaterContent[cell] * landAreaFrac / cf;
          wghmState.cell(cell).snow(dm - 1) = dailyWaterBalance.G_snow[cell] * landAreaFrac / cf;
          wghmState.cell(cell).soil(dm - 1) = dailyWaterBalance.G_soilWaterContent[cell] * landAreaFrac / cf;
        }
      }
    }
    ctx.discharge(0, 365, q.data() + y * per);
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

  // outputs: state (as wg_state_view fields), discharge, December's state-file
  // cells, the additional-output columns and both snow tables
  std::vector<double> st(24 * (size_t)n + (size_t)n * r.nband);
  std::vector<int32_t> ist(3 * (size_t)n);
  wg_state_view v{};
  double *sp = st.data();
  double **dfields[] = {&v.canopy, &v.soil, &v.snow, &v.lai_precsum, &v.gw, &v.river, &v.loclake, &v.locwetl,
                        &v.glolake, &v.glowetl, &v.res, &v.rf_loclake, &v.rf_locwetl, &v.rf_glolake, &v.rf_glowetl,
                        &v.rf_res, &v.k_release, &v.laf, &v.laf_prev, &v.fswb_next};
  for (auto *fp : dfields) { *fp = sp; sp += n; }
  v.snow_band = sp;
  v.lai_days = ist.data(); v.lai_status = ist.data() + n; v.laf_started = ist.data() + 2 * n;
  ctx.state(v);
  FILE *out = fopen((dir + "/out.bin").c_str(), "wb");
  fwrite(st.data(), 8, 20 * (size_t)n + (size_t)n * r.nband, out);
  fwrite(q.data(), 8, q.size(), out);
  for (int cell = 0; cell < n; ++cell) {
    Cell &c = wghmState.cell(cell);
    for (int d = 0; d < 31; ++d) {
      const double row[10] = {c.canopy(d), c.snow(d), c.soil(d), c.locallake(d), c.localwetland(d), c.globallake(d),
                              c.globalwetland(d), c.reservoir(d), c.river(d), c.groundwater(d)};
      fwrite(row, 8, 10, out);
    }
  }
  for (int cell = 0; cell < n; ++cell) fwrite(additionalOutIn.v[cell].data(), 8, 53, out);
  for (int cell = 0; cell < n; ++cell) fwrite(snow_in_elevation.v[cell].data(), 8, 101, out);
  for (int cell = 0; cell < n; ++cell) fwrite(snow_state.v[cell].data(), 8, 101, out);
  fclose(out);
  printf("%.6f %lld\n", secs, (long long)ctx.get() ? (long long)wg_launch_count(ctx.get()) : 0LL);
  return 0;
}
