// Compiles the C++ host side (include/wg_gpu.hpp) against the C ABI and links
// libwg_gpu.so; runs only calls that need no GPU.
#include <cstdio>
#include <cstring>

#include "wg_gpu.hpp"

struct FakeStateFile {};
struct FakeCalib {};

int main() {
  // status strings and argument checks work without a device
  if (std::strcmp(wg_status_string(WG_OK), "ok") != 0) return 1;
  if (wg_create(nullptr, nullptr, nullptr) != WG_ERR_INVALID) return 2;
  wg_region r{};
  wg_options o{};
  try {
    wg::Context c(r, o);   // ncell = 0 -> WG_ERR_INVALID before any device call
    return 3;
  } catch (const wg::Error &e) {
    if (e.status != WG_ERR_INVALID) return 4;
  }
  // the entry points without a context refuse before touching a device
  if (wg_run_steps(nullptr, 1, 0, 1, 0, 1) != WG_ERR_INVALID) return 5;
  if (wg_upload_longwave(nullptr, 0, 1, nullptr) != WG_ERR_INVALID) return 6;
  if (wg_get_water_temp(nullptr, nullptr, nullptr) != WG_ERR_INVALID) return 7;
  if (wg_get_river_temp(nullptr, 0, 1, nullptr) != WG_ERR_INVALID) return 8;
  if (wg_upload_water_use(nullptr, 0, 1, 1, nullptr, nullptr, nullptr, nullptr) != WG_ERR_INVALID) return 9;
  if (wg_get_water_use(nullptr, nullptr) != WG_ERR_INVALID) return 10;
  if (wg_set_water_use_inputs(nullptr, nullptr) != WG_ERR_INVALID) return 11;
  std::printf("ok\n");
  return 0;
}
