// wg_volume.cuh -- water volume held by one state index (used by the balance kernels).
#pragma once
#include "wg_device.h"

namespace wg {

// Volume of the state at index i (slot s) [km3]: land storages (mm of the land
// fraction they were last rescaled to) plus groundwater and surface-water storages.
template <class R>
__device__ __forceinline__ double cell_volume(const DevCellsT<R> &c, const DevStateT<R> &st, size_t N, int s,
                                              size_t i) {
  double snow = 0.;
  for (int e = 0; e < c.nband; ++e) snow += (double)st.snow_band[(size_t)e * N + i];
  snow /= (double)c.nband;
  const double laf = st.laf_started[i] ? (double)st.laf_prev[i] : (double)st.laf[i];
  const double f = (double)c.area[s] * (laf / 100.) / 1000000.;
  return ((double)st.canopy[i] + snow + (double)st.soil[i]) * f + (double)st.gw[i] + (double)st.river[i] +
         (double)st.loclake[i] + (double)st.locwetl[i] + (double)st.glolake[i] + (double)st.glowetl[i] +
         (double)st.res[i];
}

}  // namespace wg
