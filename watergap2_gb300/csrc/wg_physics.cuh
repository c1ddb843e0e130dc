// wg_physics.cuh -- per-cell physics of one day, as device functions.
//
// vertical_cell: dailyWaterBalanceClass::calcNewDay (source/daily.cpp:94-1257)
//                with laiClass::getDailyLai (source/lai.cpp:152-293);
// routing_cell:  one cell of routingClass::routing (source/routing.cpp:1835-4520)
//                with getRiverVelocity / getNewRiverVelocity (routing.cpp:7274-7341);
// fraction_update: the land-area-fraction update of routing.cpp:5034-5188 and
//                updateLandAreaFrac (routing.cpp:5343-5352).
//
// Templated on the arithmetic type R of state and fluxes: double for the plain
// FP64 path, float for the mixed-precision and ensemble paths (whose confluence
// sums and balance sums stay FP64; see wg_kernels.cu).  The control flow is the
// reference's, branch for branch.  To spend as few instructions as possible on
// GB300's slow FP64 pipe, divisions by per-cell constants are replaced by
// products with reciprocals prepared on the host, repeated divisors are inverted
// once, pow(T,4) is two squarings and exp/log/pow come from wg_fastmath.cuh; each
// of these changes a result by a few ulp at most, far inside the 1e-10 bound.
#pragma once
#include "wg_device.h"
#include "wg_fastmath.cuh"
#include "wg_wtemp.cuh"

namespace wg {

#define WG_MIN_STOR_VOL 1.e-15   // routingClass::minStorVol (routing.h:24)

__constant__ short c_first_day_in_month[12] = {1, 32, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335};

__device__ __forceinline__ int month_of(int doy) {
  int m = 0;
#pragma unroll
  for (int k = 1; k < 12; ++k) m += (doy >= c_first_day_in_month[k]) ? 1 : 0;
  return m;
}

template <class R> struct M;
template <> struct M<double> {
  static __device__ __forceinline__ double exp(double x) { return fm::exp(x); }
  static __device__ __forceinline__ double pow(double x, double y) { return fm::pow(x, y); }
  static __device__ __forceinline__ double rcp(double x) { return fm::rcp_pos(x); }   // x normal, nonzero
  static __device__ __forceinline__ double fabs_(double x) { return fabs(x); }
  // 1 - exp(-k) as the reference writes it (its rounding is the parity target)
  static __device__ __forceinline__ double one_m_exp_neg(double k, double e) { return 1. - e; }
};
template <> struct M<float> {
  static __device__ __forceinline__ float exp(float x) { return expf(x); }
  static __device__ __forceinline__ float pow(float x, float y) { return (x > 0.f) ? powf(x, y) : 0.f; }
  static __device__ __forceinline__ float rcp(float x) { return 1.0f / x; }
  static __device__ __forceinline__ float fabs_(float x) { return fabsf(x); }
  // 1 - exp(-k) without the cancellation of the subtraction: a slow river's
  // small k leaves 1 - expf(-k) with a relative error of 1e-7 / k in FP32
  static __device__ __forceinline__ float one_m_exp_neg(float k, float) { return -expm1f(-k); }
};

// Operations rounded once each and never contracted into an FMA (FP64), for the
// few expressions whose rounding the reference's storages integrate without
// feedback: a reservoir's release is not a function of its storage, so a
// rounding that differs from the reference's in the same direction every day
// (a folded constant like 1e9 / 86400, a product contracted with a sum) moves
// its storage a little further each day.  FP32: the plain operations.
template <class R> struct E;
template <> struct E<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};
template <> struct E<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
  static __device__ __forceinline__ float div(float a, float b) { return a / b; }
};

// Comparisons of the day step's hot loops.  On GB300 a double compare issues on
// the FP64 pipe (2 lanes per SM per clock) like an FMA; these give the same
// answers for every non-NaN operand from integer instructions on the bit
// patterns: x >= 0 orders like its bits as a signed integer, x < 0 like the
// negated magnitude (key below, which maps -0 and +0 to the same key), and a
// compare with a positive constant needs no key at all.  FP32 compares are
// cheap and stay as they are.
template <class R> struct C;
template <> struct C<double> {
  static __device__ __forceinline__ long long key(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : (long long)(0x8000000000000000ull - (unsigned long long)b);
  }
  static __device__ __forceinline__ bool gt(double a, double b) { return key(a) > key(b); }
  static __device__ __forceinline__ bool le(double a, double b) { return key(a) <= key(b); }
  static __device__ __forceinline__ bool lt(double a, double b) { return key(a) < key(b); }
  static __device__ __forceinline__ bool lt0(double a) { return key(a) < 0; }
  static __device__ __forceinline__ bool gt0(double a) { return __double_as_longlong(a) > 0; }
  static __device__ __forceinline__ bool le0(double a) { return __double_as_longlong(a) <= 0; }
  // a < c and a <= c for a constant c > 0
  static __device__ __forceinline__ bool lt_c(double a, double c) { return __double_as_longlong(a) < __double_as_longlong(c); }
  // a > c and |a| <= c for a constant c > 0
  static __device__ __forceinline__ bool gt_c(double a, double c) { return __double_as_longlong(a) > __double_as_longlong(c); }
  static __device__ __forceinline__ bool abs_le_c(double a, double c) {
    return (__double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFll) <= __double_as_longlong(c);
  }
  static __device__ __forceinline__ bool is_zero(double a) { return (__double_as_longlong(a) << 1) == 0; }
  static __device__ __forceinline__ bool is_one(double a) { return __double_as_longlong(a) == 0x3FF0000000000000ll; }
};
template <> struct C<float> {
  static __device__ __forceinline__ bool gt(float a, float b) { return a > b; }
  static __device__ __forceinline__ bool le(float a, float b) { return a <= b; }
  static __device__ __forceinline__ bool lt(float a, float b) { return a < b; }
  static __device__ __forceinline__ bool lt0(float a) { return a < 0.f; }
  static __device__ __forceinline__ bool gt0(float a) { return a > 0.f; }
  static __device__ __forceinline__ bool le0(float a) { return a <= 0.f; }
  static __device__ __forceinline__ bool lt_c(float a, float c) { return a < c; }
  static __device__ __forceinline__ bool gt_c(float a, float c) { return a > c; }
  static __device__ __forceinline__ bool abs_le_c(float a, float c) { return fabsf(a) <= c; }
  static __device__ __forceinline__ bool is_zero(float a) { return a == 0.f; }
  static __device__ __forceinline__ bool is_one(float a) { return a == 1.f; }
};

template <class R>
struct VOut {
  R rs, gwr, transfer, owp, owpet;
  R land_in, land_evap, land_leak;
};

// laiClass::dailyLai_growing (lai.cpp:179-241)
template <class R>
__device__ __forceinline__ R lai_growing(int &days, int init, int &status, bool evergreen, bool arid, R lmin, R lmax,
                                         R &psum, R prec) {
  const R inv30 = R(1.0 / 30.0);
  if (status == 0) {
    if (days >= init) {
      days++;
      psum += prec;
      if (C<R>::gt_c(psum, R(40.))) {
        if (days >= init + 30) { days = init + 30; status = 1; }
        return lmin + (lmax - lmin) * R(days - init) * inv30;
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
    if (days <= 0) { days = 0; status = 0; psum = R(0); }
    return lmax - (lmax - lmin) * R(30 - days) * inv30;
  }
  if (arid && C<R>::lt_c(prec, R(0.5))) days--;
  else days = 30 + init;
  return lmax;
}

// laiClass::dailyLai_nogrowing (lai.cpp:243-293)
template <class R>
__device__ __forceinline__ R lai_nogrowing(int &days, int init, int &status, R lmin, R lmax, R &psum, R prec) {
  const R inv30 = R(1.0 / 30.0);
  if (status == 0) {
    if (days > init) {
      days++;
      psum += prec;
      if (C<R>::gt_c(psum, R(40.))) {
        if (days >= init + 30) { days = init + 30; status = 1; }
        return lmin + (lmax - lmin) * R(days - init) * inv30;
      }
      days = init;
      return lmin;
    }
    psum += prec;
    return lmin;
  }
  if (days <= 30) {
    days--;
    if (days <= 0) { days = 0; status = 0; psum = R(0); }
    return lmax - (lmax - lmin) * R(30 - days) * inv30;
  }
  days--;
  return lmax;
}

// Where one cell-day's output terms go (FP64): the sums of the day's month, field
// k at mo[k * mos] (DevMonthly::vert; null: none), the day's values, field k at
// dd[k * dds] (DevMonthly::dvert; null: none), and the cell's constants for Kc and
// total PET, field k at vk[k * vks] (DevMonthly::vconst).
struct VSink {
  double *mo;
  size_t mos;
  double *dd;
  size_t dds;
  const double *vk;
  size_t vks;
};

// dailyWaterBalanceClass::calcNewDay for one cell (daily.cpp:94-1257).
//   c, s        : per-cell constants and the cell's slot
//   gamma_soil  : runoff exponent (P_GAMRUN_C, times a member's factor in an ensemble)
//   canopy ...  : the cell's state, read and written through references
//   band        : the cell's snow bands, band[e * bstride]
//   Pin         : precipitation (times a member's factor in an ensemble)
//   OUT, vs     : the output grids (monthly and daily) of the cell-day
template <class R, bool OUT = false>
__device__ __forceinline__ void vertical_cell(const DevCellsT<R> &c, int s, R gamma_soil, R &canopy, R &soil,
                                              R &gsnow, R *band, size_t bstride, int &days, int &status, R &psum,
                                              R landAreaFrac, R prevLAF, R Pin, float Tf, float SWf, R ext_rad,
                                              R inv_s0, VOut<R> &o, const VSink *vs = nullptr) {
  typedef M<R> m;
  const int B = c.nband;
  const R invB = c.invB;
  const uint32_t flags = c.flags[s];
  const bool arid = (flags & F_ARID) != 0;
  R transfer = R(0);
  const R cfa = c.cfa[s];
  R dailyPrec = c.mprec[s] * Pin;                                 // daily.cpp:248
  const R T = R(Tf);
  const R temp2 = T + R(237.3);
  const R inv_t2 = m::rcp(temp2);
  const R e_s = R(0.6108) * m::exp(R(17.27) * T * inv_t2);
  const R alpha = c.alpha[s], maxDailyPET = c.pet_mxdy[s];
  const R a_c = arid ? R(1.35) : R(1.00), b_c = arid ? R(-0.35) : R(0.00);

  // LAI state machine (lai.cpp:152-177); the temperature tests use the float input
  R dailyLai;
  if (Tf > 8.f)
    dailyLai = lai_growing<R>(days, c.init_days[s], status, (flags & F_EVERGREEN) != 0, arid, c.lai_min[s], c.lai_max[s],
                              psum, dailyPrec);
  else
    dailyLai = lai_nogrowing<R>(days, c.init_days[s], status, c.lai_min[s], c.lai_max[s], psum, dailyPrec);

  typedef C<R> cmp;
  const R albedo = cmp::gt_c(gsnow, R(3.)) ? c.albedo_snow[s] : c.albedo[s];                 // daily.cpp:366-379
  const R lat_heat = (Tf > 0.f) ? R(2.501) - R(0.002361) * T : R(2.835);      // daily.cpp:382-387
  const R rlh = m::rcp(lat_heat);
  const R solar_rad = R(0.0864) * rlh * R(SWf);
  R solar_fraction = (ext_rad == R(0)) ? R(0) : solar_rad * inv_s0;          // daily.cpp:430-448
  if (cmp::gt_c(solar_fraction, R(1.))) solar_fraction = R(1.);
  const R ff = a_c * solar_fraction + b_c;
  const R net_emissivity = R(-0.02) + R(0.261) * m::exp(R(-0.000777) * T * T);
  const R tK = T + R(273.2);
  const R tK2 = tK * tK;
  const R net_lw = (-ff * net_emissivity * R(0.000000004903) * (tK2 * tK2)) * rlh;
  const R net_rad = c.mnetrad[s] * (solar_rad * (R(1.) - albedo) + net_lw);
  const R ow_net_rad = solar_rad * R(1. - 0.08) + net_lw;
  const R inc_svp = R(4098.) * e_s * (inv_t2 * inv_t2);                     // daily.cpp:484-532
  const R gamma = R(0.0016286 * 101.3) * rlh;
  const R apet = alpha * inc_svp * m::rcp(inc_svp + gamma);
  const R dailyPET = cmp::le0(net_rad) ? R(0) : apet * net_rad;
  const R owPET = cmp::le0(ow_net_rad) ? R(0) : apet * ow_net_rad;
  o.owp = dailyPrec;
  o.owpet = owPET;
  // the output grids: the monthly sums (daily.cpp:1281-1386, grid_store 2) and the
  // day's values (daily.cpp:1388-1399, 1472-1540, grid_store 5/6), each term filed
  // as soon as it is known so that none stays live to the end of the cell-day.
  // Radiation in W/m2 (lat_heat / 0.0864 per mm/day); the land terms weighted by
  // the day's land share of the continental area; the storages at the day's (the
  // month's) end.  Only continental cells run this (cells without continental
  // area run no vertical balance).  The reference divides each land term by
  // contfreq; here one refined reciprocal of contfreq per cell-day and products
  // with constants give the same values to a few ulp (a correctly rounded FP64
  // division costs about ten FP64-pipe operations, and the FP64 pipe bounds the
  // step).
  [[maybe_unused]] double mw = 0.;       // landAreaFrac / contfreq
  if constexpr (OUT) {
    if (vs) {
      const double conv = (double)lat_heat * (1.0 / 0.0864);
      const double ns = (double)solar_rad * (1. - (double)albedo);
      const double cf = (double)c.contfreq[s], rcf = fm::rcp_pos(cf);
      const double lf = (double)landAreaFrac, lf100 = lf * 0.01;
      mw = lf * rcf;
      // total PET over land and fresh water (daily.cpp:1303, 1484)
      const double fw = vs->vk[3 * vs->vks];
      const double tpet = ((cf - fw) * (double)dailyPET + fw * (double)owPET) * rcf;
      const double alb = (double)albedo * lf100 + 0.08 * (1. - lf100);
      if (double *m = vs->mo) {
        const size_t k = vs->mos;
        m[0] += (double)dailyPrec;
        m[k] += (double)T;
        m[2 * k] += (double)ext_rad * conv;
        m[3 * k] += ((double)solar_rad - ns) * conv;
        m[4 * k] += (double)solar_rad * conv;
        m[5 * k] += ns * conv;
        m[6 * k] += (double)net_lw * conv;
        m[7 * k] += (double)net_rad * conv;
        m[8 * k] += (double)owPET;
        m[9 * k] += (double)dailyPET;
        m[13 * k] += (double)dailyLai;
        m[14 * k] += alb;
        m[32 * k] += tpet;
      }
      if (double *dd = vs->dd) {
        const size_t k = vs->dds;
        const double *vk = vs->vk;
        dd[0] = (double)dailyPrec;
        dd[k] = (double)T;
        dd[2 * k] = (double)dailyPET;
        dd[3 * k] = tpet;
        dd[4 * k] = (double)dailyLai;
        dd[5 * k] = vk[0] + vk[vs->vks] * ((double)dailyLai - vk[2 * vs->vks]);   // lai.cpp:295-306
        dd[6 * k] = alb;
        dd[17 * k] = (double)ext_rad * conv;
        dd[18 * k] = (double)solar_rad * conv;
        dd[19 * k] = ((double)solar_rad - ns) * conv;
        dd[20 * k] = ns * conv;
        dd[21 * k] = (double)net_lw * conv;
        dd[22 * k] = (double)net_rad * conv;
      }
    }
  }

  R lsc = R(0), initialStorage = R(0);
  R canopyEvapo = R(0), prec_to_soil = R(0), soilPET = R(0), snowEvapo = R(0), effPrec = R(0);
  R immediate = R(0), dailyAET = R(0), runoff = R(0), total = R(0), gwr = R(0), pot = R(0);
  R overflow = R(0), neg_land_aet = R(0), cellAET = R(0), gwr_route = R(0), leak = R(0);
  const bool land = cmp::gt0(landAreaFrac);
  // prevLAF / landAreaFrac; exactly 1 while the land fraction does not change, and
  // then the storages are not rescaled (x * 1 = x)
  const R ratio = !land ? R(0) : (prevLAF == landAreaFrac ? R(1) : prevLAF / landAreaFrac);
  const bool rescale = !cmp::is_one(ratio);

  // interception (daily.cpp:825-895)
  [[maybe_unused]] R out_maxcs = R(0);   // max_canopy_storage, 0 without leaves (daily.cpp:789, 847)
  if (!land) {
    transfer = canopy;
    canopy = R(0);
  } else {
    if (rescale) canopy *= ratio;
    if (cmp::abs_le_c(canopy, R(WG_MIN_STOR_VOL))) canopy = R(0);
    initialStorage = canopy;
    if (cmp::gt_c(dailyLai, R(0.00001))) {
      const R maxcs = c.mcwh[s] * dailyLai;
      if constexpr (OUT) out_maxcs = maxcs;
      const R deficiency = maxcs - canopy;
      if (cmp::lt(dailyPrec, deficiency)) {
        canopy += dailyPrec;
        prec_to_soil = R(0);
      } else {
        canopy = maxcs;
        prec_to_soil = dailyPrec - deficiency;
      }
      const R cwc = canopy;
      canopyEvapo = dailyPET * m::pow(cwc * m::rcp(maxcs), R(0.66666666));   // maxcs > 1e-5 mcwh
      if (cmp::gt(canopyEvapo, cwc)) {
        canopyEvapo = cwc;
        soilPET = dailyPET - cwc;
        canopy = R(0);
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
  if (cmp::lt0(soilPET)) soilPET = R(0);
  if constexpr (OUT) {
    if (vs) {   // the canopy's terms: its state does not change after this
      const double ic = (double)canopyEvapo * mw, cw = (double)canopy * mw, mx = (double)out_maxcs * mw;
      if (double *m = vs->mo) {
        m[15 * vs->mos] += ic;
        m[16 * vs->mos] += cw;
        m[17 * vs->mos] += mx;
      }
      if (double *dd = vs->dd) {
        dd[7 * vs->dds] = ic;
        dd[8 * vs->dds] = cw;
        dd[9 * vs->dds] = mx;
      }
    }
  }

  // snow in elevation bands (daily.cpp:897-1062).  Whether a band gets snowfall
  // (temp_elev <= P_T_SNOWFZ, daily.cpp:982) decides where the day's precipitation
  // goes; the FP32 paths take that decision as the FP64 path does, from the float
  // temperature and a per-band float threshold prepared on the host, so that FP32
  // rounding of temp_elev never moves a band's precipitation between snow and rain.
  constexpr bool fp32 = sizeof(R) == 4;
  R snowChange = R(0), gs = R(0);
  // the monthly outputs' band sums (daily.cpp:983, 998, 1032-1041): the bands with
  // snowfall and with rain (each adds the day's precipitation above the canopy;
  // counted on the integer pipe and multiplied once), melt, snow-covered bands
  [[maybe_unused]] int n_snowfall = 0, n_rainfall = 0, n_cover = 0;
  [[maybe_unused]] R out_melt = R(0);
  bool above0 = cmp::gt(R(0), c.t_snowfz[s]);   // band 0 above freezing: the soil runs (daily.cpp:1076)
  int thresh = 0;
  const R t_snowfz = c.t_snowfz[s], t_snowmt = c.t_snowmt[s], ddf_m = c.ddf_m[s];
  for (int e = 0; e < B; ++e) {
    R sb = band[e * bstride];
    R temp_elev = T - c.band_dt[(size_t)e * c.n + s];
    bool snowfall = fp32 ? Tf <= c.snow_thr[(size_t)e * c.n + s] : cmp::le(temp_elev, t_snowfz);
    if (land && cmp::is_zero(sb) && !snowfall) {
      // no snow and no snowfall in this band: the steps below would keep it at
      // zero, melt nothing and pass the precipitation on -- the same bits, without
      // the band's arithmetic and store
      if (e == 0) above0 = true;
      effPrec += prec_to_soil;
      if constexpr (OUT) ++n_rainfall;
      continue;
    }
    if (!land) {
      transfer += sb * invB;
      sb = R(0);
      gs = R(0);
    } else {
      R effBefore, melt = R(0);
      if (rescale) sb *= ratio;
      if (cmp::abs_le_c(sb, R(WG_MIN_STOR_VOL))) sb = R(0);
      initialStorage = sb;
      if (cmp::gt_c(sb, R(1000.))) {
        if (thresh == 0) {
          thresh = c.band_el[(size_t)e * c.n + s];
        } else if (thresh > 0) {
          // the remembered threshold elevation's temperature, rounded as the reference
          // rounds it (no contraction into an FMA); the FP32 paths decide in FP64
          temp_elev = T - (R(thresh) - c.elev0[s]) * c.t_gradnt[s];
          if constexpr (fp32) {
            const double te = __dsub_rn((double)Tf, __dmul_rn((double)thresh - (double)c.elev0[s], c.thr64[s]));
            snowfall = te <= c.thr64[(size_t)c.n + s];
          } else {
            temp_elev = __dsub_rn(T, __dmul_rn(R(thresh) - c.elev0[s], c.t_gradnt[s]));
            snowfall = cmp::le(temp_elev, t_snowfz);
          }
        }
      }
      if (snowfall) {
        effBefore = R(0);
        sb += prec_to_soil;
        if (cmp::gt(sb, soilPET)) {
          sb -= soilPET;
          snowEvapo += soilPET;
        } else {
          snowEvapo += sb;
          sb = R(0);
        }
      } else {
        effBefore = prec_to_soil;
      }
      if (cmp::gt(temp_elev, t_snowmt) && !cmp::lt0(sb)) {
        melt = ddf_m * (temp_elev - t_snowmt);
        if (cmp::gt(melt, sb)) {
          melt = sb;
          sb = R(0);
        } else {
          sb -= melt;
        }
      }
      snowChange += sb - initialStorage;
      if (e == 0) above0 = !snowfall;
      gs += sb;
      effPrec += effBefore + melt;
      if constexpr (OUT) {
        if (snowfall) ++n_snowfall;
        else ++n_rainfall;
        out_melt += melt;
        if (cmp::gt0(sb)) ++n_cover;
      }
    }
    band[e * bstride] = sb;
  }
  if (land) {
    gs *= invB;
    effPrec *= invB;
    snowEvapo *= invB;
    snowChange *= invB;
    lsc += snowChange;
  }
  gsnow = gs;
  if constexpr (OUT) {
    if (vs) {   // the snow's terms
      // per band of the cell's land (1 / bands), without land the sums are 0
      const double pb = (double)dailyPrec * (double)invB * mw, bw = (double)invB * mw;
      const double sf = (double)n_snowfall * pb, sm = (double)out_melt * bw, swe = (double)gsnow * mw;
      const double cov = (double)n_cover * bw;
      if (double *m = vs->mo) {
        const size_t k = vs->mos;
        m[18 * k] += sf;
        m[19 * k] += (double)n_rainfall * pb;
        m[20 * k] += sm;
        m[21 * k] += (double)snowEvapo * mw;
        m[22 * k] += swe;
        m[23 * k] += cov;
      }
      if (double *dd = vs->dd) {
        const size_t k = vs->dds;
        dd[10 * k] = sf;
        dd[11 * k] = sm;
        dd[12 * k] = swe;
        dd[13 * k] = cov;
      }
    }
  }

  // immediate runoff from built-up area (daily.cpp:1068-1071)
  if (cmp::gt0(c.built_up[s])) {
    immediate = R(0.5) * effPrec * c.built_up[s];
    effPrec -= immediate;
  }

  // soil, AET, runoff, groundwater recharge (daily.cpp:1080-1239)
  if (!land) {
    transfer += soil;
    transfer *= cfa;
    soil = R(0);
  } else {
    const R Smax = c.smax[s];
    if (rescale) soil *= ratio;
    initialStorage = soil;
    if (cmp::gt(soil, Smax)) {
      overflow = soil - Smax;
      soil = Smax;
    }
    if (above0) {
      if (cmp::gt0(Smax)) {
        const R sat = soil * c.inv_smax[s];
        runoff = effPrec * m::pow(sat, gamma_soil);
        const R lim = (maxDailyPET - canopyEvapo) * sat;
        dailyAET = cmp::gt(soilPET, lim) ? lim : soilPET;
        soil += effPrec - dailyAET - runoff;
        if (cmp::abs_le_c(soil, R(WG_MIN_STOR_VOL))) soil = R(0);
        effPrec = R(0);
        if (cmp::lt0(soil)) {
          dailyAET += soil;
          soil = R(0);
        }
        runoff *= cfa;
        immediate *= cfa;
        const R fgr = c.fg[s] * runoff;
        gwr = cmp::lt(c.rgmax[s], fgr) ? c.rgmax[s] : fgr;
        // the reference's inland-sink test here reads a grid nothing fills (globals.cpp:8),
        // so the arid rule applies by aridity and texture alone
        if ((flags & F_ARID_GW) && cmp::le(dailyPrec, c.pcritgwa[s])) {
          pot = gwr;
          gwr = R(0);
        }
        runoff -= pot;
        soil += pot * c.inv_cfa[s];
        if (cmp::gt(soil, Smax)) {
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
      dailyAET = R(0);
      leak -= cfa * immediate;   // built-up runoff is dropped in this branch
    }
    gwr_route = gwr;   // G_dailyGwRecharge (daily.cpp:1232)
    lsc += soil - initialStorage;
    cellAET = (lsc - dailyPrec) * (cfa - R(1.0)) + (dailyAET + canopyEvapo + snowEvapo) * cfa;
    if (cmp::lt0(cellAET)) {
      neg_land_aet = cellAET;
      cellAET = R(0);
    }
  }
  // surface runoff (daily.cpp:1244-1257)
  if (cmp::lt0(neg_land_aet)) total = total + neg_land_aet;
  if (cmp::lt0(total)) {
    leak -= total;
    total = R(0);
  }
  if (cmp::lt0(total - gwr)) {
    soil += total - gwr;
    gwr = total;
  }
  o.rs = total - gwr;
  o.gwr = gwr_route;
  o.transfer = transfer;
  o.land_in = dailyPrec;
  o.land_evap = cellAET;
  o.land_leak = leak;
  if constexpr (OUT) {
    if (vs) {   // the soil's terms and the storages at the day's end
      const double sw = (double)soil * mw, sr = ((double)total - (double)gwr) * mw, gr = (double)gwr * mw;
      const double a = (double)c.area[s] * (double)landAreaFrac * 1e-8;   // area [km2] / 1e6 * landAreaFrac / 100
      const double cs = (double)canopy * a, ss = (double)gsnow * a, ls = (double)soil * a;
      if (double *m = vs->mo) {
        const size_t k = vs->mos;
        m[10 * k] += (double)dailyAET * mw;
        m[11 * k] += (double)cellAET * mw;
        m[12 * k] += ((double)dailyAET + (double)canopyEvapo + (double)snowEvapo) * mw;
        m[24 * k] += sw;
        m[25 * k] += (double)total * mw;
        m[26 * k] += (double)immediate;
        m[27 * k] += sr;
        m[28 * k] += gr;
        m[29 * k] = cs;
        m[30 * k] = ss;
        m[31 * k] = ls;
      }
      if (double *dd = vs->dd) {
        const size_t k = vs->dds;
        dd[14 * k] = sw;
        dd[15 * k] = sr;
        dd[16 * k] = gr;
        dd[23 * k] = cs;
        dd[24 * k] = ss;
        dd[25 * k] = ls;
        dd[26 * k] = (double)cellAET * mw;   // the land part of routing's cell AET
      }
    }
  }
}

// Routing terms of one cell-day for the output grids (routing.cpp:3964-4238,
// 4525-4660): the open-water evaporation of the cell's water bodies [km3] (the
// reference's dailyOpenWaterEvap_km3 without the inland sink's transported
// volume: each body's evaporation in mm, reduced where the storage limits it,
// times its area), the groundwater runoff [km3], the wetlands' extents [km2], the
// reservoir's inflow and outflow [km3] and the precipitation on the global lake
// and the reservoir [km3].
struct RoutOut {
  double owe, gw_runoff, lw_ext, gw_ext, res_in, res_out, p_lake;
  double actual_use, nug;   // water use: the day's actual use from surface water, NUg [km3]
};

template <class R>
struct RTerms {
  R p_ow, e_ow, leak;
  R velocity;   // river flow velocity of the day [km/d]
};

// Routing state of one cell (surface water and groundwater storages).
template <class R>
struct RState {
  R gw, river, loclake, locwetl, glolake, glowetl, res;
  R rf_loclake, rf_locwetl, rf_glolake, rf_glowetl, rf_res, k_release;
};

// getRiverVelocity / getNewRiverVelocity (routing.cpp:7274-7341)
template <class R>
__device__ __forceinline__ R river_velocity(const DevCellsT<R> &c, int s, R riverInflow, R S) {
  typedef M<R> m;
  const R bw = c.bw[s];
  R depth, csa;
  if (c.velo_opt == 1) {
    const R Q = riverInflow * R(1.0e9 / 86400.);
    depth = R(0.349) * m::pow(Q, R(0.341));
    csa = depth * (R(2.0) * depth + bw);
  } else {
    csa = (S * c.inv_len[s]) * R(1000000.);
    depth = -bw * R(0.25) + sqrt(bw * bw * R(1.0 / 16.0) + R(0.5) * csa);
  }
  const R wp = bw + R(2.0 * 2.23606797749979) * depth;   // 2 sqrt(5)
  const R hr = csa * m::rcp(wp);
  const R v = c.inv_mr[s] * m::pow(hr, R(2. / 3.)) * c.sqrt_slope[s] * R(86.4);
  return (v < R(0.00001)) ? R(0.00001) : v;
}

// routingClass::updateNetAbstractionGW (routing.cpp:5503-5572): the day's net
// abstraction from groundwater after the previous day's unsatisfied surface-water
// demand w[0] -- return flows of irrigation from surface water are reduced (or
// given back) in the proportion that reaches groundwater.  w: the cell's
// water-use state, row stride N.
__device__ __forceinline__ double wu_update_nag(double *w, size_t N, double nug, double frgi) {
  const double rem = w[0];
  double ui = w[1 * N], uo = w[2 * N], rrf = w[3 * N];
  const double wdr = w[4 * N], cons = w[5 * N];
  double out = nug;
  if (rem > 1.e-12) {
    if (wdr > 0.) {
      const double eff = cons / wdr;
      const double factor = 1. - (1. - frgi) * (1. - eff);
      double wnew = 1. / factor * (wdr * factor - rem);
      if (wnew < 0.) {
        wnew = 0.;
        ui += wdr * factor;
        uo += rem - (wdr * factor);
      } else {
        ui += rem;
      }
      const double change = frgi * (1. - eff) * (wnew - wdr);
      rrf += change;
      w[0] = 0.;
      out = nug - change;
    } else {
      uo += rem;
    }
  } else if (rem < -1.e-12) {
    double from_irrig = rem + uo;
    if (from_irrig >= 0.) {
      uo += rem;
      w[0] = 0.;
    } else {
      uo = 0.;
      w[0] = 0.;
      if (ui != 0.) {
        double ratio = from_irrig / ui;
        if (ratio < -1.) {
          ratio = -1.;
          from_irrig = ui * -1.;
        }
        const double change = ratio * rrf;
        ui += from_irrig;
        rrf += change;
        out = nug - change;
      }
    }
  }
  w[1 * N] = ui; w[2 * N] = uo; w[3 * N] = rrf;
  return out;
}

// End of a year for the cell's water-use state (annualWaterUsePostProcessing,
// routing.cpp:5256-5296).
__device__ __forceinline__ void wu_year_end(double *w, size_t N) {
  double tot = w[6 * N], ui = w[1 * N], uo = w[2 * N], rrf = w[3 * N];
  const double prev = w[7 * N];
  if (tot < prev) {
    w[7 * N] = tot; w[8 * N] = ui; w[9 * N] = uo; w[10 * N] = rrf;
    ui = 0.; uo = 0.; rrf = 0.; tot = 0.;
  } else {
    tot -= prev; ui -= w[8 * N]; uo -= w[9 * N]; rrf -= w[10 * N];
    if ((ui + uo) < 0.) {
      ui = 0.; uo = 0.; rrf = 0.;
    } else if (uo < 0.) {
      ui += uo; uo = 0.;
    } else if (ui < 0.) {
      uo += ui; ui = 0.; rrf = 0.;
    }
    if (rrf > 0.) { rrf = 0.; ui = 0.; }
  }
  w[6 * N] = tot; w[1 * N] = ui; w[2 * N] = uo; w[3 * N] = rrf;
}

// One cell of routingClass::routing (routing.cpp:1835-4520) given the vertical
// outputs and the summed upstream inflow (FP64 for every precision); returns the
// transported volume.  WT (FP64): the water temperature of each water body runs
// through wtd as soon as the body's routing is done (the reference reads the
// same terms after the cell's routing, routing.cpp:4287-4356: each body's
// storage before the day, its evaporation after any reduction, its reduction
// factor and outflow, and the local runoff).  WU: water use (subtract_use = 2, satisfied in the cell):
// wu points at the tables (per cell: slot s, stride c.n) and the state (per
// member: state index si, stride NN), wrow is the offset of the day's table row.
// RO: the terms of routing's output grids into *ro.
template <class R, bool WT = false, bool WU = false, bool GL = false, bool RO = false>
__device__ __forceinline__ R routing_cell(const DevCellsT<R> &c, int s, RState<R> &st, int doy, int month, R laf,
                                          R laf_prev, const VOut<R> &v, double inflow_up, RTerms<R> &rt,
                                          wt::WtDay *wtd = nullptr, const DevWaterUse *wu = nullptr, size_t wrow = 0,
                                          size_t si = 0, size_t NN = 0, RoutOut *ro = nullptr) {
  typedef M<R> m;
  const uint32_t fl = c.flags[s];
  const R cfa = c.cfa[s];
  rt.p_ow = R(0); rt.e_ow = R(0); rt.leak = R(0);
  if constexpr (RO) *ro = RoutOut{};
  R remainingUse = R(0), dailyActualUse = R(0), remUseGL = R(0), remUseRes = R(0);
  double prevTotalUnsat = 0.;
  double *W = nullptr;
  if constexpr (WU) {
    W = wu->st + si;
    if (doy == 1) {   // annualInit (routing.cpp:994-1010)
      W[7 * NN] = W[6 * NN]; W[8 * NN] = W[1 * NN]; W[9 * NN] = W[2 * NN]; W[10 * NN] = W[3 * NN];
      W[11 * NN] = 0.;
    }
  }
  const R f_land = c.area_f[s] * laf;
  typedef C<R> cmp;
  R dlsr = cmp::le0(laf) ? v.transfer * c.area_f[s] * laf_prev : v.rs * f_land;
  // groundwater (routing.cpp:2061-2200)
  const R gw0 = st.gw;
  R netGWin = v.gwr * f_land;
  if constexpr (WU) {   // routing.cpp:1926-1933 (and the other groundwater variants)
    const size_t tn = (size_t)c.n;
    double nug = wu->tab[wrow + tn + s];
    if (W[0] != 0.) nug = wu_update_nag(W, NN, nug, wu->frgi[s]);
    if constexpr (RO) ro->nug = nug;   // G_dailydailyNUg (routing.cpp:3747)
    netGWin -= R(nug);
    rt.e_ow += R(nug);
    remainingUse = R(wu->tab[wrow + s]);   // routing.cpp:2225-2290
    if constexpr (GL) {   // routing.cpp:2199-2222: NUs aggregated over the GLWD unit
      const double agg = wu->tab[wrow + 5 * tn + s];
      if (fl & (F_GLOLAKE | F_RES)) remainingUse = R(agg);                  // the unit's outflow cell
      else if (wu->unit_of[s] != -1) remainingUse = R(agg + W[12 * NN]);   // a riparian cell
    }
    if (wu->delayed) {   // routing.cpp:2236-2244
      prevTotalUnsat = W[6 * NN];
      remainingUse = R((double)remainingUse + prevTotalUnsat);
      W[6 * NN] = 0.;
    }
  }
  [[maybe_unused]] const R totalDesiredUse = remainingUse;
  R gw = gw0 * c.gw_e[s] + c.gw_ik[s] * netGWin * c.gw_ome[s];
  if (cmp::abs_le_c(gw, R(WG_MIN_STOR_VOL))) gw = R(0);
  R gw_runoff = gw0 - gw + netGWin;
  if (cmp::le0(gw_runoff)) {
    gw_runoff = R(0);
    gw = gw0 + netGWin;
    if (cmp::abs_le_c(gw, R(WG_MIN_STOR_VOL))) gw = R(0);
  }
  st.gw = gw;
  if constexpr (RO) ro->gw_runoff = (double)gw_runoff;
  R inflow = dlsr + gw_runoff;
  R into_river = R(0), gw_into_river = R(0), local_gw = gw_runoff;
  if (c.frac_routing && !(fl & F_SINK)) {
    // fractional routing (routing.cpp:1897-1907, 1911-1915, 2024-2033): the runoff
    // from outside the water bodies' catchment flows directly into the river; arid
    // cells send all their groundwater runoff there
    const R fc = c.fcatch[s];
    into_river = (R(1.) - fc) * dlsr;
    if (fl & F_ARID) {
      local_gw = R(0);
      inflow = fc * dlsr;
      gw_into_river = gw_runoff;
    } else {
      gw_into_river = (R(1.) - fc) * gw_runoff;
      local_gw = fc * gw_runoff;
      inflow = (fc * dlsr) + local_gw;
    }
  }
  if constexpr (WT) wtd->runoff(inflow, local_gw, into_river, gw_into_river);
  const R owp = v.owp, owpet = v.owpet;
  R outflow = R(0);
  const R a6 = c.a6[s];

  if (fl & F_LOCLAKE) {  // local lake (routing.cpp:2318-2490)
    const R S0 = st.loclake, maxS = c.maxs_ll[s], rf = st.rf_loclake;
    R evapo = (R(1.0) - cfa) * owp * rf + cfa * owpet * rf;
    if (evapo < R(0)) evapo = R(0);
    const R pin = owp * rf * a6 * c.ll100[s];
    const R TI = inflow + pin;
    const R PETgwr = evapo * a6 * c.ll100[s];
    R PETgwrMax = S0 + maxS + TI;
    const R avail = PETgwrMax;
    if (PETgwrMax < R(0)) PETgwrMax = R(0);
    R S;
    if (PETgwr > PETgwrMax) {
      S = -maxS;
      rt.e_ow += avail;
      if constexpr (WT || RO) evapo *= PETgwrMax / PETgwr;   // routing.cpp:2400-2404
    } else {
      S = S0 + TI - PETgwr;
      rt.e_ow += PETgwr;
    }
    rt.p_ow += pin;
    if (S0 > R(0)) {
      outflow = c.sw_k[s] * S0 * m::pow(S0 * c.inv_maxs_ll[s], R(1.5));
      if (S <= R(0)) outflow = R(0);
      else if (outflow > S) outflow = S;
    } else outflow = R(0);
    S -= outflow;
    if (m::fabs_(S) <= R(WG_MIN_STOR_VOL)) S = R(0);
    if (S > maxS) {
      outflow += S - maxS;
      S = maxS;
    }
    inflow = outflow;
    if constexpr (WT) wtd->loclake((double)S0 + (double)maxS, evapo, rf, outflow);
    if constexpr (RO) ro->owe += (double)evapo * (double)a6 * (double)c.ll100[s];
    R r = R(1.) - m::pow(m::fabs_(S - maxS) * (R(0.5) * c.inv_maxs_ll[s]), c.evx[s]);
    st.loclake = S;
    st.rf_loclake = r < R(0) ? R(0) : (r > R(1) ? R(1) : r);
  }
  if (fl & F_LOCWETL) {  // local wetland (routing.cpp:2495-2617)
    const R S0 = st.locwetl, maxS = c.maxs_lw[s], rf = st.rf_locwetl;
    R evapo = (R(1.0) - cfa) * owp * rf + cfa * owpet * rf;
    if (evapo < R(0)) evapo = R(0);
    const R pin = owp * rf * a6 * c.lw100[s];
    const R TI = inflow + pin;
    const R PETgwr = evapo * a6 * c.lw100[s];
    const R PETgwrMax = S0 + TI;
    R S;
    if (PETgwr > PETgwrMax) {
      S = R(0);
      rt.e_ow += PETgwrMax;
      if constexpr (WT || RO) evapo *= PETgwrMax / PETgwr;
    } else {
      S = S0 + TI - PETgwr;
      rt.e_ow += PETgwr;
    }
    rt.p_ow += pin;
    if (m::fabs_(S) <= R(WG_MIN_STOR_VOL)) S = R(0);
    if (S > R(0)) {
      outflow = c.sw_k[s] * S * m::pow(S * c.inv_maxs_lw[s], R(2.5));
      if (outflow > S) outflow = S;
    } else outflow = R(0);
    S -= outflow;
    if (S > maxS) {
      outflow += S - maxS;
      S = maxS;
    }
    inflow = outflow;
    if constexpr (WT) wtd->locwetl(S0, evapo, rf, outflow);
    if constexpr (RO) {   // routing.cpp:2509-2524
      ro->owe += (double)evapo * (double)a6 * (double)c.lw100[s];
      ro->lw_ext = (double)rf * (double)c.area[s] * (double)c.lw100[s];
    }
    R r = R(1.) - m::pow(m::fabs_(S - maxS) * c.inv_maxs_lw[s], c.evx[s]);
    st.locwetl = S;
    st.rf_locwetl = r < R(0) ? R(0) : (r > R(1) ? R(1) : r);
  }
  inflow = R((double)inflow + inflow_up);   // routing.cpp:2623-2624
  if constexpr (WT) wtd->locals_done();
  if (fl & F_GLOLAKE) {  // global lake (routing.cpp:2630-2804)
    const R S0 = st.glolake, maxS = c.maxs_gl[s], rf = st.rf_glolake;
    R evapo = (R(1.0) - cfa) * owp + cfa * owpet * rf;
    if (evapo < R(0)) evapo = R(0);
    const R pin = owp * c.la6[s];
    const R TI = inflow + pin;
    R PU = evapo * c.la6[s];
    R remGL0 = R(0);
    if constexpr (WU) {   // routing.cpp:2676-2692
      remUseGL = (fl & F_RES) ? R(0.5) * remainingUse : remainingUse;
      remGL0 = remUseGL;
      PU += remUseGL;
    }
    const R PUmax = TI + maxS + S0;
    rt.p_ow += pin;
    R S;
    if (PU > PUmax) {
      S = -maxS;
      outflow = R(0);
      rt.e_ow += PUmax;
      if constexpr (WT || RO) evapo *= PUmax / PU;
      if constexpr (WU) remUseGL = (remUseGL > R(0)) ? remUseGL - remUseGL * PUmax / PU : R(0);
    } else {
      if constexpr (WU) remUseGL = R(0);
      S = S0 * c.sw_e[s] + c.sw_ik[s] * (TI - PU) * c.sw_ome[s];
      outflow = TI + S0 - S - PU;
      if (S > maxS) {
        outflow += S - maxS;
        S = maxS;
      }
      if (outflow < R(0)) {
        outflow = R(0);
        S = S0 + TI - PU;
      }
      rt.e_ow += PU;
    }
    if (m::fabs_(S) <= R(WG_MIN_STOR_VOL)) S = R(0);
    inflow = outflow;
    if constexpr (WU) dailyActualUse = remGL0 - remUseGL;   // routing.cpp:2788
    if constexpr (WT) wtd->glolake((double)S0 + (double)maxS, evapo, outflow);
    if constexpr (RO) {   // routing.cpp:2648-2664
      ro->owe += (double)evapo * (double)c.la6[s];
      ro->p_lake += (double)pin;
    }
    R r = R(1.) - m::pow(m::fabs_(S - maxS) * (R(0.5) * c.inv_maxs_gl[s]), c.evx[s]);
    st.glolake = S;
    st.rf_glolake = r < R(0) ? R(0) : (r > R(1) ? R(1) : r);
  }
  if (fl & F_RES) {  // reservoir (routing.cpp:2807-3082), each expression rounded as the reference rounds it
    typedef E<R> x;
    const R S0 = st.res, maxS = c.rcap[s], rf = st.rf_res;
    R evapo = x::add(x::mul(x::sub(R(1.0), cfa), owp), x::mul(cfa, x::mul(owpet, rf)));   // routing.cpp:2832-2836
    if (evapo < R(0)) evapo = R(0);
    const R pin = x::mul(owp, c.ra6[s]);
    const R TI = x::add(inflow, pin);
    const R PETgwr = x::mul(evapo, c.ra6[s]);
    const R PETgwrMax = x::add(S0, TI);
    rt.p_ow += pin;
    R remRes0 = R(0);
    if constexpr (WU) {   // routing.cpp:2869-2877
      remUseRes = (fl & F_GLOLAKE) ? R(0.5) * remainingUse + remUseGL : remainingUse;
      remRes0 = remUseRes;
    }
    R S;
    if constexpr (RO) {   // routing.cpp:2826, 2853-2854
      ro->res_in = (double)inflow;
      ro->p_lake += (double)pin;
    }
    if (PETgwr > PETgwrMax) {
      S = S0 + TI - PETgwrMax;
      rt.e_ow += PETgwrMax;
      if constexpr (WT || RO) evapo *= PETgwrMax / PETgwr;
    } else {
      S = S0 + TI - PETgwr;
      rt.e_ow += PETgwr;
    }
    if constexpr (WU) {   // net abstraction down to 10 % of the capacity (routing.cpp:2922-2946)
      const R floor10 = c.rcap01[s];
      if (remUseRes < R(0)) {
        S -= remUseRes;
        rt.e_ow += remUseRes;
        remUseRes = R(0);
      } else if (S > floor10) {
        if (remUseRes < S - floor10) {
          S -= remUseRes;
          rt.e_ow += remUseRes;
          remUseRes = R(0);
        } else {
          const R used = S - floor10;
          remUseRes -= used;
          S = floor10;
          rt.e_ow += used;
        }
      }
    }
    if (m::fabs_(S) <= R(WG_MIN_STOR_VOL)) S = R(0);
    R K = st.k_release;
    if (month == c.start_month[s] - 1 && doy == c_first_day_in_month[month]) {
      K = (S < c.rcap01[s]) ? R(0.1) : x::div(S, x::mul(maxS, R(0.85)));   // routing.cpp:2959-2962
      st.k_release = K;
    }
    // the provisional release of an irrigation reservoir follows the month's demand
    const R prov = WU ? R(wu->tab[wrow + 4 * (size_t)c.n + s]) : c.prov_rel[s];
    R release;   // m3/s (routing.cpp:3003-3008)
    if (c.c_ratio[s] >= R(0.5)) release = x::mul(K, prov);
    else
      release = x::add(x::mul(x::mul(c.c4[s], K), prov),
                       x::div(x::mul(x::mul(c.one_m_c4[s], inflow), R(1.0e9)), R(86400.)));
    // km3 per day; a tenth below 10 % of the capacity (routing.cpp:3012-3017)
    outflow = (S >= c.rcap01[s]) ? x::div(x::mul(release, R(86400.)), R(1.0e9))
                                 : x::div(x::mul(x::mul(R(0.1), release), R(86400.)), R(1.0e9));
    if (outflow < R(0)) outflow = R(0);
    S -= outflow;
    if (S > maxS) {
      outflow += S - maxS;
      S = maxS;
    }
    if (S < R(0)) {
      outflow += S;
      S = R(0);
    }
    inflow = outflow;
    if constexpr (WU) dailyActualUse += remRes0 - remUseRes;   // routing.cpp:3068
    if constexpr (WT) wtd->res(S0, evapo, outflow);
    if constexpr (RO) {   // routing.cpp:2837-2844, 3040
      ro->owe += (double)evapo * (double)c.ra6[s];
      ro->res_out = (double)outflow;
    }
    R r = R(1.) - m::pow(x::div(m::fabs_(S - maxS), maxS), R(2.81383));   // routing.cpp:3071-3072
    st.res = S;
    st.rf_res = r < R(0) ? R(0) : (r > R(1) ? R(1) : r);
  }
  if constexpr (WU) {   // routing.cpp:3083-3172
    if (fl & (F_RES | F_GLOLAKE)) {
      const R remAfter = (fl & F_RES) ? remUseRes : remUseGL;
      if constexpr (GL) {
        // what the lake or reservoir left of its unit's NUs goes back to the unit's
        // riparian cells in proportion to their NUs, as demand of their next routing;
        // the unit's cells in cell order, as the reference's loop over all cells
        const size_t tn = (size_t)c.n;
        const int u = wu->unit_of[s];
        const double agg = wu->tab[wrow + 5 * tn + s], own = wu->tab[wrow + s];
        const double rUseAllocUnsat = (double)totalDesiredUse - agg;
        const double left = (double)remAfter - rUseAllocUnsat;
        for (int k = wu->unit_ptr[u]; k < wu->unit_ptr[u + 1]; ++k) {
          const int i = wu->unit_idx[k];
          double *rip_i = wu->st + 12 * NN + (size_t)i;   // one member: state index = slot
          const double nus_i = wu->tab[wrow + i];
          if (left > 0.) {
            if (own <= 0.) {
              if (i == s) {
                remainingUse = (agg < 0) ? remAfter : R(rUseAllocUnsat);
                W[12 * NN] = 0.;
              } else {
                *rip_i = (nus_i <= 0.) ? 0. : (nus_i / (agg - own)) * left;
              }
            } else {
              if (i == s) {
                remainingUse = R((own / agg) * left + rUseAllocUnsat);
                W[12 * NN] = 0.;
              } else {
                *rip_i = (nus_i < 0.) ? 0. : nus_i / agg * left;
              }
            }
          } else {
            *rip_i = 0.;
            W[12 * NN] = 0.;
            remainingUse = remAfter;
          }
        }
      } else {
        remainingUse = remAfter;
      }
    }
  }
  if (fl & F_GLOWETL) {  // global wetland (routing.cpp:3178-3297)
    const R S0 = st.glowetl, maxS = c.maxs_gw[s], rf = st.rf_glowetl;
    R evapo = (R(1.0) - cfa) * owp * rf + cfa * owpet * rf;
    if (evapo < R(0)) evapo = R(0);
    const R pin = owp * rf * a6 * c.gw100[s];
    const R TI = inflow + pin;
    const R PETgwr = evapo * a6 * c.gw100[s];
    const R PETgwrMax = TI + S0;
    rt.p_ow += pin;
    R S;
    if (PETgwr > PETgwrMax) {
      S = R(0);
      outflow = R(0);
      rt.e_ow += PETgwrMax;
      if constexpr (WT || RO) evapo *= PETgwrMax / PETgwr;
    } else {
      S = S0 * c.sw_e[s] + c.sw_ik[s] * (TI - PETgwr) * c.sw_ome[s];
      outflow = TI + S0 - S - PETgwr;
      rt.e_ow += PETgwr;
    }
    if (S > maxS) {
      outflow += S - maxS;
      S = maxS;
    }
    if (m::fabs_(S) <= R(WG_MIN_STOR_VOL)) S = R(0);
    inflow = outflow;
    if constexpr (WT) wtd->glowetl(S0, evapo, rf, outflow);
    if constexpr (RO) {   // routing.cpp:3194-3210
      ro->owe += (double)evapo * (double)a6 * (double)c.gw100[s];
      ro->gw_ext = (double)rf * (double)c.area[s] * (double)c.gw100[s];
    }
    R r = R(1.) - m::pow(m::fabs_(S - maxS) * c.inv_maxs_gw[s], c.evx[s]);
    st.glowetl = S;
    st.rf_glowetl = r < R(0) ? R(0) : (r > R(1) ? R(1) : r);
  }
  // river (routing.cpp:3385-3514)
  if (c.frac_routing && !(fl & F_SINK)) {   // routing.cpp:3408-3412
    inflow += into_river;
    inflow += gw_into_river;
  }
  const R S0 = st.river;
  const R velocity = (c.velo_opt == 0) ? c.default_velocity : river_velocity<R>(c, s, inflow, S0);
  rt.velocity = velocity;
  const R K = velocity * c.inv_len[s];
  const R eK = m::exp(-K);
  const R omeK = m::one_m_exp_neg(K, eK);
  R S, transported;
  const R remRiver0 = remainingUse;
  if constexpr (WU) {   // the use the river can meet (routing.cpp:3465-3514)
    const R maxUse = inflow + K * S0 * eK * m::rcp(omeK);
    if (remRiver0 > maxUse) {
      S = R(0);
      transported = inflow + S0 - maxUse;
      rt.e_ow += maxUse;
      remainingUse = (remRiver0 > R(0)) ? remRiver0 - remRiver0 * maxUse / remRiver0 : R(0);
    } else {
      S = S0 * eK + (inflow - remRiver0) * omeK * m::rcp(K);
      if (cmp::abs_le_c(S, R(WG_MIN_STOR_VOL))) S = R(0);
      transported = inflow + S0 - S - remRiver0;
      rt.e_ow += remRiver0;
      remainingUse = R(0);
    }
  } else if (cmp::lt0(inflow * omeK + K * S0 * eK)) {   // sign of RivEvapoRemUseMax (routing.cpp:3444-3449)
    const R maxUse = inflow + K * S0 * eK * m::rcp(omeK);   // K >= 1e-5 / length: omeK > 0
    S = R(0);
    transported = inflow + S0 - maxUse;
  } else {
    S = S0 * eK + inflow * omeK * m::rcp(K);
    if (cmp::abs_le_c(S, R(WG_MIN_STOR_VOL))) S = R(0);
    transported = inflow + S0 - S;
  }
  if (cmp::lt0(transported)) {
    rt.leak -= transported;
    transported = R(0);
  }
  st.river = S;
  if constexpr (WU) {
    // what is left comes from the local lake, down to -maxStorage (routing.cpp:3590-3625)
    if ((fl & F_LOCLAKE) && remainingUse > R(0)) {
      const R maxS = c.maxs_ll[s];
      R L = st.loclake;
      if (L > -maxS) {
        if (remainingUse < maxS + L) {
          L -= remainingUse;
          rt.e_ow += remainingUse;
          remainingUse = R(0);
        } else {
          const R used = maxS + L;
          remainingUse -= used;
          L = -maxS;
          rt.e_ow += used;
        }
      }
      st.loclake = L;
      R r = R(1.) - m::pow(m::fabs_(L - maxS) * (R(0.5) * c.inv_maxs_ll[s]), c.evx[s]);
      st.rf_loclake = r < R(0) ? R(0) : (r > R(1) ? R(1) : r);
    }
    dailyActualUse += remRiver0 - remainingUse;
    if constexpr (RO) ro->actual_use = (double)dailyActualUse;   // routing.cpp:3746
    // the cell's bookkeeping (routing.cpp:3736, 3906-3919)
    W[11 * NN] += (double)dailyActualUse;
    if (wu->delayed) {   // routing.cpp:3900-3905
      W[0] = (double)remainingUse - prevTotalUnsat;
      W[6 * NN] = (double)remainingUse;
    } else {
      W[6 * NN] += (double)remainingUse;
      W[0] = (double)remainingUse;
    }
    W[4 * NN] = wu->tab[wrow + 2 * (size_t)c.n + s];
    W[5 * NN] = wu->tab[wrow + 3 * (size_t)c.n + s];
    if (doy == 365) wu_year_end(W, NN);
  }
  if (c.statcorr) {   // station correction (statcorrOpt = 1, routing.cpp:3929-3931)
    const R corrected = transported * c.statcorr[s];
    rt.leak += corrected - transported;   // water the correction adds (removes)
    transported = corrected;
  }
  return transported;
}

// Land-area fraction for the next day (routing.cpp:5034-5188, 5343-5352); returns
// the new land fraction and updates fswb_next.
template <class R>
__device__ __forceinline__ R fraction_next(uint32_t fl, const RState<R> &s, R ll100, R lw100, R gw100, R laf,
                                           R &fswb_next) {
  R f = R(0);
  if ((fl & F_LOCLAKE) && s.rf_loclake > R(0)) f += s.rf_loclake * ll100;
  if ((fl & F_LOCWETL) && s.rf_locwetl > R(0)) f += s.rf_locwetl * lw100;
  if ((fl & F_GLOWETL) && s.rf_glowetl > R(0)) f += s.rf_glowetl * gw100;
  const R changePct = (f - fswb_next) * R(100.);
  fswb_next = f;
  const R next = laf - changePct;
  return next < R(0) ? R(0) : next;
}

}  // namespace wg
