// wg_fastmath.cuh -- FP64 exp / log / pow for the day step on GB300.
//
// GB300 executes FP64 at 1/64 of its FP32 rate, and the FP64 day step is bound by
// the FP64 pipe, so these functions trade the last-ulp accuracy of CUDA's
// libdevice routines for fewer FP64 instructions.  They follow the published
// table-driven methods of P. T. P. Tang:
//   exp: "Table-driven implementation of the exponential function in IEEE
//        floating-point arithmetic", ACM TOMS 15(2), 1989 -- x = (64k + j) ln2/64 + r,
//        exp(x) = 2^k * 2^(j/64) * exp(r), |r| <= ln2/128, Taylor polynomial of degree 5.
//   log: "Table-driven implementation of the logarithm function in IEEE
//        floating-point arithmetic", ACM TOMS 16(4), 1990 -- x = 2^m (F + f),
//        F = 1 + j/128, log x = m ln2 + log F + log1p(f/F), |f/F| <= 1/256,
//        series of log1p to degree 7.
// The tables (2^(j/64), log F, 1/F) are filled on the host from the C library by
// fill_fastmath_tables() in wg_capi.cpp.  Accuracy: about 1 ulp for exp and the
// reciprocal rcp_pos; log to a few ulp of max(|log x|, 1) (just below x = 1 the
// sum m ln2 + log F cancels, leaving an absolute error, which is what pow passes
// on); pow(x, y) =
// exp(y log x) has relative error ~ |y log x| * 2^-52, far inside the 1e-10
// parity bound of the FP64 path.  Only finite positive arguments occur on the
// hot path; x <= 0 in pow returns 0 (the hot path's pow arguments are >= 0 and
// pow(0, y>0) = 0), overflow is not reachable by its arguments.
#pragma once
#include <stdint.h>

namespace wg {
namespace fm {

// tables, filled from the host (the one translation unit that includes this file)
__device__ double g_exp2_tab[64];     // 2^(j/64)
__device__ double g_logF_tab[129];    // log(1 + j/128)
__device__ double g_invF_tab[129];    // 1 / (1 + j/128)

__device__ __forceinline__ double ldexp_fast(double v, int k) {
  // v in [0.5, 4): multiply by 2^k through the exponent field; two steps below the
  // normal range so that subnormal results round once
  if (k >= -1000) return __hiloint2double(__double2hiint(v) + (k << 20), __double2loint(v));
  const double a = __hiloint2double(__double2hiint(v) + ((k + 600) << 20), __double2loint(v));
  return a * 2.409919865102884e-181;   // 2^-600
}

__device__ __forceinline__ double exp(double x) {
  const double inv_l = 92.33248261689366;           // 64 / ln 2
  const double l1 = 0.01083042469326756;            // ln2/64 to 32 bits: n*l1 is exact
  const double l2 = 2.9815858269852933e-12;         // ln2/64 - l1
  // range test on the bit pattern (integer pipe): |x| >= 708 is never on the hot
  // path, so the exact thresholds are only compared there
  if ((__double_as_longlong(x) & 0x7fffffffffffffffll) >= 0x4086200000000000ll) {   // |x| >= 708
    if (x < -745.2) return 0.0;
    if (x > 709.78) return __longlong_as_double(0x7ff0000000000000ll);
  }
  // n = round(x * 64/ln2) with the 1.5 * 2^52 shifter: the low word of t is n and
  // t - shifter is n as a double (one FMA and one add instead of a round and two
  // conversions on the FP64 pipe)
  const double shifter = 6755399441055744.0;
  const double t = fma(x, inv_l, shifter);
  const int n = __double2loint(t);
  const double nd = t - shifter;
  double r = fma(-nd, l1, x);
  r = fma(-nd, l2, r);
  double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  q = fma(q, r, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  const double p = fma(q * r, r, r);                 // exp(r) - 1
  const double s = g_exp2_tab[n & 63];
  return ldexp_fast(fma(s, p, s), n >> 6);
}

// natural log of a positive normal number
__device__ __forceinline__ double log(double x) {
  const double ln2_hi = 0.6931471803691238;          // ln2 to 32 bits: m*ln2_hi is exact
  const double ln2_lo = 1.9082149292705877e-10;      // ln2 - ln2_hi
  int hi = __double2hiint(x);
  const int lo = __double2loint(x);
  int m = (hi >> 20) - 1023;
  const int hm = hi & 0x000fffff;
  const double y = __hiloint2double(hm | 0x3ff00000, lo);   // y in [1, 2)
  // F = 1 + j/128 nearest to y, from the mantissa bits (integer pipe): j rounds
  // the top 7 mantissa bits, half up; F is built from j's bits
  const int j = (hm + 0x1000) >> 13;
  const double F = __hiloint2double(0x3ff00000 + (j << 13), 0);
  const double f = y - F;                             // exact
  const double u = f * g_invF_tab[j];
  // log1p(u) = u - u^2/2 + u^3/3 - ... to degree 7
  double q = fma(u, -1.0 / 7.0, 1.0 / 6.0);
  q = fma(q, u, -1.0 / 5.0);
  q = fma(q, u, 1.0 / 4.0);
  q = fma(q, u, -1.0 / 3.0);
  q = fma(q, u, 0.5);
  const double u2 = u * u;
  const double l1p = fma(-q, u2, u);
  const double md = (double)m;
  return fma(md, ln2_hi, g_logF_tab[j] + fma(md, ln2_lo, l1p));
}

// 1/x for finite normal nonzero x: the hardware's approximate reciprocal
// (rcp.approx.ftz.f64, relative error checked against 2^-20 by the tests) refined
// by one third-order Newton-Raphson step r' = r (1 + e + e^2), e = 1 - x r
// (P. Markstein, "IA-64 and Elementary Functions", 2000, ch. 8), which cubes the
// relative error: three FMAs on the FP64 pipe instead of a correctly rounded
// division's longer sequence.  Result within about 1 ulp of 1/x (not always
// correctly rounded).  The hot path calls it only with divisors bounded away from
// zero (temperature + 237.3, latent heat, the canopy capacity, the wetted perimeter,
// the river's outflow constant).
__device__ __forceinline__ double rcp_pos(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
}

// x^y for x >= 0, y > 0 (the hot path's exponents are positive constants or
// calibration parameters)
__device__ __forceinline__ double pow(double x, double y) {
  const long long b = __double_as_longlong(x);
  if (b <= 0) return 0.0;                              // x <= 0 (and -0)
  if (b == 0x3ff0000000000000ll) return 1.0;           // x == 1
  return fm::exp(y * fm::log(x));
}

}  // namespace fm

}  // namespace wg
