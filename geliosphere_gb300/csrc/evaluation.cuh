// Spectrum evaluation on the device: the reference evaluators' FP64 weights
// and binnings, applied to each exit record as it happens.
//
//   2D    Algorithm/src/TwoDimensionBpResults.cpp:40-105
//   1D B-p Algorithm/src/OneDimensionBpResults.cpp:20-87
//   1D F-p Algorithm/src/OneDimensionFpResults.cpp:19-88
//   constants Algorithm/include/ResultConstants.hpp:19-117
//
// In the reference the simulation prints each record to log.dat with "%g"
// (six significant digits) and the evaluator reads it back.  round6() below
// reproduces that printf -> strtod round trip exactly, so a spectrum binned
// here equals the spectrum the reference evaluator computes from the log
// file of the same records (bin edges such as the AMS edges coincide with
// injection energies of the 1e-4 GeV reference grid, so this matters).
#pragma once
#include <cstdint>
#include <cstddef>
#include "gelio.h"
#include "pow10_table.h"

namespace gelio {

// FP64 constants of ResultConstants.hpp:19-55.
constexpr double kM0 = 1.67261e-27;
constexpr double kQ = 1.60219e-19;
constexpr double kC = 2.99793e8;
constexpr double kT0w = kM0 * kC * kC;
constexpr double kTr = 0.938;

// Flat layout of gelio_spectra, in doubles.
constexpr int kOffLogW = offsetof(gelio_spectra, log_w) / 8;
constexpr int kOffLogW2 = offsetof(gelio_spectra, log_w2) / 8;
constexpr int kOffLogN = offsetof(gelio_spectra, log_n) / 8;
constexpr int kOffE2W = offsetof(gelio_spectra, e2_w) / 8;
constexpr int kOffE2W2 = offsetof(gelio_spectra, e2_w2) / 8;
constexpr int kOffE2N = offsetof(gelio_spectra, e2_n) / 8;
constexpr int kOffE3W = offsetof(gelio_spectra, e3_w) / 8;
constexpr int kOffE3W2 = offsetof(gelio_spectra, e3_w2) / 8;
constexpr int kOffE3N = offsetof(gelio_spectra, e3_n) / 8;
constexpr int kOffE4W = offsetof(gelio_spectra, e4_w) / 8;
constexpr int kOffE4W2 = offsetof(gelio_spectra, e4_w2) / 8;
constexpr int kOffE4N = offsetof(gelio_spectra, e4_n) / 8;
constexpr int kOffSpWeber = offsetof(gelio_spectra, sp_weber) / 8;
constexpr int kOffSpJgr = offsetof(gelio_spectra, sp_jgr) / 8;
constexpr int kOffSpBurger = offsetof(gelio_spectra, sp_burger) / 8;
constexpr int kOffSpN = offsetof(gelio_spectra, sp_n) / 8;
constexpr int kOffSpWeber2 = offsetof(gelio_spectra, sp_weber2) / 8;
constexpr int kOffSpJgr2 = offsetof(gelio_spectra, sp_jgr2) / 8;
constexpr int kOffSpBurger2 = offsetof(gelio_spectra, sp_burger2) / 8;
constexpr int kOffUlyW = offsetof(gelio_spectra, uly_w) / 8;
constexpr int kOffUlyW2 = offsetof(gelio_spectra, uly_w2) / 8;
constexpr int kOffUlyN = offsetof(gelio_spectra, uly_n) / 8;
constexpr int kOffAmsW = offsetof(gelio_spectra, ams_w) / 8;
constexpr int kOffAmsW2 = offsetof(gelio_spectra, ams_w2) / 8;
constexpr int kOffAmsN = offsetof(gelio_spectra, ams_n) / 8;
constexpr int kOffGridW = offsetof(gelio_spectra, grid_w) / 8;
constexpr int kOffGridW2 = offsetof(gelio_spectra, grid_w2) / 8;
constexpr int kOffGridN = offsetof(gelio_spectra, grid_n) / 8;
constexpr int kOffNParticles = offsetof(gelio_spectra, n_particles) / 8;
constexpr int kOffNRecords = offsetof(gelio_spectra, n_records) / 8;
constexpr int kOffNSteps = offsetof(gelio_spectra, n_steps) / 8;
constexpr int kOffNLost = offsetof(gelio_spectra, n_lost) / 8;
constexpr int kOffNCapped = offsetof(gelio_spectra, n_step_capped) / 8;
constexpr int kSpecDoubles = sizeof(gelio_spectra) / 8;
static_assert(sizeof(gelio_spectra) % 8 == 0, "spectra layout");

// Window of the layout each dimensionality touches (used to size the
// per-block shared-memory histogram): 1D models use [0, kOffSpWeber) plus
// the grid and counters, 2D models [kOffSpWeber, kSpecDoubles).
constexpr int kWin2DLo = kOffSpWeber;
constexpr int kWin1DLo = 0;
constexpr int kWinHi = kSpecDoubles;

// Bin tables, filled by the host from the reference definitions.
struct BinTables {
  double sp[32];        // SPbins (ResultConstants.hpp:86-90)
  double uly[4];        // UlyssesBins
  double ams[72];       // AmsBins
  double bp_log[81];    // binb[i] = 10^(X - i dlT), i < NT = 80 (OneDimensionBpResults.cpp:25-31)
  double fp_log[25];    // binb[i] = 10^((i+1)/5 - 3)          (OneDimensionFpResults.cpp:24-27)
  float sp30[30];       // getSolarPropInjection energies 0.01 * 1.5^k
};

// ---------------------------------------------------------------------------
// printf("%g") -> strtod round trip: x rounded to six significant digits.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double pow10_hi(int k) { return kPow10Hi[k + 40]; }
__device__ __forceinline__ double pow10_lo(int k) { return kPow10Lo[k + 40]; }

static __device__ __noinline__ double round6(double xin) {
  if (!(xin != 0.0) || !(fabs(xin) < 1e300)) return xin;   // 0, NaN, huge: unchanged
  const double sign = (xin < 0.0) ? -1.0 : 1.0;
  const double x = fabs(xin);
  int e = (int)floor(log10(x));
  if (e < -34 || e > 34) return xin;
  // exact decimal exponent: 10^e <= x < 10^(e+1)
  if (x < pow10_hi(e)) --e;
  else if (x >= pow10_hi(e + 1)) ++e;
  const int k = 5 - e;                        // x * 10^k in [1e5, 1e6)
  // m = rint(x * 10^k) with the product carried in double-double
  const double ph = pow10_hi(k), pl = pow10_lo(k);
  const double p = x * ph;
  const double perr = fma(x, ph, -p) + x * pl;
  double m = rint(p);
  const double frac = (p - m) + perr;          // exact remainder relative to m
  if (frac > 0.5) m += 1.0;
  else if (frac < -0.5) m -= 1.0;
  else if (frac == 0.5 || frac == -0.5) {
    // exact tie: round half to even
    const double mm = (frac > 0.0) ? m + 1.0 : m - 1.0;
    if (fmod(mm, 2.0) == 0.0) m = mm;
  }
  // value m * 10^-k, correctly rounded
  if (k <= 0) return sign * (m * pow10_hi(-k));   // 10^-k exact for -k <= 22
  const double dh = pow10_hi(k), dl = pow10_lo(k);
  double y = m / dh;
  // one correction with the double-double divisor: y = m / (dh + dl)
  const double res = fma(-y, dh, m) - y * dl;
  y = y + res / dh;
  return sign * y;
}

// Momentum in SI from kinetic energy in GeV, as the evaluators compute it:
// Tkinw = T 1e9 q; Rig = sqrt(Tkinw (Tkinw + 2 T0w)) / q; p = Rig q / c.
__device__ __forceinline__ double p_si(double T) {
  const double Tw = __dmul_rn(__dmul_rn(T, 1e9), kQ);
  const double rig = __ddiv_rn(__dsqrt_rn(__dmul_rn(Tw, __dadd_rn(Tw, __dmul_rn(2.0, kT0w)))), kQ);
  return __ddiv_rn(__dmul_rn(rig, kQ), kC);
}

// LIS fluxes of TwoDimensionBpResults.cpp:50-76.
__device__ __forceinline__ double lis_weber(double T) {
  const double l = log(T);
  const double tem5 = 21.1 * exp(-2.8 * l);
  const double tem6 = 1.0 + (5.85 * exp(-1.22 * l)) + (1.18 * exp(-2.54 * l));
  return tem5 / tem6;
}
__device__ __forceinline__ double lis_usoskin(double T) {
  const double tt = T + kTr;
  const double t2 = tt + kTr;
  const double beta = sqrt(T * t2) / tt;
  double tem = (T + 0.67) / 1.67;
  tem = exp(-3.93 * log(tem));
  double j = 2.7e3 * exp(1.12 * log(T)) * tem;
  return j / (beta * beta);
}
__device__ __forceinline__ double lis_burger(double T) {
  double tem = sqrt((T * T) + (2.0 * T * 0.938));
  double j = 1.9 * 1.0e4 * exp(-2.78 * log(tem));
  tem = sqrt((T * T) + (2.0 * T * 0.938));
  tem = 0.4866 * exp(-2.51 * log(tem));
  return j / (1 + tem);
}

// Yamada et al. 1998 weight of OneDimensionBpResults.cpp:58-60 (no 1e45
// scaling) and of OneDimensionFpResults.cpp:56-57 (scaled by 1e-45).
__device__ __forceinline__ double yamada(double p) {
  const double w = (kM0 * kM0 * kC * kC * kC * kC) + (p * p * kC * kC);
  return exp(-1.85 * log(w)) / p;
}

// Kinetic energy [GeV] from an SI momentum, as OneDimensionFpResults.cpp:51-54.
__device__ __forceinline__ double fp_tkin_from_p(double p1AU) {
  const double T0 = kM0 * kC * kC / (kQ * 1e9);
  const double Rig = p1AU * kC / kQ;
  double T = sqrt((T0 * T0 * kQ * kQ * 1e9 * 1e9) + (kQ * kQ * Rig * Rig)) - (T0 * kQ * 1e9);
  return T / (kQ * 1e9);
}

// Log bin of an energy over the grid section.
__device__ __forceinline__ int grid_log_bin(double T, double lo_log, double inv_dlog, int bins) {
  if (!(T > 0.0) || bins <= 0) return -1;
  const double x = (log(T) - lo_log) * inv_dlog;
  if (!(x >= 0.0)) return -1;
  const int b = (int)x;
  return (b < bins) ? b : -1;
}

// SolarProp window bin (1..29) of TwoDimensionBpResults.cpp:80-89, 0 if none.
__device__ __forceinline__ int bin_sp(double Ti, const BinTables &t) {
  for (int ii = 1; ii < 30; ii++)
    if ((Ti > t.sp[ii] * 0.99) && (Ti < t.sp[ii] * 1.01)) return ii;
  return 0;
}
__device__ __forceinline__ int bin_uly(double Ti, const BinTables &t) {
  for (int ii = 1; ii < 3; ii++)
    if ((Ti > t.uly[ii]) && (Ti < t.uly[ii + 1])) return ii;
  return 0;
}
__device__ __forceinline__ int bin_ams(double Ti, const BinTables &t) {
  if (!(Ti > t.ams[1]) || !(Ti < t.ams[71])) return 0;
  int lo = 1, hi = 70;          // find ii with ams[ii] < Ti < ams[ii+1]
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (t.ams[mid] < Ti) lo = mid; else hi = mid - 1;
  }
  return (Ti > t.ams[lo] && Ti < t.ams[lo + 1]) ? lo : 0;
}
// 1D B-p spelog bin: index ii+1 for binb[ii+1] < Ti < binb[ii], ii in [0, 78].
__device__ __forceinline__ int bin_bp_log(double Ti, const BinTables &t) {
  if (!(Ti < t.bp_log[0]) || !(Ti > t.bp_log[79])) return -1;
  int lo = 0, hi = 78;          // binb decreasing: find ii with binb[ii+1] < Ti
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (t.bp_log[mid + 1] < Ti) hi = mid; else lo = mid + 1;
  }
  return (Ti > t.bp_log[lo + 1] && Ti < t.bp_log[lo]) ? lo + 1 : -1;
}
// 1D F-p spelog bin: binb[i] < T < binb[i+1], i in [0, 23].
__device__ __forceinline__ int bin_fp_log(double T, const BinTables &t) {
  if (!(T > t.fp_log[0]) || !(T < t.fp_log[24])) return -1;
  int lo = 0, hi = 23;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (t.fp_log[mid] < T) lo = mid; else hi = mid - 1;
  }
  return (T > t.fp_log[lo] && T < t.fp_log[lo + 1]) ? lo : -1;
}
// Linear binnings of the 1D evaluators: 1-based index into spe1e2/1e3/4e2.
__device__ __forceinline__ int bin_e2(double T) { const int e = (int)trunc(T); return (e > 0 && e < 101) ? e : 0; }
__device__ __forceinline__ int bin_e3(double T) { const int e = (int)trunc((T + 0.05) * 10); return (e > 0 && e < 1001) ? e : 0; }
__device__ __forceinline__ int bin_e4(double T) { const int e = (int)trunc((T + 0.125) * 4); return (e > 0 && e < 401) ? e : 0; }

// ---------------------------------------------------------------------------
// One evaluated record: weights and bins of every section it lands in.
// ---------------------------------------------------------------------------
struct Contribution {
  double w[3];          // section weights (2D: Weber, Usoskin, Burger; 1D: ref, -, -)
  double gw[3];         // grid-section weights
  int b_sp, b_uly, b_ams;              // 2D
  int b_log, b_e2, b_e3, b_e4;         // 1D
  int b_grid;
};

// 2D record: injection energy Ti (1 AU) and exit energy Te (100 AU), both
// already passed through round6 (the log.dat columns Tkininj and Tkin).
__device__ inline void eval_2d(double Ti, double Te, const BinTables &t, Contribution &o) {
  const double p = p_si(Te);
  const double p1AU = p_si(Ti);
  const double ratio = (p1AU * p1AU) / (p * p);
  // TwoDimensionBpResults.cpp:50-54: the Weber LIS is evaluated at Tkininj.
  o.w[0] = lis_weber(Ti) / (p * p) * p1AU * p1AU;
  o.w[1] = lis_usoskin(Te) / (p * p) * p1AU * p1AU;
  o.w[2] = lis_burger(Te) / (p * p) * p1AU * p1AU;
  o.gw[0] = lis_weber(Te) * ratio;
  o.gw[1] = lis_usoskin(Te) * ratio;
  o.gw[2] = lis_burger(Te) * ratio;
  o.b_sp = bin_sp(Ti, t);
  o.b_uly = bin_uly(Ti, t);
  o.b_ams = bin_ams(Ti, t);
}

// 1D B-p record: Ti = log column "Tkin" (1 AU injection energy), Te = column
// "Tkininj" (100 AU exit energy) -- the reference writes the exit energy
// first (OneDimensionBpModel.cu:192) and reads it as Tkininj.
__device__ inline void eval_bp(double Ti, double Te, const BinTables &t, Contribution &o) {
  const double p = p_si(Te);
  const double p1AU = p_si(Ti);
  double w = yamada(p);
  w = w * p1AU * p1AU;
  const double ratio = (p1AU * p1AU) / (p * p);
  o.w[0] = w; o.w[1] = 0.0; o.w[2] = 0.0;
  o.gw[0] = w;
  o.gw[1] = lis_weber(Te) * ratio;
  o.gw[2] = lis_burger(Te) * ratio;
  o.b_log = bin_bp_log(Ti, t);
  o.b_e2 = bin_e2(Ti);
  o.b_e3 = bin_e3(Ti);
  o.b_e4 = bin_e4(Ti);
}

// 1D F-p record: p100AU, p1AU (SI), r, sumac as read from log.dat.
__device__ inline void eval_fp(double p100AU, double p1AU, double r, double sumac,
                               const BinTables &t, Contribution &o, double &T1AU) {
  const double T = fp_tkin_from_p(p1AU);
  double w0 = yamada(p100AU) / 1e45;
  double w = w0 * p1AU * p1AU * exp(sumac);
  if (r < 0.3) w = 0.0;
  T1AU = T;
  o.w[0] = w; o.w[1] = 0.0; o.w[2] = 0.0;
  o.gw[0] = w; o.gw[1] = 0.0; o.gw[2] = 0.0;
  o.b_log = bin_fp_log(T, t);
  o.b_e2 = bin_e2(T);
  o.b_e3 = bin_e3(T);
  o.b_e4 = bin_e4(T);
}

}  // namespace gelio
