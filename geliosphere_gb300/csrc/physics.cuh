// Per-particle SDE steps of the four heliospheric transport models.
//
// Each step restates the reference GPU kernels' equations (paths relative to
// the reference project):
//   2D Geliosphere   CUDAKernel/src/GeliosphereModel.cu:82-390
//   2D SolarProp     CUDAKernel/src/SolarPropLikeModel.cu:95-247
//   1D B-p           CUDAKernel/src/OneDimensionBpModel.cu:69-140
//   1D F-p           CUDAKernel/src/OneDimensionFpModel.cu:73-141
// in a form arranged for sm_103a:
//   * kinetic energy and rigidity in GeV / GV instead of SI (the reference's
//     FP32 T0^2 q^2 1e18 intermediates sit next to FLT_MIN); the kinetic
//     energy from momentum uses P^2 / (sqrt(T0^2 + P^2) + T0), which is the
//     reference's sqrt(T0^2 + P^2) - T0 without the cancellation;
//   * powf(Cb, 1.5 / 2.5 / 3) become products of Cb and one sqrt; repeated
//     divisions become multiplications by a handful of reciprocals;
//   * the FP32 state (r, theta, T, p, sumac) is updated with Kahan
//     compensation, so tens of thousands of steps do not accumulate rounding;
//   * the noise terms with coefficients that are identically zero in the
//     reference (B13 = B23 = 0 because Krph = Ktph = 0) are not evaluated.
// The same templates are instantiated in FP64 (the FP64-step variant).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gelio {

// ---------------------------------------------------------------------------
// Constants, with the values and FP32 arithmetic of CosmicConstants.cu:14-41.
// ---------------------------------------------------------------------------
constexpr float kPi = 3.141592654f;
constexpr float kT0 = (float)(1.67261e-27 * 2.99793e8 * 2.99793e8 / (1.60219e-19 * 1e9));
constexpr float kOmega = 2.866e-6f;
constexpr float kA = 3.4f;
constexpr float kKonvF = 9.0e-5f / 2.0f;
constexpr float kRh = 0.0046367333333333f;
constexpr float kThetaLo = 1.7f * kPi / 180.0f;    // GeliosphereModel.cu:97
constexpr float kThetaHi = 178.3f * kPi / 180.0f;
constexpr float kC53 = 5.0f / 3.4f;
constexpr float kTwoPi = 2.0f * kPi;
// SolarPropLikeModel.cu:213 uses the fixed constant of CosmicConstants.cu:37.
constexpr float kDriftThetaConstantSP = -1.0f * 1.0f * (9.0e-5f / 2.0f) * (2.0f / (3.0f * 3.4f));

// Model ids (match GELIO_MODEL_* in gelio.h).
constexpr int kModelFp = 0;
constexpr int kModelBp = 1;
constexpr int kModelSolarProp = 2;
constexpr int kModelGeliosphere = 3;

// ---------------------------------------------------------------------------
// Precision policy.
// ---------------------------------------------------------------------------
template <class R> struct Math;

template <> struct Math<float> {
  static constexpr bool kCompensate = true;
  __device__ static __forceinline__ float sqrt(float x) { return sqrtf(x); }
  __device__ static __forceinline__ float rsqrt(float x) { return rsqrtf(x); }
  __device__ static __forceinline__ float rcp(float x) { return __fdividef(1.0f, x); }
  __device__ static __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
  __device__ static __forceinline__ void sincos(float x, float *s, float *c) { sincosf(x, s, c); }
  __device__ static __forceinline__ float sin(float x) { return sinf(x); }
  __device__ static __forceinline__ float acos(float x) { return acosf(x); }
  __device__ static __forceinline__ float atan(float x) { return atanf(x); }
  __device__ static __forceinline__ float abs(float x) { return fabsf(x); }
  __device__ static __forceinline__ float copysign(float x, float y) { return copysignf(x, y); }
};

template <> struct Math<double> {
  static constexpr bool kCompensate = false;
  __device__ static __forceinline__ double sqrt(double x) { return ::sqrt(x); }
  __device__ static __forceinline__ double rsqrt(double x) { return ::rsqrt(x); }
  __device__ static __forceinline__ double rcp(double x) { return 1.0 / x; }
  __device__ static __forceinline__ double div(double a, double b) { return a / b; }
  __device__ static __forceinline__ void sincos(double x, double *s, double *c) { ::sincos(x, s, c); }
  __device__ static __forceinline__ double sin(double x) { return ::sin(x); }
  __device__ static __forceinline__ double acos(double x) { return ::acos(x); }
  __device__ static __forceinline__ double atan(double x) { return ::atan(x); }
  __device__ static __forceinline__ double abs(double x) { return fabs(x); }
  __device__ static __forceinline__ double copysign(double x, double y) { return ::copysign(x, y); }
};

// Kahan-compensated scalar: value v, running compensation c (true ~ v - c).
template <class R> struct Acc {
  R v, c;
  __device__ __forceinline__ void set(R x) { v = x; c = R(0); }
  __device__ __forceinline__ void add(R d) {
    if constexpr (Math<R>::kCompensate) {
      const R y = d - c;
      const R t = v + y;
      c = (t - v) - y;
      v = t;
    } else {
      v += d;
    }
  }
  __device__ __forceinline__ void negate() { v = -v; c = -c; }
};

// Raw parameters of one simulation (device copy of gelio_sim_params, resolved).
struct SimDev {
  float K0, V, dt, r_inj, theta_inj, tilt, polarity, ratio, delta0;
  float injection_max, inj_min, inj_max;
  int model, injection, inj_points, flags;
  float grid_min, grid_max;
  int grid_bins;
  int grid_is_points;        // grid bin = LOG_GRID point index
  uint32_t key0, key1;       // Philox key
  long long n_particles;
  double grid_log_lo, grid_inv_dlog;
};

// Per-lane constants of the current particle's simulation, in precision R.
template <class R> struct Consts {
  R V, dt, sqdt, K0, ratio, one_m_ratio, delta0, alphaM;
  R ov, ov2;          // omega / V and its square
  R kpar_c;           // K0 * (5/3.4) / 3
  R kd_c;             // K0 / (3 * (5/3.4))
  R inv_3c53;         // 1 / (3 * (5/3.4))
  R d0rh2;            // delta0^2 / rh^2
  R drift2;           // polarity * konvF * 2 / (3A)
  R drift1;           // polarity * konvF * 1 / (3A)
  R dtheta_sp;        // SolarProp theta drift constant
  R adv;              // 1D: (2/3) V dt; 2D: (2/3) V dt as well
  R sq2K0dt;          // sqrt(2 K0 dt)
};

template <class R>
__device__ __forceinline__ void make_consts(const SimDev &s, Consts<R> &k) {
  using M = Math<R>;
  const R V = (s.model == kModelBp) ? -(R)s.V : (R)s.V;   // CosmicConstants.cu:73-83
  k.V = V;
  k.dt = (R)s.dt;
  k.sqdt = M::sqrt(k.dt);
  k.K0 = (R)s.K0;
  k.ratio = (R)s.ratio;
  k.one_m_ratio = R(1) - k.ratio;
  k.delta0 = (R)s.delta0;
  k.alphaM = (R)s.tilt;
  k.ov = M::div((R)kOmega, V);
  k.ov2 = k.ov * k.ov;
  k.kpar_c = k.K0 * (R)kC53 * M::rcp(R(3));
  k.kd_c = M::div(k.K0, R(3) * (R)kC53);
  k.inv_3c53 = M::rcp(R(3) * (R)kC53);
  k.d0rh2 = M::div(k.delta0 * k.delta0, (R)kRh * (R)kRh);
  k.drift2 = (R)s.polarity * (R)kKonvF * M::div(R(2), R(3) * (R)kA);
  k.drift1 = (R)s.polarity * (R)kKonvF * M::div(R(1), R(3) * (R)kA);
  k.dtheta_sp = (s.flags & 1) ? -(R)s.polarity * (R)kKonvF * M::div(R(2), R(3) * (R)kA)
                              : (R)kDriftThetaConstantSP;
  k.adv = R(2) * V * k.dt * M::rcp(R(3));
  k.sq2K0dt = M::sqrt(R(2) * k.K0 * k.dt);
}

// ---------------------------------------------------------------------------
// Injection energies (GeV, FP32 exactly as specified so the oracle can
// reproduce them bit for bit).
// ---------------------------------------------------------------------------

// CosmicUtils.cu:17-34 with injectionMax * quantityPerEnergy computed in FP32
// and the integer parts taken exactly (the reference's float division is exact
// for the particle indices below 2^24 it is used with).
__device__ __forceinline__ float inj_reference_uniform(unsigned long long s, float injection_max) {
  const float mq = __fmul_rn(injection_max, 10000.0f);
  const unsigned long long m = (unsigned long long)mq;
  if ((float)s > mq && m > 0ull) s -= (s / m) * m;
  const unsigned long long mod = (s >= 10000ull) ? s / 10000ull : 0ull;
  const float frac = __fdiv_rn((float)(s - mod * 10000ull + 1ull), 10000.0f);
  return __fadd_rn((float)mod, frac);
}

// Constants.hpp:234-239 (the CPU models' grid): from + (id mod 1e4) * step.
__device__ __forceinline__ float inj_cpu_uniform(unsigned long long s, float injection_max) {
  const double step = ((double)injection_max - 0.0001) / 10000.0;
  return (float)(0.0001 + (double)(s % 10000ull) * step);
}

__device__ __forceinline__ float inj_solarprop(unsigned long long s, const float *sp30) {
  return sp30[(int)(s % 30ull)];
}

// ---------------------------------------------------------------------------
// Lane state.
// ---------------------------------------------------------------------------
template <class R> struct Lane {
  Acc<R> r, th, T, P, sumac;
  R Pt, q;             // F-p: the rigidity T was computed from, 1 / sqrt(Pt^2 + T0^2)
  float thn;           // FP32 2D models: theta = 2 pi thn + th once theta has left [0, 2 pi)
  float Tinj;
  float rrec;          // F-p: r of the last 1 AU crossing, before a reflection undoes the step
  uint32_t steps;
  int sim;
  int gbin;
  unsigned long long pid;
  uint32_t key0, key1;
  R zc0, zc1, zc2;     // 2D Geliosphere: normals drawn for the next steps of the group of four
};

// Outcome of one step.
enum StepResult : int { kContinue = 0, kRecordAndStop = 1, kStop = 2, kRecordAndContinue = 3 };

// ---------------------------------------------------------------------------
// Theta bookkeeping of the 2D models.
//
// The reference reflects theta once per step (GeliosphereModel.cu:366-377):
//   theta < 0 -> |theta|;  theta > 2 pi -> theta - 2 pi;  else theta > pi -> 2 pi - theta.
// Near the poles the drift terms (1/sin^3 theta) can throw theta far outside
// [0, pi]; a single reflection does not bring it back, and such "runaway"
// trajectories (about 16% of 2D exits) keep |theta| up to 1e20 and beyond.
// In FP64 their sin/cos still see the phase of theta; a plain FP32 theta
// loses it above 2^24 rad (it freezes and its sin/cos are quantised), which
// shortens those trajectories by ~10% and biases the low-energy spectra.
// The FP32 kernels therefore keep a runaway theta as 2 pi * thn + phase with
// the phase in [0, 2 pi): the reference's reflections act exactly on that
// value, sin/cos use the full-precision phase, and FP64's freezing of theta
// (an update below half an FP64 ulp of |theta| leaves it unchanged) is
// reproduced.  Trajectories whose theta stays in [0, 2 pi) never take this path.
// ---------------------------------------------------------------------------
constexpr float kTwoPiHi = 6.28318548202514648f;     // 2 pi = kTwoPiHi + kTwoPiLo
constexpr float kTwoPiLo = -1.74845553e-7f;
constexpr float kInvTwoPi = 0.159154943091895336f;

template <class R>
__device__ __forceinline__ R theta_full(const Lane<R> &L) {
  if constexpr (sizeof(R) == 4) return fmaf(L.thn, kTwoPiHi, L.th.v);
  else return L.th.v;
}

__device__ __forceinline__ void phase_normalise(Acc<float> &ph, float &n) {
  float x = ph.v;
  if (x >= 0.0f && x < kTwoPiHi) return;
  const float k = floorf(x * kInvTwoPi);
  x = fmaf(-k, kTwoPiHi, x);
  x = fmaf(-k, kTwoPiLo, x);
  n += k;
  if (x < 0.0f) { x += kTwoPiHi; n -= 1.0f; }
  if (x >= kTwoPiHi) { x -= kTwoPiHi; n += 1.0f; }
  ph.set(x);
}

// sin and cos of the compensated phase v - c (first order in the residual c,
// |c| <= ulp(v)/2): keeps sin(theta) accurate near theta = pi, where an FP32
// theta alone is only known to 2.4e-7 rad.
template <class R>
__device__ __forceinline__ void phase_sincos(const Acc<R> &ph, R *s, R *c) {
  Math<R>::sincos(ph.v, s, c);
  if constexpr (Math<R>::kCompensate) {
    const R s0 = *s, c0 = *c;
    *s = fmaf(-ph.c, c0, s0);
    *c = fmaf(ph.c, s0, c0);
  }
}

// The reference's single reflection of theta (theta < 0 -> |theta|; theta > 2 pi
// -> theta - 2 pi; else theta > pi -> 2 pi - theta) as selects, not branches.
template <class R>
__device__ __forceinline__ void reflect_theta(Acc<R> &t) {
  R v = t.v, c = t.c;
  const bool neg = v < R(0);
  v = neg ? -v : v;
  c = neg ? -c : c;
  const bool over = v > (R)kTwoPi;
  const bool flip = !over && v > (R)kPi;
  const R w = over ? v - (R)kTwoPi : (R)kTwoPi - v;
  t.v = (over || flip) ? w : v;
  t.c = (over || flip) ? R(0) : c;
}

template <class R>
__device__ __forceinline__ void theta_update(Lane<R> &L, R dth) {
  if constexpr (sizeof(R) == 8) {
    L.th.add(dth);
    reflect_theta(L.th);
  } else {
    if (L.thn == 0.0f) {
      L.th.add(dth);
      reflect_theta(L.th);
      if (L.th.v >= kTwoPiHi) phase_normalise(L.th, L.thn);   // runaway: switch representation
    } else {
      // an update below half an FP64 ulp of |theta| leaves theta unchanged
      if (fabsf(dth) < fabsf(L.thn) * kTwoPiHi * 1.1102230246251565e-16f) dth = 0.0f;
      L.th.add(dth);
      phase_normalise(L.th, L.thn);
      if (L.thn < 0.0f) {                       // theta < 0 -> |theta|
        L.thn = -L.thn - 1.0f;
        L.th.set(kTwoPiHi - L.th.v);
        phase_normalise(L.th, L.thn);
      }
      if (L.thn >= 1.0f && !(L.thn == 1.0f && L.th.v == 0.0f)) {
        L.thn -= 1.0f;                          // theta > 2 pi -> theta - 2 pi
      } else if (L.thn == 0.0f && L.th.v > kPi) {
        L.th.set(kTwoPi - L.th.v);              // theta > pi -> 2 pi - theta
      } else if (L.thn == 1.0f && L.th.v == 0.0f) {
        L.thn = 0.0f;                           // theta == 2 pi -> 0
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 2D Geliosphere: GeliosphereModel.cu:82-390 (Eq. 16-44 of the Geliosphere
// model description, drifts of Kappl 2016 Eq. 26-37).
//
// The same equations, evaluated with shared factors so that the step issues
// fewer FP32 instructions (the kernel is bound by instruction issue):
//   * beta P, r^2 / sqrt(Cb), (1 - ratio) kd / Cb^2.5 and the drift prefactor
//     P beta r gamma / Cb are formed once;
//   * K0 beta P (Eq. 39) = 3 (5/3.4) kd, so Eq. 38-42 collapse to
//     dKtt / r^2 = -CKtt0 (ratio kd / Cb^1.5 + 9 (5/3.4) (1 - ratio) kd rd2 / Cb^2.5)
//     off the poles, and Eq. 44 / r = -3 dKrtr gamma^2 cot(theta);
//   * Eq. 35-36: 2 r sqrt(Cb) - r^2 COmega / (2 sqrt(Cb)) = (2 r Cb - r^2 COmega / 2) / sqrt(Cb)
//     (and the Cb^1.5 form likewise), so one 2 r Cb serves both;
//   * Eq. 16: Krr Ktt - Krt^2 = Kper (Ktt + dK / Cb) exactly (Krt^2 = rd2 (dK / Cb)^2),
//     which also removes the cancellation of the difference; sqrt(dt) goes
//     into one factor sqrt(2 dt / Ktt) shared by B11 and B12, and B22 sqrt(dt)
//     = Ktt sqrt(2 dt / Ktt) / r;
//   * Eq. 23: T (T + 2 T0) / (T + T0) = P beta;
//   * dt and 1 / r are applied once to the summed deterministic terms of dr
//     and dtheta.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ int step_geliosphere(Lane<R> &L, const Consts<R> &k, R n1, R n2, R n4) {
  using M = Math<R>;
  const R r = L.r.v, T = L.T.v;
  const R th = theta_full(L);
  const R T0 = (R)kT0;
  const R Tp = T + T0;
  const R T2 = Tp + T0;
  const R P = M::sqrt(T * T2);               // rigidity [GV]
  const R inv_Tp = M::rcp(Tp);
  const R beta = P * inv_Tp;
  const R bP = beta * P;
  R s, c;
  phase_sincos(L.th, &s, &c);
  const R inv_s = M::rcp(s);
  const R cot = c * inv_s;
  const bool polarA = (th < (R)kThetaLo) || (th > (R)kThetaHi);   // Eq. 25 branch
  const bool nonpolarB = (th > (R)kThetaLo) && (th < (R)kThetaHi);
  const R inv_rh = R(1) / (R)kRh;
  const R delta = polarA ? (R)0.003f : k.delta0 * inv_s;
  const R deltarh = delta * inv_rh;
  const R deltarh2 = deltarh * deltarh;
  const R gamma = r * k.ov * s;                 // Eq. 24
  const R gamma2 = gamma * gamma;
  const R r2 = r * r;
  const R inv_r = M::rcp(r);
  const R rd2 = r2 * deltarh2;
  const R Cb = R(1) + gamma2 + rd2;            // Eq. 26
  const R inv_Cb = M::rcp(Cb);
  const R sqCb = M::sqrt(Cb);
  const R isqCb = M::rcp(sqCb);
  const R inv_Cb15 = inv_Cb * isqCb;
  const R inv_Cb25 = inv_Cb15 * inv_Cb;
  const R r2isq = r2 * isqCb;
  const R Pc = (P < (R)0.1f) ? (R)0.1f : P;
  const R Kpar = k.kpar_c * beta * Pc * r2isq;                  // Eq. 32
  const R Kper = k.ratio * Kpar;                                // Eq. 33
  const R dKC = (Kpar - Kper) * inv_Cb;
  const R Krr = Kper + dKC;                                     // Eq. 27
  const R Ktt = Kper + rd2 * dKC;                               // Eq. 28
  const R Krt = deltarh * r * dKC;                              // Eq. 29
  // Eq. 16-18 with sqrt(dt): B11 = sqrt(2 Kper (Ktt + dKC) / Ktt), B12 = Krt sqrt(2 / Ktt),
  // B22 = sqrt(2 Ktt) / r
  const R w = M::sqrt(R(2) * k.dt * M::rcp(Ktt));
  const R noise_r = w * (n1 * M::sqrt(Kper * (Ktt + dKC)) + n2 * Krt);
  const R noise_th = n4 * Ktt * w * inv_r;
  const R kd = k.kd_c * bP;                                     // K0 beta P / (3 * 5/3.4)
  const R rkd = k.ratio * kd;
  const R okdC25 = k.one_m_ratio * kd * inv_Cb25;
  const R tr = R(2) * r;
  const R r2COmega = tr * r2 * (k.ov2 * s * s + deltarh2);     // r^2 COmega, Eq. 34
  const R trCb = tr * Cb;
  const R dKrr = rkd * (trCb - R(0.5) * r2COmega) * inv_Cb15    // Eq. 36
               + okdC25 * (trCb - R(1.5) * r2COmega);           // Eq. 35
  const R CKtt0 = s * c * k.ov2 * r2;                           // Eq. 37
  const R dKrtr = okdC25 * deltarh * r2;                        // Eq. 43
  R dKtt_r2, dKrtt_r;                                           // dKtt / r^2, dKrtt / r
  if (nonpolarB) {
    dKtt_r2 = -CKtt0 * (rkd * inv_Cb15 + R(9) * (R)kC53 * okdC25 * rd2);   // Eq. 38-42
    dKrtt_r = R(-3) * dKrtr * gamma2 * cot;                               // Eq. 44
  } else {
    const R inv_s2 = inv_s * inv_s;
    const R cot_s2 = cot * inv_s2;                              // c / s^3
    const R CKtt = CKtt0 - r2 * k.d0rh2 * cot_s2;
    dKtt_r2 = -rkd * CKtt * inv_Cb15
            - k.one_m_ratio * kd * r2 * k.d0rh2 * (R(2) * cot_s2 * inv_Cb15 + R(3) * CKtt * inv_s2 * inv_Cb25);
    dKrtt_r = -okdC25 * r2 * (k.delta0 * inv_rh) * cot * inv_s * (R(1) - R(2) * rd2 + R(4) * gamma2);
  }
  // Wavy current sheet drifts, Kappl 2016 Eq. 26 and 32-37.
  // xarg = alphaM + 2 pi / 180 * Larmor / r, Larmor = 0.0225 P r^2 / (A sqrt(Cb))
  const R xarg = k.alphaM + (R)(2.0 * (double)kPi / 180.0 * 0.0225 / (double)kA) * P * (r * isqCb);
  const R q = (R)kPi * M::rcp(M::sin(xarg)) - R(1);
  const R alphaH = M::acos(M::rcp(q));
  // tan(acos(1 / q)) = sqrt(1 - 1/q^2) q = sign(q) sqrt(q^2 - 1): q < 0 where the
  // Larmor term carries xarg past pi (high rigidity near the poles)
  const R tanH = M::copysign(M::sqrt(q * q - R(1)), q);
  const R inv_alphaH = M::rcp(alphaH);
  const R arg = (R(1) + (R)(-2.0 / (double)kPi) * th) * tanH;      // pi of the reference's FP32 constant
  const R f = M::atan(arg) * inv_alphaH;
  const R fprime = (R)(-2.0 / (double)kPi) * tanH * inv_alphaH * M::rcp(R(1) + arg * arg);
  const R H = k.drift1 * bP * r * gamma * inv_Cb;              // drift1 P beta r gamma / Cb
  const R dc = R(2) * H * f * inv_Cb;                          // drift2 P beta r gamma f / Cb^2
  const R DriftR = dc * cot;
  const R DriftTheta = -dc * (R(2) + gamma2);
  const R DriftSheetR = H * fprime;
  // Eq. 21-22 plus the drifts
  const R det_r = (-k.V + dKrr + DriftR + DriftSheetR + dKrtt_r)
                + inv_r * (R(2) * Krr + Krt * cot);
  const R det_th = dKrtr + dKtt_r2 + inv_r * (R(2) * Krt + DriftTheta + Ktt * cot * inv_r);
  const R dr = det_r * k.dt + noise_r;
  const R dth = det_th * k.dt + noise_th;
  const R dT = -k.adv * bP * inv_r;                                    // Eq. 23
  L.r.add(dr);
  theta_update(L, dth);
  L.T.add(-dT);
  const bool rneg = L.r.v < R(0);                // reflect r < 0 (a select, not a branch)
  L.r.v = rneg ? -L.r.v : L.r.v;
  L.r.c = rneg ? -L.r.c : L.r.c;
  // NaN or r == 100 end the reference loop
  return (L.r.v > R(100)) ? kRecordAndStop : ((L.r.v < R(100)) ? kContinue : kStop);
}

// ---------------------------------------------------------------------------
// 2D SolarProp-like: SolarPropLikeModel.cu:95-247 (Kappl 2016 Eq. 13-18, 26,
// 32-37, 42-44).
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ int step_solarprop(Lane<R> &L, const Consts<R> &k, R z0, R z1) {
  // The same equations with shared factors, as in the 2D Geliosphere step:
  // beta P, r^2 / sqrt(1 + gamma^2), the drift prefactor P beta r gamma / (1 + gamma^2);
  // Eq. 44: 2 r sqrt(g1) - r^2 tmp / (2 sqrt(g1)) = (2 r g1 - r^2 tmp / 2) / sqrt(g1) (and
  // the g1^1.5 form likewise); Eq. 18: T (T + 2 T0) / (T + T0) = P beta; dt and 1 / r applied
  // once to the summed terms of dr and dtheta.
  using M = Math<R>;
  const R r = L.r.v, T = L.T.v;
  const R th = theta_full(L);
  const R T0 = (R)kT0;
  R s, c;
  phase_sincos(L.th, &s, &c);
  const R inv_s = M::rcp(s);
  const R cot = c * inv_s;
  const R gamma = r * k.ov * s;
  const R gamma2 = gamma * gamma;
  const R Tp = T + T0;
  const R P = M::sqrt(T * (Tp + T0));
  const R beta = P * M::rcp(Tp);
  const R bP = beta * P;
  const R g1 = R(1) + gamma2;
  const R inv_g1 = M::rcp(g1);
  const R sq1 = M::sqrt(g1);
  const R isq1 = M::rcp(sq1);
  const R inv_g1_15 = inv_g1 * isq1;
  const R inv_g1_25 = inv_g1_15 * inv_g1;
  const R r2 = r * r;
  const R inv_r = M::rcp(r);
  const R r2isq = r2 * isq1;
  const R tr = R(2) * r;
  const R r2tmp = tr * r2 * k.ov2 * s * s;                                      // r^2 tmp, Eq. 44
  const R trg1 = tr * g1;
  const R kbr = k.K0 * bP * (R)(5.0 / (3.0 * (double)3.4f));                   // K0 beta P 5 / (3 * 3.4)
  const R dKrr = kbr * (k.ratio * (trg1 - R(0.5) * r2tmp) * inv_g1_15
                        + k.one_m_ratio * (trg1 - R(1.5) * r2tmp) * inv_g1_25);
  const R Pc = (P < (R)0.1f) ? (R)0.1f : P;
  const R Kpar = k.kpar_c * beta * Pc * r2isq;                                  // Eq. 42
  const R Kper = k.ratio * Kpar;                                                // Eq. 43
  const R Krr = Kper + (Kpar - Kper) * inv_g1;                                  // Eq. 14
  const R Ktt = Kper;                                                           // Eq. 15
  const R dt = k.dt;
  // Wavy current sheet drifts (Eq. 26, 32-37), as in the 2D Geliosphere step
  const R xarg = k.alphaM + (R)(2.0 * (double)kPi / 180.0 * 0.0225 / (double)kA) * P * (r * isq1);
  const R q = (R)kPi * M::rcp(M::sin(xarg)) - R(1);
  const R alphaH = M::acos(M::rcp(q));
  const R tanH = M::copysign(M::sqrt(q * q - R(1)), q);                      // tan(acos(1 / q))
  const R inv_alphaH = M::rcp(alphaH);
  const R arg = (R(1) + (R)(-2.0 / (double)kPi) * th) * tanH;
  const R f = M::atan(arg) * inv_alphaH;
  const R fprime = (R)(-2.0 / (double)kPi) * tanH * inv_alphaH * M::rcp(R(1) + arg * arg);
  const R H = bP * r * gamma * inv_g1;                                          // P beta r gamma / g1
  const R D2 = H * f * inv_g1;
  const R DriftR = k.drift2 * D2 * cot;                                         // Eq. 35
  const R DriftSheetR = k.drift1 * H * fprime;                                  // Eq. 37
  const R DriftTheta = k.dtheta_sp * D2 * (R(2) + gamma2);                      // Eq. 36
  // Eq. 16-18
  const R dr = (-k.V + dKrr + DriftR + DriftSheetR + R(2) * Krr * inv_r) * dt
             + z0 * M::sqrt(R(2) * Krr * dt);
  const R dth = dt * inv_r * (Ktt * cot * inv_r * inv_g1 + DriftTheta)
              + z1 * M::sqrt(R(2) * Ktt * dt) * inv_r;
  const R dT = -k.adv * bP * inv_r;
  L.r.add(dr);
  theta_update(L, dth);
  L.T.add(-dT);
  const bool rneg = L.r.v < R(0);
  L.r.v = rneg ? -L.r.v : L.r.v;
  L.r.c = rneg ? -L.r.c : L.r.c;
  return (L.r.v > R(100)) ? kRecordAndStop : ((L.r.v < R(100)) ? kContinue : kStop);
}

// ---------------------------------------------------------------------------
// 1D B-p: OneDimensionBpModel.cu:69-140 (Eq. 5-7, 12-14).  V < 0.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ int step_bp(Lane<R> &L, const Consts<R> &k, R z) {
  using M = Math<R>;
  const R r = L.r.v;
  const R T0 = (R)kT0;
  // beta of the current T from the rigidity Pt that T was computed from and
  // q = 1 / sqrt(Pt^2 + T0^2) = 1 / (T + T0), both carried from the previous
  // step: sqrt(T (T + 2 T0)) / (T + T0) = Pt q in exact arithmetic.  After an
  // undone step T, Pt and q keep the rejected values, as T does in the
  // reference; the rigidity of Eq. 7 and 14 is the (restored) P.
  const R beta0 = L.Pt * L.q;
  const R Rig = L.P.v;
  const Acc<R> Psave = L.P;
  const Acc<R> rsave = L.r;
  const R inv_r = M::rcp(r);
  L.P.add(-k.adv * Rig * inv_r);                        // Eq. 14
  const R Kdiff = k.K0 * beta0 * Rig;                   // Eq. 7
  const R dr = (k.V + R(2) * Kdiff * inv_r) * k.dt + z * M::sqrt(R(2) * Kdiff * k.dt);   // Eq. 13
  L.r.add(dr);
  const R Pn = L.P.v;
  const R xn = Pn * Pn + T0 * T0;
  const R qn = M::rsqrt(xn);
  const R Tn = Pn * Pn * M::rcp(xn * qn + T0);          // P^2 / (sqrt(P^2 + T0^2) + T0)
  L.T.set(Tn);
  L.Pt = Pn;
  L.q = qn;
  const R beta = Pn * qn;                               // beta of Tn
  const R rn = L.r.v;
  // The rare events as selects, not branches; Tn < 200 GeV is tested as
  // Pn^2 < 200 (200 + 2 T0).
  const bool window = beta > (R)0.01f && Pn * Pn < (R)(200.0 * (200.0 + 2.0 * (double)kT0));
  const bool exits = window && rn > R(100) && (rn - dr) < R(100);
  const bool slow = !window && beta < (R)0.01f;
  const bool undo = rn < (R)0.3f && !exits && !slow;    // reflecting inner boundary: undo r and p
  L.r.v = undo ? rsave.v : L.r.v;
  L.r.c = undo ? rsave.c : L.r.c;
  L.P.v = undo ? Psave.v : L.P.v;
  L.P.c = undo ? Psave.c : L.P.c;
  return exits ? kRecordAndStop : ((slow || !(L.r.v < (R)100.0002f)) ? kStop : kContinue);
}

// ---------------------------------------------------------------------------
// 1D F-p: OneDimensionFpModel.cu:73-141 (Eq. 5-11).  Records every 1 AU crossing.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ int step_fp(Lane<R> &L, const Consts<R> &k, R z) {
  using M = Math<R>;
  const R r = L.r.v;
  const R T0 = (R)kT0;
  // Rigidity and beta of the current T from the momentum Pt that T was
  // computed from and q = 1 / sqrt(Pt^2 + T0^2) = 1 / (T + T0), both carried
  // from the previous step: sqrt(T (T + 2 T0)) = Pt and Pt / (T + T0) = Pt q
  // in exact arithmetic.  This takes two square roots and a reciprocal off
  // the step's dependent chain; an F-p run is bounded by the latency of its
  // longest trajectory.
  const R Pt = L.Pt, q = L.q;
  const R beta = Pt * q;
  const R inv_r = M::rcp(r);
  L.sumac.add(R(2) * k.adv * inv_r);                    // Eq. 11: 4 V dt / (3 r)
  const Acc<R> Psave = L.P;
  const Acc<R> rsave = L.r;
  L.P.add(-k.adv * L.P.v * inv_r);                      // Eq. 10
  const R Kdiff = k.K0 * beta * Pt;                     // Eq. 7
  // Eq. 9; sqrt(2 Kdiff dt) = Pt sqrt(2 K0 dt) sqrt(q)
  const R dr = (k.V + R(2) * Kdiff * inv_r) * k.dt + z * (Pt * k.sq2K0dt * M::sqrt(q));
  L.r.add(dr);
  const R Pn = L.P.v;
  const R Pn2 = Pn * Pn;
  const R xn = Pn2 + T0 * T0;
  const R qn = M::rsqrt(xn);
  const R Tn = Pn2 * M::rcp(xn * qn + T0);              // P^2 / (sqrt(P^2 + T0^2) + T0)
  L.T.set(Tn);
  L.Pt = Pn;                     // T keeps the rejected step's value if the step is undone below
  L.q = qn;
  const R rn = L.r.v;
  // The rare events as selects, not branches (a lone trajectory's chain is
  // latency-bound and its branches stall it).  Tn < 100 GeV is tested as
  // Pn^2 < 100 (100 + 2 T0), so the test does not wait for the reciprocal of Tn.
  const bool window = beta > (R)0.01f && Pn2 < (R)(100.0 * (100.0 + 2.0 * (double)kT0));
  const bool slow = !window && beta < (R)0.01f;                 // stop, the step kept
  const bool cross = window && (rn - R(1)) / ((rn - dr) - R(1)) < R(0);
  L.rrec = cross ? (float)rn : L.rrec;   // the record keeps the crossing's r even if the step is undone
  const bool undo = !slow && rn < (R)0.1f;                      // undo r and p (T keeps the rejected value)
  L.r.v = undo ? rsave.v : L.r.v;
  L.r.c = undo ? rsave.c : L.r.c;
  L.P.v = undo ? Psave.v : L.P.v;
  L.P.c = undo ? Psave.c : L.P.c;
  const bool out = !(L.r.v < (R)100.0002f);
  const int ended = cross ? kRecordAndStop : kStop;
  const int going = cross ? kRecordAndContinue : kContinue;
  return slow ? kStop : (out ? ended : going);
}

}  // namespace gelio
