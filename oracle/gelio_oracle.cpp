// gelio_oracle.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// CPU (FP64) restatement of the reference's SDE hot path, used only by the
// tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
// checker.  Nothing in geliosphere_gb300/ links or calls this library.
//
// Two flavours, both written from the reference sources (paths relative to
// the reference project):
//
// * "cpu" flavour: the reference CPU models' per-thread loops, literally,
//   including their std::mt19937 + std::normal_distribution<float> random
//   stream (libstdc++), their constants (Constants.hpp:14-239) and quirks
//   (sqrtf on a double beta, the injection-id repetition per energy loop).
//   Seeded like the reference, it reproduces the reference CPU models'
//   output records, which pins this restatement to the reference itself:
//     GeliosphereCpuModel.cpp:55-409, SolarPropLikeCpuModel.cpp:55-258,
//     OneDimensionBpCpuModel.cpp:54-143, OneDimensionFpCpuModel.cpp:53-155.
//
// * "gpu" flavour: the reference GPU kernels' semantics in FP64, with the
//   FP32 constant values of CosmicConstants.cu:14-41, driven by the engine's
//   Philox4x32-10 stream (Salmon et al. SC'11; implemented again here) and
//   its normal-to-term mapping.  Used to replay trajectories and check the
//   CUDA kernels:
//     GeliosphereModel.cu:61-392, SolarPropLikeModel.cu:78-249,
//     OneDimensionBpModel.cu:54-142, OneDimensionFpModel.cu:59-143,
//     CosmicUtils.cu:17-40.
//
// * evaluators: TwoDimensionBpResults.cpp:13-106, OneDimensionBpResults.cpp:
//   13-112, OneDimensionFpResults.cpp:13-113 on parsed log.dat rows.
//
// Parity anchor: the reference has no tests or golden vectors; the "cpu"
// flavour is pinned against the reference CPU models and evaluators
// compiled from source (oracle/ref_harness.cpp), whose outputs are committed
// under tests/golden/.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <thread>
#include <atomic>
#include <vector>
#include <chrono>

#include "../include/gelio.h"

namespace {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// ---------------------------------------------------------------------------
void philox(const uint32_t in[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t x0 = in[0], x1 = in[1], x2 = in[2], x3 = in[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int i = 0; i < 10; ++i) {
    const uint64_t a = (uint64_t)0xD2511F53u * x0;
    const uint64_t b = (uint64_t)0xCD9E8D57u * x2;
    const uint32_t y0 = (uint32_t)(b >> 32) ^ x1 ^ k0;
    const uint32_t y1 = (uint32_t)b;
    const uint32_t y2 = (uint32_t)(a >> 32) ^ x3 ^ k1;
    const uint32_t y3 = (uint32_t)a;
    x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

double unit24(uint32_t x) {   // the engine's uniform (2 (x >> 9) + 1) 2^-24, exact
  return (double)(2u * (x >> 9) + 1u) * (1.0 / 16777216.0);
}

// The engine's four normals for counter word `ctr0` of a trajectory.
void philox_normals(uint32_t ctr0, uint32_t stream, uint64_t pid, const uint32_t key[2], double z[4]) {
  const uint32_t c[4] = {ctr0, stream, (uint32_t)pid, (uint32_t)(pid >> 32)};
  uint32_t o[4];
  philox(c, key, o);
  const double pi = 3.14159265358979323846;
  const double ra = std::sqrt(-2.0 * std::log(unit24(o[0])));
  const double rb = std::sqrt(-2.0 * std::log(unit24(o[2])));
  z[0] = ra * std::cos(2.0 * pi * unit24(o[1]));
  z[1] = ra * std::sin(2.0 * pi * unit24(o[1]));
  z[2] = rb * std::cos(2.0 * pi * unit24(o[3]));
  z[3] = rb * std::sin(2.0 * pi * unit24(o[3]));
}

// ---------------------------------------------------------------------------
// GPU-flavour constants: the FP32 values of CosmicConstants.cu:14-41.
// ---------------------------------------------------------------------------
struct GpuK {
  double Pi = (double)3.141592654f;
  double T0 = (double)(float)(1.67261e-27 * 2.99793e8 * 2.99793e8 / (1.60219e-19 * 1e9));
  double omega = (double)2.866e-6f;
  double A = (double)3.4f;
  double konvF = (double)(9.0e-5f / 2.0f);
  double rh = (double)0.0046367333333333f;
  double thlo = (double)(1.7f * 3.141592654f / 180.0f);
  double thhi = (double)(178.3f * 3.141592654f / 180.0f);
  double c53 = (double)(5.0f / 3.4f);
  double dthc = (double)(-1.0f * 1.0f * (9.0e-5f / 2.0f) * (2.0f / (3.0f * 3.4f)));
  double twoPi = (double)(2.0f * 3.141592654f);
};

// Injection energies of the engine (FP32 results).
float inj_reference_uniform(uint64_t s, float injection_max) {   // CosmicUtils.cu:17-34
  const float mq = injection_max * 10000.0f;
  const uint64_t m = (uint64_t)mq;
  if ((float)s > mq && m > 0) s -= (s / m) * m;
  const uint64_t mod = (s >= 10000) ? s / 10000 : 0;
  const float frac = (float)(s - mod * 10000 + 1) / 10000.0f;
  return (float)mod + frac;
}

float injection(const gelio_sim_params &p, uint64_t pid) {
  switch (p.injection) {
    case GELIO_INJ_REFERENCE_UNIFORM: return inj_reference_uniform(pid, p.injection_max);
    case GELIO_INJ_SOLARPROP_GRID: return (float)(0.01 * std::pow(1.5, (double)(pid % 30)));
    case GELIO_INJ_LOG_GRID: {
      const int np = p.inj_points;
      const uint64_t k = pid % (uint64_t)np;
      const double f = (np > 1) ? (double)k / (double)(np - 1) : 0.0;
      const double lmin = std::log((double)p.inj_min), lmax = std::log((double)p.inj_max);
      return (float)std::exp(lmin + f * (lmax - lmin));
    }
    case GELIO_INJ_LOG_UNIFORM: {
      const uint32_t key[2] = {(uint32_t)p.seed, (uint32_t)(p.seed >> 32)};
      const uint32_t c[4] = {0u, 1u, (uint32_t)pid, (uint32_t)(pid >> 32)};
      uint32_t o[4];
      philox(c, key, o);
      const double u = ((double)o[0] + 0.5) * 2.3283064365386963e-10;
      const double lmin = std::log((double)p.inj_min), lmax = std::log((double)p.inj_max);
      return (float)std::exp(lmin + u * (lmax - lmin));
    }
    default: {
      const double step = ((double)p.injection_max - 0.0001) / 10000.0;
      return (float)(0.0001 + (double)(pid % 10000) * step);
    }
  }
}

// Rounding-noise control: the relative perturbation (1 + eps s), s = +-1
// drawn by a splitmix64 hash of (particle, step, variable).  Applied to r,
// theta and T after every step of a 2D replay (noise_on_increments = 0) it
// stands for one rounding of each state variable per step at relative
// precision eps (an uncompensated state, as in the FP64 kernels); applied to
// the increments dr, dtheta, dT instead (noise_on_increments = 1) it stands
// for increments computed at relative precision eps added to a compensated
// state (the FP32 kernels).  With eps = 0 the replay is the exact
// restatement.  Test infrastructure only:
// it measures how fast two replays that differ at rounding level part
// (the 2D maps are chaotic near the poles and near r = 0).
double noise_factor(double eps, uint64_t pid, uint32_t step, uint32_t var) {
  if (eps == 0.0) return 1.0;
  uint64_t z = pid * 0x9E3779B97F4A7C15ull + ((uint64_t)step << 2) + var + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (z & 1ull) ? 1.0 + eps : 1.0 - eps;
}

// ---------------------------------------------------------------------------
// GPU flavour, one trajectory.  Literal FP64 restatement of the kernels.
// ---------------------------------------------------------------------------
struct Traj {
  int status = 1;
  uint32_t steps = 0;
  int nrec = 0;
  double Tinj = 0, T = 0, r = 0, aux = 0;
  double Trec = 0, rrec = 0, auxrec = 0;
};

void gpu_geliosphere(const gelio_sim_params &p, uint64_t pid, uint64_t max_steps, Traj &t, double eps = 0.0,
                     int noise_on_increments = 0) {
  const GpuK K;
  const uint32_t key[2] = {(uint32_t)p.seed, (uint32_t)(p.seed >> 32)};
  const double V = p.V, dt = p.dt, K0 = p.K0, ratio = p.ratio, delta0 = p.delta0;
  const double alphaM = p.tilt, polarity = p.polarity;
  const double Pi = K.Pi, T0 = K.T0, omega = K.omega, A = K.A, konvF = K.konvF, rh = K.rh;
  double r = p.r_injection, theta = p.theta_injection;
  double Tkin = injection(p, pid);
  t.Tinj = Tkin;
  double beta, Rig, COmega, dKtt, dr, Krr, Bfactor, Kpar, dKrr, Ktt, Kper, dTkin, gamma, gamma2, Cb, Cb2;
  double dtheta, Bfield, Larmor, alphaH, arg, f, fprime, DriftR, DriftTheta, DriftSheetR;
  double delta, deltarh, deltarh2, Krt, B11, B12, B22;
  double sin3, sin2, dKtt1, dKtt2, dKtt3, dKtt4, CKtt, dKrtr, dKrtt, dKper;
  uint32_t step = 0;
  double grp[12];      // the twelve normals of the current group of four steps
  while (r < 100.0) {
    if (step >= max_steps) { t.status = 2; break; }
    // group g = step / 4 draws counters 3g, 3g + 1, 3g + 2; step 4g + p
    // takes normals 3p .. 3p + 2 of the group
    if ((step & 3u) == 0u)
      for (uint32_t k = 0; k < 3; ++k) philox_normals(3u * (step >> 2) + k, 0u, pid, key, grp + 4 * k);
    const double *z = grp + 3 * (step & 3u);
    ++step;
    beta = std::sqrt(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
    Rig = std::sqrt(Tkin * (Tkin + (2.0 * T0)));
    if ((theta < K.thlo) || (theta > K.thhi)) delta = 0.003f;
    else delta = delta0 / std::sin(theta);
    deltarh = delta / rh;
    deltarh2 = deltarh * deltarh;
    gamma = (r * omega) * std::sin(theta) / V;
    gamma2 = gamma * gamma;
    Cb = 1.0 + gamma2 + (r * r * deltarh2);
    Cb2 = Cb * Cb;
    Bfactor = K.c53 * r * r / std::sqrt(Cb);
    if (Rig < (double)0.1f) Kpar = K0 * beta * (double)0.1f * Bfactor / 3.0;
    else Kpar = K0 * beta * Rig * Bfactor / 3.0;
    Kper = ratio * Kpar;
    Krr = Kper + ((Kpar - Kper) / Cb);
    Ktt = Kper + (r * r * deltarh2 * (Kpar - Kper) / Cb);
    Krt = deltarh * (Kpar - Kper) * r / Cb;
    // Eq. 16-20 with Kphph = 1, Krph = Ktph = 0
    const double B11Temp = (Krt * Krt) - (Krr * Ktt);
    B11 = std::sqrt(2.0 * B11Temp / (-Ktt));
    B12 = (-Krt) / (-Ktt) * std::sqrt(2.0 * Ktt);
    B22 = std::sqrt(2.0 * Ktt) / r;
    COmega = 2.0 * r * omega * omega * std::sin(theta) * std::sin(theta) / (V * V);
    COmega = COmega + (2.0 * r * deltarh2);
    dKper = ratio * K0 * beta * Rig * ((2.0 * r * std::sqrt(Cb)) - (r * r * COmega / (2.0 * std::sqrt(Cb)))) /
            (3.0 * K.c53 * Cb);
    dKrr = dKper + ((1.0 - ratio) * K0 * beta * Rig *
                    ((2.0 * r * std::pow(Cb, 1.5)) - (r * r * COmega * 3.0 * std::sqrt(Cb) / 2.0)) /
                    (3.0 * K.c53 * std::pow(Cb, 3.0)));
    if ((theta > K.thlo) && (theta < K.thhi)) {
      CKtt = std::sin(theta) * std::cos(theta) * (omega * omega * r * r / (V * V));
      dKtt1 = (-1.0 * ratio * K0 * beta * Rig * r * r * CKtt) / (3.0 * K.c53 * std::pow(Cb, 1.5));
      dKtt2 = (1.0 - ratio) * K0 * beta * Rig * r * r * r * r * deltarh2;
      dKtt4 = 3.0 * CKtt / std::pow(Cb, 2.5);
      dKtt = dKtt1 - (dKtt2 * dKtt4);
    } else {
      sin2 = std::sin(theta) * std::sin(theta);
      sin3 = std::sin(theta) * std::sin(theta) * std::sin(theta);
      CKtt = std::sin(theta) * std::cos(theta) * (omega * omega * r * r / (V * V));
      CKtt = CKtt - (r * r * delta0 * delta0 * std::cos(theta) / (rh * rh * sin3));
      dKtt1 = (-1.0 * ratio * K0 * beta * Rig * r * r * CKtt) / (3.0 * K.c53 * std::pow(Cb, 1.5));
      dKtt2 = (1.0 - ratio) * K0 * beta * Rig * r * r * r * r * delta0 * delta0 / (rh * rh);
      dKtt3 = -2.0 * (std::cos(theta) / sin3) / (3.0 * K.c53 * std::pow(Cb, 1.5));
      dKtt4 = 3.0 * (CKtt / sin2) / (3.0 * K.c53 * std::pow(Cb, 2.5));
      dKtt = dKtt1 + (dKtt2 * (dKtt3 - dKtt4));
    }
    dKrtr = (1.0 - ratio) * K0 * beta * Rig * deltarh * r * r / (3.0 * K.c53 * std::pow(Cb, 2.5));
    if ((theta > K.thlo) && (theta < K.thhi)) {
      dKrtt = (1.0 - ratio) * K0 * beta * Rig * r * r * r / (3.0 * K.c53 * rh * std::pow(Cb, 2.5));
      dKrtt = -1.0 * dKrtt * delta;
      dKrtt = dKrtt * 3.0 * gamma2 * std::cos(theta) / std::sin(theta);
    } else {
      dKrtt = (1.0 - ratio) * K0 * beta * Rig * r * r * r / (3.0 * K.c53 * rh * std::pow(Cb, 2.5));
      dKrtt = -1.0 * dKrtt * delta0 * std::cos(theta) / (std::sin(theta) * std::sin(theta));
      dKrtt = dKrtt * (1.0 - (2.0 * r * r * deltarh2) + (4.0 * gamma2));
    }
    dr = ((-1.0 * V) + (2.0 * Krr / r) + dKrr) * dt;
    dr = dr + (dKrtt * dt / r) + (Krt * std::cos(theta) * dt / (r * std::sin(theta)));
    dr = dr + (z[0] * B11 * std::sqrt(dt));
    dr = dr + (z[1] * B12 * std::sqrt(dt));
    dtheta = (Ktt * std::cos(theta)) / (r * r * std::sin(theta));
    dtheta = (dtheta * dt) + (dKtt * dt / (r * r));
    dtheta = dtheta + (dKrtr * dt) + (2.0 * Krt * dt / r);
    dtheta = dtheta + (z[2] * B22 * std::sqrt(dt));
    dTkin = -2.0 * V * ((Tkin + T0 + T0) / (Tkin + T0)) * Tkin * dt / (3.0 * r);
    Bfield = A * std::sqrt(Cb) / (r * r);
    Larmor = 0.0225 * Rig / Bfield;
    alphaH = Pi / std::sin(alphaM + (2.0 * Larmor * Pi / (r * 180.0)));
    alphaH = alphaH - 1.0;
    alphaH = 1.0 / alphaH;
    alphaH = std::acos(alphaH);
    arg = (1.0 - (2.0 * theta / Pi)) * std::tan(alphaH);
    f = std::atan(arg) / alphaH;
    DriftR = polarity * konvF * (2.0 / (3.0 * A)) * Rig * beta * r * std::cos(theta) * gamma * f / (Cb2 * std::sin(theta));
    DriftTheta = -1.0 * polarity * konvF * (2.0 / (3.0 * A)) * Rig * beta * r * gamma * (2.0 + (gamma * gamma)) * f / Cb2;
    fprime = 1.0 + (arg * arg);
    fprime = std::tan(alphaH) / fprime;
    fprime = -1.0 * fprime * 2.0 / (Pi * alphaH);
    DriftSheetR = polarity * konvF * (1.0 / (3.0 * A)) * Rig * beta * r * gamma * fprime / Cb;
    dr = dr + ((DriftR + DriftSheetR) * dt);
    dtheta = dtheta + (DriftTheta * dt / r);
    if (eps != 0.0 && noise_on_increments) {
      dr *= noise_factor(eps, pid, step, 0);
      dtheta *= noise_factor(eps, pid, step, 1);
      dTkin *= noise_factor(eps, pid, step, 2);
    }
    r = r + dr;
    theta = theta + dtheta;
    Tkin = Tkin - dTkin;
    if (eps != 0.0 && !noise_on_increments) {
      r *= noise_factor(eps, pid, step, 0);
      theta *= noise_factor(eps, pid, step, 1);
      Tkin *= noise_factor(eps, pid, step, 2);
    }
    if (theta < 0.0) theta = std::fabs(theta);
    if (theta > K.twoPi) theta = theta - K.twoPi;
    else if (theta > Pi) theta = K.twoPi - theta;
    if (r < 0.0) r = -1.0 * r;
    if (r > 100.0) {
      t.status = 0; t.nrec = 1; t.Trec = Tkin; t.rrec = r; t.auxrec = theta;
      break;
    }
  }
  t.steps = step; t.T = Tkin; t.r = r; t.aux = theta;
}

void gpu_solarprop(const gelio_sim_params &p, uint64_t pid, uint64_t max_steps, Traj &t, double eps = 0.0,
                   int noise_on_increments = 0) {
  const GpuK K;
  const uint32_t key[2] = {(uint32_t)p.seed, (uint32_t)(p.seed >> 32)};
  const double V = p.V, dt = p.dt, K0 = p.K0, ratio = p.ratio, alphaM = p.tilt, polarity = p.polarity;
  const double Pi = K.Pi, T0 = K.T0, omega = K.omega, A = K.A, konvF = K.konvF;
  const double dthc = (p.flags & GELIO_FLAG_SOLARPROP_THETA_DRIFT_POLARITY)
                          ? -1.0 * polarity * konvF * (2.0 / (3.0 * A)) : K.dthc;
  double r = p.r_injection, theta = p.theta_injection;
  double Tkin = injection(p, pid);
  t.Tinj = Tkin;
  uint32_t step = 0;
  double z[4] = {0, 0, 0, 0};
  while (r < 100.0) {
    if (step >= max_steps) { t.status = 2; break; }
    if ((step & 1u) == 0u) philox_normals(step >> 1, 0u, pid, key, z);
    const double g0 = z[(step & 1u) * 2], g1 = z[(step & 1u) * 2 + 1];
    ++step;
    const double sineTheta = std::sin(theta);
    const double gamma = (r * omega) * sineTheta / V;
    const double gamma2 = gamma * gamma;
    const double Rig = std::sqrt(Tkin * (Tkin + (2.0 * T0)));
    const double beta = std::sqrt(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
    const double dKrrTmp = 2.0 * r * omega * omega * sineTheta * sineTheta / (V * V);
    double dKrr = ratio * K0 * beta * Rig * ((2.0 * r * std::sqrt(1.0 + gamma2)) - (r * r * dKrrTmp / (2.0 * std::sqrt(1.0 + gamma2)))) / (1.0 + gamma2);
    dKrr = dKrr + ((1.0 - ratio) * K0 * beta * Rig * ((2.0 * r * std::pow(1.0 + gamma2, 1.5)) - (r * r * dKrrTmp * 3.0 * std::sqrt(1.0 + gamma2) / 2.0)) / std::pow(1.0 + gamma2, 3.0));
    dKrr = dKrr * 5.0 / (3.0 * (double)3.4f);      // SolarPropLikeModel.cu:120 (FP32 literal)
    const double Bfactor = K.c53 * (r * r) / std::sqrt(1.0 + gamma2);
    const double RigC = (Rig < (double)0.1f) ? (double)0.1f : Rig;
    const double Kpar = K0 * beta * RigC * Bfactor / 3.0;
    const double Kper = ratio * Kpar;
    const double Krr = Kper + ((Kpar - Kper) / (1.0 + gamma2));
    double dr = ((-1.0 * V) + (2.0 * Krr / r) + dKrr) * dt;
    dr += (g0 * std::sqrt(2.0 * Krr * dt));
    const double cosineTheta = std::cos(theta);
    const double Ktt = Kper;
    double dtheta = (Ktt * cosineTheta) / (r * r * sineTheta);
    dtheta = (dtheta * dt) / (1.0 + gamma2);
    dtheta = dtheta + ((g1 * std::sqrt(2.0 * Ktt * dt)) / r);
    double dTkin = -2.0 * V * ((Tkin + T0 + T0) / (Tkin + T0)) * Tkin * dt / (3.0 * r);
    const double Bfield = A * std::sqrt((1.0 + gamma2)) / (r * r);
    const double Larmor = 0.0225 * Rig / Bfield;
    double alphaH = Pi / std::sin(alphaM + (2.0 * Larmor * Pi / (r * 180.0)));
    alphaH = alphaH - 1.0;
    alphaH = 1.0 / alphaH;
    alphaH = std::acos(alphaH);
    const double arg = (1.0 - (2.0 * theta / Pi)) * std::tan(alphaH);
    const double f = std::atan(arg) / alphaH;
    double fprime = 1.0 + (arg * arg);
    fprime = std::tan(alphaH) / fprime;
    fprime = -1.0 * fprime * 2.0 / (Pi * alphaH);
    const double g12 = (1.0 + gamma2) * (1.0 + gamma2);
    const double DriftR = polarity * konvF * (2.0 / (3.0 * A)) * Rig * beta * r * cosineTheta * gamma * f / ((g12) * sineTheta);
    const double DriftSheetR = polarity * konvF * (1.0 / (3.0 * A)) * Rig * beta * r * gamma * fprime / (1.0 + gamma2);
    dr = dr + ((DriftR + DriftSheetR) * dt);
    const double DriftTheta = dthc * Rig * beta * r * gamma * (2.0 + (gamma2)) * f / (g12);
    dtheta += (DriftTheta * dt / r);
    if (eps != 0.0 && noise_on_increments) {
      dr *= noise_factor(eps, pid, step, 0);
      dtheta *= noise_factor(eps, pid, step, 1);
      dTkin *= noise_factor(eps, pid, step, 2);
    }
    r = r + dr;
    theta = theta + dtheta;
    Tkin = Tkin - dTkin;
    if (eps != 0.0 && !noise_on_increments) {
      r *= noise_factor(eps, pid, step, 0);
      theta *= noise_factor(eps, pid, step, 1);
      Tkin *= noise_factor(eps, pid, step, 2);
    }
    if (theta < 0.0) theta = std::fabs(theta);
    if (theta > K.twoPi) theta = theta - K.twoPi;
    else if (theta > Pi) theta = K.twoPi - theta;
    if (r < 0.0) r = -1.0 * r;
    if (r > 100.0) {
      t.status = 0; t.nrec = 1; t.Trec = Tkin; t.rrec = r; t.auxrec = theta;
      break;
    }
  }
  t.steps = step; t.T = Tkin; t.r = r; t.aux = theta;
}

// Kinetic energy [GeV] from momentum, as the GPU kernels' Eq. 6 "in J"
// (OneDimensionBpModel.cu:114) with p expressed as rigidity P [GV]:
// T = (sqrt(T0^2 q^2 1e18 + q^2 Rig^2) - T0 q 1e9) / (q 1e9), Rig = P 1e9.
double tkin_from_P(double P, double T0) {
  const double q = 1.60219e-19;
  const double RigV = P * 1e9;
  return (std::sqrt((T0 * T0 * q * q * 1e9 * 1e9) + (q * q * RigV * RigV)) - (T0 * q * 1e9)) / (q * 1e9);
}

void gpu_bp(const gelio_sim_params &p, uint64_t pid, uint64_t max_steps, Traj &t) {
  const GpuK K;
  const uint32_t key[2] = {(uint32_t)p.seed, (uint32_t)(p.seed >> 32)};
  const double V = -(double)p.V, dt = p.dt, K0 = p.K0, T0 = K.T0;
  double r = p.r_injection;
  double Tkin = injection(p, pid);
  t.Tinj = Tkin;
  double P = std::sqrt(Tkin * (Tkin + (2.0 * T0)));   // rigidity [GV] of pinj
  uint32_t step = 0;
  double z[4] = {0, 0, 0, 0};
  bool recorded = false;
  while (r < (double)100.0002f) {
    if (step >= max_steps) { t.status = 2; break; }
    if ((step & 3u) == 0u) philox_normals(step >> 2, 0u, pid, key, z);
    const double n = z[step & 3u];
    ++step;
    double beta = std::sqrt(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
    const double Rig = P;
    const double pp = P;
    P -= (2.0 * V * pp * dt / (3.0 * r));
    const double Kdiff = K0 * beta * Rig;
    const double dr = (V + (2.0 * Kdiff / r)) * dt + (n * std::sqrt(2.0 * Kdiff * dt));
    r += dr;
    Tkin = tkin_from_P(P, T0);
    beta = std::sqrt(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
    if (beta > (double)0.01f && Tkin < 200.0) {
      if ((r > 100.0) && ((r - dr) < 100.0)) {
        t.status = 0; t.nrec = 1; t.Trec = Tkin; t.rrec = r; t.auxrec = 0.0;
        recorded = true;
        break;
      }
    } else if (beta < (double)0.01f) {
      break;
    }
    if (r < (double)0.3f) {
      r -= dr;
      P = pp;
    }
  }
  (void)recorded;
  t.steps = step; t.T = Tkin; t.r = r; t.aux = 0.0;
}

void gpu_fp(const gelio_sim_params &p, uint64_t pid, uint64_t max_steps, Traj &t) {
  const GpuK K;
  const uint32_t key[2] = {(uint32_t)p.seed, (uint32_t)(p.seed >> 32)};
  const double V = p.V, dt = p.dt, K0 = p.K0, T0 = K.T0;
  double r = (double)100.0001f;
  double Tkin = injection(p, pid);
  t.Tinj = Tkin;
  double P = std::sqrt(Tkin * (Tkin + (2.0 * T0)));
  double sumac = 0.0;
  uint32_t step = 0;
  double z[4] = {0, 0, 0, 0};
  t.status = 1;
  while (r < (double)100.0002f) {
    if (step >= max_steps) { t.status = 2; break; }
    if ((step & 3u) == 0u) philox_normals(step >> 2, 0u, pid, key, z);
    const double n = z[step & 3u];
    ++step;
    const double beta = std::sqrt(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
    const double Rig = std::sqrt(Tkin * (Tkin + (2.0 * T0)));
    sumac += ((4.0 * V / (3.0 * r)) * dt);
    const double pp = P;
    P -= (2.0 * V * pp * dt / (3.0 * r));
    const double Kdiff = K0 * beta * Rig;
    const double dr = (V + (2.0 * Kdiff / r)) * dt + (n * std::sqrt(2.0 * Kdiff * dt));
    r += dr;
    Tkin = tkin_from_P(P, T0);
    if (beta > (double)0.01f && Tkin < 100.0) {
      if ((r - 1.0) / ((r - dr) - 1.0) < 0.0) {
        if (t.nrec == 0) { t.Trec = Tkin; t.rrec = r; t.auxrec = sumac; }
        ++t.nrec;
      }
    } else if (beta < (double)0.01f) {
      break;
    }
    if (r < (double)0.1f) {
      r -= dr;
      P = pp;
    }
  }
  if (t.status != 2) t.status = (t.nrec > 0) ? 0 : 1;
  t.steps = step; t.T = Tkin; t.r = r; t.aux = sumac;
}

// ---------------------------------------------------------------------------
// CPU flavour: the reference CPU models' simulation(threadNumber,
// availableThreads, iteration), with the reference's constants.
// ---------------------------------------------------------------------------
const double kM0 = 1.67261e-27, kQ = 1.60219e-19, kC = 2.99793e8;
const double kPiD = 3.1415926535897932384626433832795;
const double kT0 = kM0 * kC * kC / (kQ * 1e9);
const double kT0w = kM0 * kC * kC;
const double kOmegaD = 2.866e-6, kAD = 3.4, kKonvFD = 9.0e-5 / 2.0;
const double kRhD = 695510.0 / 150000000.0;
const double kSPbins[30] = {0.01, 0.015, 0.0225, 0.03375, 0.050625,
  0.0759375, 0.113906, 0.170859, 0.256289, 0.384434, 0.57665,
  0.864976, 1.29746, 1.9462, 2.91929, 4.37894, 6.56841, 9.85261,
  14.7789, 22.1684, 33.2526, 49.8789, 74.8183, 112.227, 168.341,
  252.512, 378.768, 568.151, 852.227, 1278.34};

double cpu_injection(unsigned long long id, double from, double to, int bins) {   // Constants.hpp:234-239
  const double step = (to - from) / bins;
  return from + ((id % bins) * step);
}

}  // namespace

// Resolved statics of the reference CPU models (Constants.hpp) for one run.
extern "C" struct gor_cpu_params {
  double V, dt, K0, ratio, delta0, alphaM, polarity, rInit, thetainj;
  int useUniformInjection;
  double uniformEnergyInjectionMaximum;
  // Not in the reference: an injection grid for the 2D models' block loop.
  // With inj_energies set, a block injects inj_per_point particles at each
  // of the inj_points energies (in place of 500 at each of the 30 SolarProp
  // energies); zero / null keeps the reference's injection.
  const float *inj_energies;
  int inj_points, inj_per_point;
};

namespace {

// Output row layout per model: the SimulationOutput members in order.
// 2D: Tkininj, Tkin, r, w, thetainj, theta (GeliosphereCpuModel.hpp:20-28)
// B-p: Tkin, Tkininj, r, w (pushed as {Tkin, Tkininj, r, w})
// F-p: pinj, p, r, w, sumac
struct RowSink {
  double *rows;
  int64_t cap, n;
  int ncol;
  void push(const double *v) {
    if (n < cap) std::memcpy(rows + n * ncol, v, sizeof(double) * ncol);
    ++n;
  }
};

void cpu_geliosphere(const gor_cpu_params &c, int threadNumber, unsigned availableThreads, int iteration,
                     std::mt19937 &generator, std::normal_distribution<float> &distribution, RowSink &out,
                     int64_t *steps_out) {
  const double V = c.V, dt = c.dt, K0 = c.K0, ratio = c.ratio, delta0 = c.delta0, alphaM = c.alphaM;
  const double polarity = c.polarity, Pi = kPiD, T0 = kT0, omega = kOmegaD, A = kAD, konvF = kKonvFD, rh = kRhD;
  double r, dr, theta, Kpar, Bfactor, COmega, Tkin, Tkininj, Rig, beta, alfa, Ktt, dKrr, dKper;
  double w, r2, gamma, gamma2, Cb, Cb2, Kper, Krr, dKtt, dKtt3, dKtt4, CKtt, Tkinw, p;
  double dtheta, dTkin, delta, deltarh, deltarh2, DriftR, DriftTheta, arg, alphaH, Larmor, Bfield, f, fprime, DriftSheetR;
  double Kphph, Krt, Krph, Ktph, B11Temp, B11, B12, B13, B22, B23, sin2, sin3, dKtt1, dKtt2, dKrtr, dKrtt;
  int64_t steps = 0;
  const int n_energy = c.inj_energies ? c.inj_points : 30, n_ppe = c.inj_energies ? c.inj_per_point : 500;
  for (int energy = 0; energy < n_energy; energy++) {
    for (int ppe = 0; ppe < n_ppe; ppe++) {
      Tkininj = c.inj_energies ? (double)c.inj_energies[energy]
                : (c.useUniformInjection)
                    ? cpu_injection(((availableThreads * iteration + threadNumber) * 500) + ppe, 0.0001, c.uniformEnergyInjectionMaximum, 10000)
                    : kSPbins[energy];
      Tkin = Tkininj;
      Tkinw = Tkin * 1e9 * kQ;
      Rig = std::sqrt(Tkinw * (Tkinw + (2.0 * kT0w))) / kQ;
      p = Rig * kQ / kC;
      w = (kM0 * kM0 * kC * kC * kC * kC) + (p * p * kC * kC);
      w = std::pow(w, -1.85) / p;
      w = w / 1e45;
      r = c.rInit;
      theta = c.thetainj;
      while (r < 100.0) {
        ++steps;
        beta = sqrtf(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
        Rig = std::sqrt(Tkin * (Tkin + (2.0 * T0)));
        r2 = r * r;
        if (theta < (1.7 * Pi / 180.) || theta > (178.3 * Pi / 180.0)) delta = 0.003;
        else delta = delta0 / std::sin(theta);
        deltarh = delta / rh;
        deltarh2 = deltarh * deltarh;
        gamma = (r * omega) * std::sin(theta) / V;
        gamma2 = gamma * gamma;
        Cb = 1.0 + gamma2 + (r2 * deltarh2);
        Cb2 = Cb * Cb;
        Bfactor = (5. / 3.4) * r2 / std::sqrt(Cb);
        if (Rig < 0.1) Kpar = K0 * beta * 0.1 * Bfactor / 3.0;
        else Kpar = K0 * beta * Rig * Bfactor / 3.0;
        Kper = ratio * Kpar;
        Krr = Kper + ((Kpar - Kper) / Cb);
        Ktt = Kper + (r2 * deltarh2 * (Kpar - Kper) / Cb);
        Kphph = 1.0;
        Krt = deltarh * (Kpar - Kper) * r / Cb;
        Krph = 0.0;
        Ktph = 0.0;
        B11Temp = (Kphph * Krt * Krt) - (2.0 * Krph * Krt * Ktph) + (Krr * Ktph * Ktph) + (Ktt * Krph * Krph) - (Krr * Ktt * Kphph);
        B11 = 2.0 * B11Temp / ((Ktph * Ktph) - (Ktt * Kphph));
        B11 = std::sqrt(B11);
        B12 = ((Krph * Ktph) - (Krt * Kphph)) / ((Ktph * Ktph) - (Ktt * Kphph));
        B12 = B12 * std::sqrt(2.0 * (Ktt - (Ktph * Ktph / Kphph)));
        B13 = std::sqrt(2.0) * Krph / std::sqrt(Kphph);
        B22 = Ktt - (Ktph * Ktph / Kphph);
        B22 = std::sqrt(2.0 * B22) / r;
        B23 = Ktph * std::sqrt(2.0 / Kphph) / r;
        COmega = 2.0 * r * omega * omega * std::sin(theta) * std::sin(theta) / (V * V);
        COmega = COmega + (2.0 * r * deltarh2);
        dKper = ratio * K0 * beta * Rig * ((2.0 * r * std::sqrt(Cb)) - (r2 * COmega / (2.0 * std::sqrt(Cb)))) / (3.0 * (5.0 / 3.4) * Cb);
        dKrr = dKper + ((1.0 - ratio) * K0 * beta * Rig * ((2.0 * r * std::pow(Cb, 1.5)) - (r2 * COmega * 3.0 * std::sqrt(Cb) / 2.0)) / (3.0 * (5.0 / 3.4) * std::pow(Cb, 3.0)));
        if ((theta > (1.7 * Pi / 180.)) && (theta < (178.3 * Pi / 180.0))) {
          CKtt = std::sin(theta) * std::cos(theta) * (omega * omega * r2 / (V * V));
          dKtt1 = (-1.0 * ratio * K0 * beta * Rig * r2 * CKtt) / (3.0 * (5.0 / 3.4) * std::pow(Cb, 1.5));
          dKtt2 = (1.0 - ratio) * K0 * beta * Rig * r2 * r2 * deltarh2;
          dKtt4 = 3.0 * CKtt / std::pow(Cb, 2.5);
          dKtt = dKtt1 - (dKtt2 * dKtt4);
        } else {
          sin2 = std::sin(theta) * std::sin(theta);
          sin3 = std::sin(theta) * std::sin(theta) * std::sin(theta);
          CKtt = std::sin(theta) * std::cos(theta) * (omega * omega * r2 / (V * V));
          CKtt = CKtt - (r2 * delta0 * delta0 * std::cos(theta) / (rh * rh * sin3));
          dKtt1 = (-1.0 * ratio * K0 * beta * Rig * r2 * CKtt) / (3.0 * (5.0 / 3.4) * std::pow(Cb, 1.5));
          dKtt2 = (1.0 - ratio) * K0 * beta * Rig * r2 * r2 * delta0 * delta0 / (rh * rh);
          dKtt3 = -2.0 * (std::cos(theta) / sin3) / (3.0 * (5.0 / 3.4) * std::pow(Cb, 1.5));
          dKtt4 = 3.0 * (CKtt / sin2) / (3.0 * (5.0 / 3.4) * std::pow(Cb, 2.5));
          dKtt = dKtt1 + (dKtt2 * (dKtt3 - dKtt4));
        }
        dKrtr = (1.0 - ratio) * K0 * beta * Rig * deltarh * r2 / (3.0 * (5.0 / 3.4) * std::pow(Cb, 2.5));
        if ((theta > (1.7 * Pi / 180.)) && (theta < (178.3 * Pi / 180.0))) {
          dKrtt = (1.0 - ratio) * K0 * beta * Rig * r2 * r / ((3.0 * (5.0 / 3.4) * rh * std::pow(Cb, 2.5)));
          dKrtt = -1.0 * dKrtt * delta;
          dKrtt = dKrtt * 3.0 * gamma2 * std::cos(theta) / std::sin(theta);
        } else {
          dKrtt = (1.0 - ratio) * K0 * beta * Rig * r2 * r / ((3.0 * (5.0 / 3.4) * rh * std::pow(Cb, 2.5)));
          dKrtt = -1.0 * dKrtt * delta0 * std::cos(theta) / (std::sin(theta) * std::sin(theta));
          dKrtt = dKrtt * (1.0 - (2.0 * r2 * deltarh2) + (4.0 * gamma2));
        }
        dr = ((-1.0 * V) + (2.0 * Krr / r) + dKrr) * dt;
        dr = dr + (dKrtt * dt / r) + (Krt * std::cos(theta) * dt / (r * std::sin(theta)));
        dr = dr + (distribution(generator) * B11 * std::sqrt(dt));
        dr = dr + (distribution(generator) * B12 * std::sqrt(dt));
        dr = dr + (distribution(generator) * B13 * std::sqrt(dt));
        dtheta = (Ktt * std::cos(theta)) / (r2 * std::sin(theta));
        dtheta = (dtheta * dt) + (dKtt * dt / r2);
        dtheta = dtheta + (dKrtr * dt) + (2.0 * Krt * dt / r);
        {
          const float n4 = distribution(generator);
          const float n5 = distribution(generator);
          dtheta = dtheta + (n4 * B22 * std::sqrt(dt)) + (n5 * B23 * std::sqrt(dt));
        }
        alfa = (Tkin + T0 + T0) / (Tkin + T0);
        dTkin = -2.0 * V * alfa * Tkin * dt / (3.0 * r);
        Bfield = A * std::sqrt(Cb) / (r * r);
        Larmor = 0.0225 * Rig / Bfield;
        alphaH = Pi / std::sin(alphaM + (2.0 * Larmor * Pi / (r * 180.0)));
        alphaH = alphaH - 1.0;
        alphaH = 1.0 / alphaH;
        alphaH = std::acos(alphaH);
        arg = (1. - (2. * theta / Pi)) * std::tan(alphaH);
        f = std::atan(arg) / alphaH;
        DriftR = polarity * konvF * (2.0 / (3.0 * A)) * Rig * beta * r * std::cos(theta) * gamma * f / (Cb2 * std::sin(theta));
        DriftTheta = -1.0 * polarity * konvF * (2.0 / (3.0 * A)) * Rig * beta * r * gamma * (2.0 + (gamma * gamma)) * f / Cb2;
        fprime = 1.0 + (arg * arg);
        fprime = std::tan(alphaH) / fprime;
        fprime = -1.0 * fprime * 2.0 / (Pi * alphaH);
        DriftSheetR = polarity * konvF * (1.0 / (3.0 * A)) * Rig * beta * r * gamma * fprime / Cb;
        dr = dr + ((DriftR + DriftSheetR) * dt);
        dtheta = dtheta + (DriftTheta * dt / r);
        r = r + dr;
        theta = theta + dtheta;
        Tkin = Tkin - dTkin;
        if (theta < 0.0) theta = std::fabs(theta);
        if (theta > 2.0 * Pi) theta = theta - (2.0 * Pi);
        else if (theta > Pi) theta = (2.0 * Pi) - theta;
        if (r < 0.0) r = -1.0 * r;
        if (r > 100.0) {
          const double row[6] = {Tkininj, Tkin, r, w, c.thetainj, theta};
          out.push(row);
          break;
        }
      }
    }
  }
  if (steps_out) *steps_out += steps;
}

void cpu_solarprop(const gor_cpu_params &c, int threadNumber, unsigned availableThreads, int iteration,
                   std::mt19937 &generator, std::normal_distribution<float> &distribution, RowSink &out,
                   int64_t *steps_out) {
  const double V = c.V, dt = c.dt, K0 = c.K0, ratio = c.ratio, alphaM = c.alphaM, polarity = c.polarity;
  const double Pi = kPiD, T0 = kT0, omega = kOmegaD, A = kAD, konvF = kKonvFD;
  double r, dr, theta, Kpar, Bfactor, dKrrTmp, Tkin, Tkininj, Rig, beta, alfa, Ktt, dKrr;
  double w, r2, gamma, gamma2, onePlusGamma, onePlusGamma2, Kper, Krr, Tkinw, p, dtheta, dTkin;
  double DriftR, DriftTheta, arg, alphaH, Larmor, Bfield, f, fprime, DriftSheetR;
  int64_t steps = 0;
  const int n_energy = c.inj_energies ? c.inj_points : 30, n_ppe = c.inj_energies ? c.inj_per_point : 500;
  for (int energy = 0; energy < n_energy; energy++) {
    for (int ppe = 0; ppe < n_ppe; ppe++) {
      Tkininj = c.inj_energies ? (double)c.inj_energies[energy]
                : (c.useUniformInjection)
                    ? cpu_injection(((availableThreads * iteration + threadNumber) * 500) + ppe, 0.0001, c.uniformEnergyInjectionMaximum, 10000)
                    : kSPbins[energy];
      Tkin = Tkininj;
      Tkinw = Tkin * 1e9 * kQ;
      Rig = std::sqrt(Tkinw * (Tkinw + (2.0 * kT0w))) / kQ;
      p = Rig * kQ / kC;
      w = (kM0 * kM0 * kC * kC * kC * kC) + (p * p * kC * kC);
      w = std::pow(w, -1.85) / p;
      w = w / 1e45;
      r = c.rInit;
      theta = c.thetainj;
      while (r < 100.0) {
        ++steps;
        beta = sqrtf(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
        Rig = std::sqrt(Tkin * (Tkin + (2.0 * T0)));
        r2 = r * r;
        gamma = (r * omega) * std::sin(theta) / V;
        gamma2 = gamma * gamma;
        onePlusGamma = 1.0 + gamma2;
        onePlusGamma2 = onePlusGamma * onePlusGamma;
        Bfactor = (5.0 / 3.4) * r2 / std::sqrt(onePlusGamma);
        if (Rig < 0.1) Kpar = K0 * beta * 0.1 * Bfactor / 3.0;
        else Kpar = K0 * beta * Rig * Bfactor / 3.0;
        Kper = ratio * Kpar;
        Krr = Kper + ((Kpar - Kper) / onePlusGamma);
        Ktt = Kper;
        dKrrTmp = 2.0 * r * omega * omega * std::sin(theta) * std::sin(theta) / (V * V);
        dKrr = ratio * K0 * beta * Rig * ((2.0 * r * std::sqrt(onePlusGamma)) - (r2 * dKrrTmp / (2.0 * std::sqrt(onePlusGamma)))) / onePlusGamma;
        dKrr = dKrr + ((1.0 - ratio) * K0 * beta * Rig * ((2.0 * r * std::pow(onePlusGamma, 1.5)) - (r2 * dKrrTmp * 3.0 * std::sqrt(onePlusGamma) / 2.0)) / std::pow(onePlusGamma, 3.0));
        dKrr = dKrr * 5.0 / (3.0 * 3.4);
        dr = ((-1.0 * V) + (2.0 * Krr / r) + dKrr) * dt;
        dr = dr + (distribution(generator) * std::sqrt(2.0 * Krr * dt));
        dtheta = (Ktt * std::cos(theta)) / (r2 * std::sin(theta));
        dtheta = dtheta * dt / onePlusGamma;
        dtheta = dtheta + ((distribution(generator) * std::sqrt(2.0 * Ktt * dt)) / r);
        alfa = (Tkin + T0 + T0) / (Tkin + T0);
        dTkin = -2.0 * V * alfa * Tkin * dt / (3.0 * r);
        Bfield = A * std::sqrt(onePlusGamma) / (r * r);
        Larmor = 0.0225 * Rig / Bfield;
        alphaH = Pi / std::sin(alphaM + (2.0 * Larmor * Pi / (r * 180.0)));
        alphaH = alphaH - 1.0;
        alphaH = 1.0 / alphaH;
        alphaH = std::acos(alphaH);
        arg = (1. - (2. * theta / Pi)) * std::tan(alphaH);
        f = std::atan(arg) / alphaH;
        DriftR = polarity * konvF * (2.0 / (3.0 * A)) * Rig * beta * r * std::cos(theta) * gamma * f / (onePlusGamma2 * std::sin(theta));
        DriftTheta = -1.0 * polarity * konvF * (2.0 / (3.0 * A)) * Rig * beta * r * gamma * (2.0 + (gamma * gamma)) * f / onePlusGamma2;
        fprime = 1.0 + (arg * arg);
        fprime = std::tan(alphaH) / fprime;
        fprime = -1.0 * fprime * 2.0 / (Pi * alphaH);
        DriftSheetR = polarity * konvF * (1.0 / (3.0 * A)) * Rig * beta * r * gamma * fprime / onePlusGamma;
        dr = dr + ((DriftR + DriftSheetR) * dt);
        dtheta = dtheta + (DriftTheta * dt / r);
        r = r + dr;
        theta = theta + dtheta;
        if (theta < 0.0) theta = std::fabs(theta);
        if (theta > 2.0 * Pi) theta = theta - (2.0 * Pi);
        else if (theta > Pi) theta = (2.0 * Pi) - theta;
        Tkin = Tkin - dTkin;
        if (r < 0.0) r = -1.0 * r;
        if (r > 100.0) {
          const double row[6] = {Tkininj, Tkin, r, w, c.thetainj, theta};
          out.push(row);
          break;
        }
      }
    }
  }
  if (steps_out) *steps_out += steps;
}

void cpu_bp(const gor_cpu_params &c, int threadNumber, unsigned availableThreads, int iteration,
            std::mt19937 &generator, std::normal_distribution<float> &distribution, RowSink &out,
            int64_t *steps_out) {
  const double V = c.V, dt = c.dt, K0 = c.K0, T0 = kT0;
  double r, dr, arnum, Tkin, Tkininj, Rig, beta, w, p, dp, pp, Kdiff;
  int64_t steps = 0;
  for (int energy = 0; energy < 101; energy++) {
    for (int ppe = 0; ppe < 250; ppe++) {
      Tkininj = cpu_injection(((availableThreads * iteration + threadNumber) * 250) + ppe, 0.0001, c.uniformEnergyInjectionMaximum, 10000);
      Tkin = Tkininj;
      Rig = std::sqrt(Tkin * (Tkin + (2.0 * T0)));
      p = Rig * 1e9 * kQ / kC;
      r = c.rInit;
      while (r < 100.0002) {
        ++steps;
        beta = sqrtf(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
        Rig = (p * kC / kQ) / 1e9;
        pp = p;
        dp = (2.0f * V * pp * dt / (3.0f * r));
        p -= dp;
        Kdiff = K0 * beta * Rig;
        arnum = distribution(generator);
        dr = (V + (2.0 * Kdiff / r)) * dt + (arnum * std::sqrt(2.0 * Kdiff * dt));
        r += dr;
        Rig = p * kC / kQ;
        Tkin = (std::sqrt((T0 * T0 * kQ * kQ * 1e9 * 1e9) + (kQ * kQ * Rig * Rig)) - (T0 * kQ * 1e9)) / (kQ * 1e9);
        beta = sqrtf(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
        if (beta > 0.01f && Tkin < 200.0f) {
          if ((r > 100.0f) && ((r - dr) < 100.0f)) {
            w = (kM0 * kM0 * kC * kC * kC * kC) + (p * p * kC * kC);
            w = (std::pow(w, -1.85) / p) / 1e45;
            const double row[4] = {Tkin, Tkininj, r, w};
            out.push(row);
            break;
          }
        } else if (beta < 0.01f) {
          break;
        }
        if (r < 0.3f) {
          r -= dr;
          p = pp;
        }
      }
    }
  }
  if (steps_out) *steps_out += steps;
}

void cpu_fp(const gor_cpu_params &c, int threadNumber, unsigned availableThreads, int iteration,
            std::mt19937 &generator, std::normal_distribution<float> &distribution, RowSink &out,
            int64_t *steps_out) {
  const double V = c.V, dt = c.dt, K0 = c.K0, T0 = kT0;
  double r, Kdiff, dr, arnum, Tkin, Tkininj, Rig, beta, w, Tkinw, p, rp, dp, pp, pinj, cfactor, sumac;
  int64_t steps = 0;
  for (int energy = 0; energy < 101; energy++) {
    for (int ppe = 0; ppe < 250; ppe++) {
      Tkininj = cpu_injection(((availableThreads * iteration + threadNumber) * 250) + ppe, 0.0001, c.uniformEnergyInjectionMaximum, 10000);
      Tkin = Tkininj;
      Tkinw = Tkin * 1e9 * kQ;
      Rig = std::sqrt(Tkinw * (Tkinw + (2.0 * kT0w))) / kQ;
      p = Rig * kQ / kC;
      pinj = p;
      w = (kM0 * kM0 * kC * kC * kC * kC) + (p * p * kC * kC);
      w = std::pow(w, -1.85) / p;
      w = w / 1e45;
      sumac = 0.0;
      r = 100.0001;
      while (r < 100.0002) {
        ++steps;
        beta = std::sqrt(Tkin * (Tkin + T0 + T0)) / (Tkin + T0);
        Rig = std::sqrt(Tkin * (Tkin + (2.0 * T0)));
        Kdiff = K0 * beta * Rig;
        arnum = distribution(generator);
        dr = (V + (2.0 * Kdiff / r)) * dt;
        dr = dr + (arnum * std::sqrt(2.0 * Kdiff * dt));
        dp = 2.0 * V * p * dt / (3.0 * r);
        cfactor = 4.0 * V / (3.0 * r);
        sumac = sumac + (cfactor * dt);
        rp = r;
        pp = p;
        r = r + dr;
        p = p - dp;
        Rig = p * kC / kQ;
        Tkin = std::sqrt((T0 * T0 * kQ * kQ * 1e9 * 1e9) + (kQ * kQ * Rig * Rig)) - (T0 * kQ * 1e9);
        Tkin = Tkin / (kQ * 1e9);
        if ((beta > 0.01) & (Tkin < 100.0)) {
          if ((r - 1.0) / ((r - dr) - 1.0) < 0.0) {
            const double row[5] = {pinj, p, r, w, sumac};
            out.push(row);
          }
        }
        if (beta < 0.01) break;
        if (r < 0.1) {
          r = rp;
          p = pp;
        }
      }
    }
  }
  if (steps_out) *steps_out += steps;
}

typedef void (*CpuModelFn)(const gor_cpu_params &, int, unsigned, int, std::mt19937 &,
                           std::normal_distribution<float> &, RowSink &, int64_t *);

CpuModelFn cpu_fn(int model) {
  switch (model) {
    case GELIO_MODEL_1D_FP: return cpu_fp;
    case GELIO_MODEL_1D_BP: return cpu_bp;
    case GELIO_MODEL_2D_SOLARPROP: return cpu_solarprop;
    default: return cpu_geliosphere;
  }
}

int cpu_cols(int model) {
  return (model >= GELIO_MODEL_2D_SOLARPROP) ? 6 : (model == GELIO_MODEL_1D_BP ? 4 : 5);
}

// ---------------------------------------------------------------------------
// Evaluators (ResultConstants.hpp; *Results.cpp), on parsed log rows.
// ---------------------------------------------------------------------------
const double kSPbinsR[32] = {0, 0.01, 0.015, 0.0225, 0.03375, 0.050625,
  0.0759375, 0.113906, 0.170859, 0.256289, 0.384434, 0.57665,
  0.864976, 1.29746, 1.9462, 2.91929, 4.37894, 6.56841, 9.85261,
  14.7789, 22.1684, 33.2526, 49.8789, 74.8183, 112.227, 168.341,
  252.512, 378.768, 568.151, 852.227, 1278.34, 0};
const double kUly[4] = {0, 0.125, 0.250, 2.0};
const double kAms[72] = {4.924000e-01, 6.207000e-01, 7.637000e-01, 9.252000e-01, 1.105000e+00,
  1.303000e+00, 1.523000e+00, 1.765000e+00, 2.034000e+00, 2.329000e+00, 2.652000e+00, 3.005000e+00,
  3.390000e+00, 3.810000e+00, 4.272000e+00, 4.774000e+00, 5.317000e+00, 5.906000e+00, 6.546000e+00,
  7.236000e+00, 7.981000e+00, 8.787000e+00, 9.653000e+00, 1.060000e+01, 1.160000e+01, 1.264000e+01,
  1.379000e+01, 1.504000e+01, 1.639000e+01, 1.784000e+01, 1.938000e+01, 2.103000e+01, 2.283000e+01,
  2.478000e+01, 2.683000e+01, 2.903000e+01, 3.138000e+01, 3.387000e+01, 3.657000e+01, 3.947000e+01,
  4.257000e+01, 4.587000e+01, 4.942000e+01, 5.322000e+01, 5.727000e+01, 6.162000e+01, 6.632000e+01,
  7.137000e+01, 7.677000e+01, 8.257000e+01, 8.882000e+01, 9.557000e+01, 1.031000e+02, 1.111000e+02,
  1.196000e+02, 1.291000e+02, 1.401000e+02, 1.526000e+02, 1.666000e+02, 1.826000e+02, 2.006000e+02,
  2.211000e+02, 2.451000e+02, 2.741000e+02, 3.096000e+02, 3.536000e+02, 4.091000e+02, 4.821000e+02,
  5.831000e+02, 7.316000e+02, 9.751000e+02, 1.464000e+03};

void eval_2d(const double *rows, int64_t n, int ncol, gelio_spectra &o) {
  const double q = kQ, c = kC, T0w = kM0 * kC * kC, Tr = 0.938;
  for (int64_t i = 0; i < n; ++i) {
    const double *row = rows + i * ncol;
    const double Tkininj = row[0], Tkin = row[1];
    double Tkinw = Tkin * 1e9 * q;
    double Rig = std::sqrt(Tkinw * (Tkinw + (2 * T0w))) / q;
    const double p = Rig * q / c;
    Tkinw = Tkininj * 1e9 * q;
    const double Rig1AU = std::sqrt(Tkinw * (Tkinw + (2 * T0w))) / q;
    const double p1AU = Rig1AU * q / c;
    const double tem5 = 21.1 * std::exp(-2.8 * std::log(Tkininj));
    const double tem6 = 1.0 + (5.85 * std::exp(-1.22 * std::log(Tkininj))) + (1.18 * std::exp(-2.54 * std::log(Tkininj)));
    const double jlis = tem5 / tem6;
    double w = jlis / (p * p);
    w = w * p1AU * p1AU;
    const double tt = Tkin + Tr;
    const double t2 = tt + Tr;
    const double beta = std::sqrt(Tkin * t2) / tt;
    double tem = (Tkin + 0.67) / 1.67;
    tem = std::exp(-3.93 * std::log(tem));
    double jlisJGR = 2.7e3 * std::exp(1.12 * std::log(Tkin)) * tem;
    jlisJGR = jlisJGR / (beta * beta);
    double wJGR = jlisJGR / (p * p);
    wJGR = wJGR * p1AU * p1AU;
    tem = std::sqrt((Tkin * Tkin) + (2.0 * Tkin * 0.938));
    double jlisBurger = 1.9 * 1.0e4 * std::exp(-2.78 * std::log(tem));
    tem = std::sqrt((Tkin * Tkin) + (2.0 * Tkin * 0.938));
    tem = 0.4866 * std::exp(-2.51 * std::log(tem));
    jlisBurger = jlisBurger / (1 + tem);
    double wBurger = jlisBurger / (p * p);
    wBurger = wBurger * p1AU * p1AU;
    for (int ii = 1; ii < 30; ii++) {
      if ((Tkininj > kSPbinsR[ii] * 0.99) && (Tkininj < kSPbinsR[ii] * 1.01)) {
        o.sp_weber[ii] += w; o.sp_jgr[ii] += wJGR; o.sp_burger[ii] += wBurger; o.sp_n[ii] += 1;
        o.sp_weber2[ii] += w * w; o.sp_jgr2[ii] += wJGR * wJGR; o.sp_burger2[ii] += wBurger * wBurger;
      }
    }
    for (int ii = 1; ii < 3; ii++) {
      if ((Tkininj > kUly[ii]) && (Tkininj < kUly[ii + 1])) {
        o.uly_w[ii] += wBurger; o.uly_w2[ii] += wBurger * wBurger; o.uly_n[ii] += 1;
      }
    }
    for (int ii = 1; ii < 71; ii++) {
      if ((Tkininj > kAms[ii]) && (Tkininj < kAms[ii + 1])) {
        o.ams_w[ii] += wBurger; o.ams_w2[ii] += wBurger * wBurger; o.ams_n[ii] += 1;
      }
    }
    o.n_records += 1;
  }
}

void lin_bins(double Tkin, double w, gelio_spectra &o) {
  const int e2 = (int)std::trunc(Tkin);
  if (e2 > 0 && e2 < 101) { o.e2_w[e2 - 1] += w; o.e2_w2[e2 - 1] += w * w; o.e2_n[e2 - 1] += 1; }
  const int e3 = (int)std::trunc((Tkin + 0.05) * 10);
  if (e3 > 0 && e3 < 1001) { o.e3_w[e3 - 1] += w; o.e3_w2[e3 - 1] += w * w; o.e3_n[e3 - 1] += 1; }
  const int e4 = (int)std::trunc((Tkin + 0.125) * 4);
  if (e4 > 0 && e4 < 401) { o.e4_w[e4 - 1] += w; o.e4_w2[e4 - 1] += w * w; o.e4_n[e4 - 1] += 1; }
}

void eval_bp(const double *rows, int64_t n, int ncol, gelio_spectra &o) {
  const double q = kQ, c = kC, m0 = kM0, T0w = kM0 * kC * kC;
  const int NT = 80;
  const double dlT = std::log10(200.0 / 0.01) / NT, X = std::log10(200.0);
  double binb[81];
  for (int i = 0; i < NT; i++) binb[i] = std::exp((X - (i * dlT)) * std::log(10.0));
  for (int64_t i = 0; i < n; ++i) {
    const double *row = rows + i * ncol;
    const double Tkininj = row[0], Tkin = row[1];
    double Tkinw = Tkininj * 1e9 * q;
    const double Rig = std::sqrt(Tkinw * (Tkinw + (2 * T0w))) / q;
    const double p = Rig * q / c;
    Tkinw = Tkin * 1e9 * q;
    const double Rig1AU = std::sqrt(Tkinw * (Tkinw + (2 * T0w))) / q;
    const double p1AU = Rig1AU * q / c;
    double w = (m0 * m0 * c * c * c * c) + (p * p * c * c);
    w = std::exp(-1.85 * std::log(w)) / p;
    w = w * p1AU * p1AU;
    // bins whose both edges are defined (binb[0..79]); see the evaluator's
    // uninitialised binb[80..299]
    for (int ii = 0; ii < NT - 1; ii++) {
      if ((Tkin > binb[ii + 1]) && (Tkin < binb[ii])) {
        o.log_w[ii + 1] += w; o.log_w2[ii + 1] += w * w; o.log_n[ii + 1] += 1;
      }
    }
    lin_bins(Tkin, w, o);
    o.n_records += 1;
  }
}

void eval_fp(const double *rows, int64_t n, int ncol, gelio_spectra &o) {
  const double q = kQ, c = kC, m0 = kM0, T0 = kT0;
  double binb[25];
  for (int i = 0; i < 25; i++) binb[i] = std::exp((((i + 1) / 5.0) - 3.0) * std::log(10));
  for (int64_t i = 0; i < n; ++i) {
    const double *row = rows + i * ncol;
    const double p100AU = row[0], p1AU = row[1], r = row[2], sumac = row[4];
    const double Rig = p1AU * c / q;
    double Tkin = std::sqrt((T0 * T0 * q * q * 1e9 * 1e9) + (q * q * Rig * Rig)) - (T0 * q * 1e9);
    Tkin = Tkin / (q * 1e9);
    double w0 = (m0 * m0 * c * c * c * c) + (p100AU * p100AU * c * c);
    w0 = std::exp(-1.85 * std::log(w0)) / p100AU;
    w0 = w0 / 1e45;
    double w = w0 * p1AU * p1AU * std::exp(sumac);
    if (r < 0.3) w = 0.0;
    for (int k = 0; k < 24; k++) {
      if (Tkin > binb[k] && Tkin < binb[k + 1]) { o.log_w[k] += w; o.log_w2[k] += w * w; o.log_n[k] += 1; }
    }
    lin_bins(Tkin, w, o);
    o.n_records += 1;
  }
}

}  // namespace

extern "C" {

void gor_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox(ctr, key, out); }

void gor_normals(uint32_t ctr0, uint32_t stream, uint64_t pid, const uint32_t key[2], double z[4]) {
  philox_normals(ctr0, stream, pid, key, z);
}

float gor_injection(const gelio_sim_params *p, uint64_t pid) { return injection(*p, pid); }

// GPU-flavour replay of particles [first, first + count).
int gor_replay(const gelio_sim_params *p, int64_t first, int64_t count, uint64_t max_steps,
               gelio_trajectory *out) {
  if (!p || !out || first < 0 || count < 0) return 1;
  if (max_steps == 0) max_steps = 100000000ull;
  for (int64_t i = 0; i < count; ++i) {
    Traj t;
    const uint64_t pid = (uint64_t)(first + i);
    switch (p->model) {
      case GELIO_MODEL_2D_GELIOSPHERE: gpu_geliosphere(*p, pid, max_steps, t); break;
      case GELIO_MODEL_2D_SOLARPROP: gpu_solarprop(*p, pid, max_steps, t); break;
      case GELIO_MODEL_1D_BP: gpu_bp(*p, pid, max_steps, t); break;
      default: gpu_fp(*p, pid, max_steps, t); break;
    }
    gelio_trajectory &o = out[i];
    o.status = t.status;
    o.steps = t.steps;
    o.n_records = t.nrec;
    o.t_injection = (float)t.Tinj;
    o.t_final = (float)t.T;
    o.r_final = (float)t.r;
    o.theta_final = (float)t.aux;
    o.t_record = (float)t.Trec;
    o.r_record = (float)t.rrec;
    o.aux_record = (float)t.auxrec;
  }
  return 0;
}

// FP64 values of the replay (the float fields of gelio_trajectory lose
// precision); out6 = [T_final, r_final, aux_final, T_rec, r_rec, aux_rec] per particle.
int gor_replay_f64(const gelio_sim_params *p, int64_t first, int64_t count, uint64_t max_steps,
                   int32_t *status, uint32_t *steps, int32_t *nrec, double *out6) {
  if (!p || first < 0 || count < 0) return 1;
  if (max_steps == 0) max_steps = 100000000ull;
  for (int64_t i = 0; i < count; ++i) {
    Traj t;
    const uint64_t pid = (uint64_t)(first + i);
    switch (p->model) {
      case GELIO_MODEL_2D_GELIOSPHERE: gpu_geliosphere(*p, pid, max_steps, t); break;
      case GELIO_MODEL_2D_SOLARPROP: gpu_solarprop(*p, pid, max_steps, t); break;
      case GELIO_MODEL_1D_BP: gpu_bp(*p, pid, max_steps, t); break;
      default: gpu_fp(*p, pid, max_steps, t); break;
    }
    status[i] = t.status; steps[i] = t.steps; nrec[i] = t.nrec;
    double *o = out6 + 6 * i;
    o[0] = t.T; o[1] = t.r; o[2] = t.aux; o[3] = t.Trec; o[4] = t.rrec; o[5] = t.auxrec;
  }
  return 0;
}

// gor_replay_f64 of a 2D model with the rounding-noise control of relative
// size eps applied after every step to r, theta and T (on_increments = 0) or
// to dr, dtheta and dT (on_increments = 1); see noise_factor.
int gor_replay_f64_noise(const gelio_sim_params *p, int64_t first, int64_t count, uint64_t max_steps,
                         double eps, int32_t on_increments, int32_t *status, uint32_t *steps, int32_t *nrec,
                         double *out6) {
  if (!p || first < 0 || count < 0) return 1;
  if (p->model != GELIO_MODEL_2D_GELIOSPHERE && p->model != GELIO_MODEL_2D_SOLARPROP) return 1;
  if (max_steps == 0) max_steps = 100000000ull;
  for (int64_t i = 0; i < count; ++i) {
    Traj t;
    const uint64_t pid = (uint64_t)(first + i);
    if (p->model == GELIO_MODEL_2D_GELIOSPHERE) gpu_geliosphere(*p, pid, max_steps, t, eps, on_increments);
    else gpu_solarprop(*p, pid, max_steps, t, eps, on_increments);
    status[i] = t.status; steps[i] = t.steps; nrec[i] = t.nrec;
    double *o = out6 + 6 * i;
    o[0] = t.T; o[1] = t.r; o[2] = t.aux; o[3] = t.Trec; o[4] = t.rrec; o[5] = t.auxrec;
  }
  return 0;
}

// CPU flavour: one simulation(threadNumber, availableThreads, iteration) call
// of the reference CPU model with a fresh std::mt19937(seed) and
// std::normal_distribution<float>(0, 1).  Writes up to max_rows rows of
// cpu_cols(model) doubles; returns the number of rows produced.
int64_t gor_cpu_block(int model, const gor_cpu_params *c, int thread_number, int available_threads,
                      int iteration, uint32_t seed, double *rows, int64_t max_rows, int64_t *steps) {
  std::mt19937 generator(seed);
  std::normal_distribution<float> distribution(0.0f, 1.0f);
  RowSink sink{rows, max_rows, 0, cpu_cols(model)};
  cpu_fn(model)(*c, thread_number, (unsigned)available_threads, iteration, generator, distribution, sink, steps);
  return sink.n;
}

int gor_cpu_cols(int model) { return cpu_cols(model); }

// Evaluate parsed log.dat rows like the reference evaluators (all rows given
// are used; the caller drops the last line as the reference's
// countLines() - 1 does).
int gor_evaluate(int model, const double *rows, int64_t n_rows, int n_cols, gelio_spectra *out) {
  if (!out || n_rows < 0 || (n_rows > 0 && !rows)) return 1;
  std::memset(out, 0, sizeof(*out));
  if (n_cols < cpu_cols(model)) return 1;
  if (model >= GELIO_MODEL_2D_SOLARPROP) eval_2d(rows, n_rows, n_cols, *out);
  else if (model == GELIO_MODEL_1D_BP) eval_bp(rows, n_rows, n_cols, *out);
  else eval_fp(rows, n_rows, n_cols, *out);
  return 0;
}

// CPU baseline: the reference CPU model's structure -- `threads` std::threads
// per iteration, each running one simulation() block of the model with its
// own generator -- for `iterations` iterations.  Returns wall seconds.
double gor_cpu_baseline(int model, const gor_cpu_params *c, int threads, int iterations, uint32_t seed,
                        int64_t *n_traj, int64_t *n_records, int64_t *n_steps) {
  if (threads < 1) threads = (int)std::thread::hardware_concurrency();
  if (threads < 1) threads = 1;
  const auto t0 = std::chrono::steady_clock::now();
  std::atomic<int64_t> rec{0}, st{0};
  for (int it = 0; it < iterations; ++it) {
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
      pool.emplace_back([&, t]() {
        std::mt19937 generator(seed + (uint32_t)(it * threads + t));
        std::normal_distribution<float> distribution(0.0f, 1.0f);
        RowSink sink{nullptr, 0, 0, cpu_cols(model)};
        int64_t s = 0;
        cpu_fn(model)(*c, t, (unsigned)threads, it, generator, distribution, sink, &s);
        rec += sink.n;
        st += s;
      });
    }
    for (auto &th : pool) th.join();
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  const int64_t per_block = (model >= GELIO_MODEL_2D_SOLARPROP) ? 30 * 500 : 101 * 250;
  if (n_traj) *n_traj = per_block * (int64_t)threads * iterations;
  if (n_records) *n_records = rec.load();
  if (n_steps) *n_steps = st.load();
  return secs;
}

// CPU baseline of a grid workload: the 2D model's reference CPU loop
// (cpu flavour) over n_cases parameter sets, each injecting per_point
// particles at every energy of params[k].inj_energies; host threads take
// (case, grid point) units from a shared counter, each with its own
// std::mt19937.  Returns wall seconds; n_traj / n_records / n_steps summed.
double gor_cpu_grid_baseline(int model, const gor_cpu_params *params, int n_cases, int threads, uint32_t seed,
                             int64_t *n_traj, int64_t *n_records, int64_t *n_steps) {
  if (!params || n_cases < 1) return -1.0;
  if (threads < 1) threads = (int)std::thread::hardware_concurrency();
  if (threads < 1) threads = 1;
  const int points = params[0].inj_points;
  const int64_t units = (int64_t)n_cases * points;
  std::atomic<int64_t> next{0}, rec{0}, st{0}, traj{0};
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    pool.emplace_back([&, t]() {
      std::mt19937 generator(seed + (uint32_t)t);
      std::normal_distribution<float> distribution(0.0f, 1.0f);
      for (int64_t u = next++; u < units; u = next++) {
        gor_cpu_params c = params[u / points];
        c.inj_energies = params[u / points].inj_energies + (u % points);
        c.inj_points = 1;
        RowSink sink{nullptr, 0, 0, cpu_cols(model)};
        int64_t s = 0;
        cpu_fn(model)(c, t, (unsigned)threads, 0, generator, distribution, sink, &s);
        rec += sink.n;
        st += s;
        traj += c.inj_per_point;
      }
    });
  }
  for (auto &th : pool) th.join();
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (n_traj) *n_traj = traj.load();
  if (n_records) *n_records = rec.load();
  if (n_steps) *n_steps = st.load();
  return secs;
}

}  // extern "C"
