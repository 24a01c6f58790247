#include "Engine.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <unistd.h>

#include "Log.hpp"
#include "ParamsCarrier.hpp"

namespace ghost {

gelio_ctx *context() {
  static gelio_ctx *ctx = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    const int st = gelio_create(&ctx, 0);
    if (st != GELIO_OK) {
      glog::error(std::string("GPU engine unavailable: ") + gelio_status_string(st));
      ctx = nullptr;
    }
  }
  if (!ctx) runFailed() = true;
  return ctx;
}

bool &runFailed() {
  static bool failed = false;
  return failed;
}

FusedSpectra &lastFused() {
  static FusedSpectra f;
  return f;
}

int modelFromName(const std::string &n) {
  if (n == "1D Fp") return GELIO_MODEL_1D_FP;
  if (n == "1D Bp") return GELIO_MODEL_1D_BP;
  if (n == "2D SolarProp-like") return GELIO_MODEL_2D_SOLARPROP;
  if (n == "2D Geliosphere") return GELIO_MODEL_2D_GELIOSPHERE;
  return -1;
}

const char *modelDirectory(int model) {
  switch (model) {
    case GELIO_MODEL_1D_FP: return "1DFP";
    case GELIO_MODEL_1D_BP: return "1DBP";
    case GELIO_MODEL_2D_SOLARPROP: return "SOLARPROPLike";
    default: return "Geliosphere2D";
  }
}

gelio_sim_params resolveSimParams(ParamsCarrier *p, int model) {
  gelio_sim_params s = {};
  s.model = model;
  const std::string name = p->getString("model", "1D Fp");
  // __constant__ defaults (CosmicConstants.cu:14-41)
  float V = 2.66667e-6f, dt = 5.0f, K0 = 0.000222f, ratio = 0.2f, delta0 = 8.7e-5f;
  float alphaM = 5.75f * 3.1415926535f / 180.0f;
  // setSolarPropConstants / setGeliosphereModelConstants
  if (name == "2D SolarProp-like") {
    ratio = p->getFloat("solarPropRatio", 0.02f);
    const float newK = p->getFloat("K0", p->getFloat("K0_default", -1.0f));
    if (newK != -1.0f && !p->getInt("K0_entered_by_user", 0)) K0 = newK;
  }
  if (name == "2D Geliosphere") {
    ratio = p->getFloat("geliosphereRatio", 0.2f);
    delta0 = p->getFloat("C_delta", 8.7e-5f);
    alphaM = p->getFloat("tilt_angle", p->getFloat("default_tilt_angle", 0.1f)) * 3.1415926535f / 180.0f;
    float newK = p->getFloat("K0", p->getFloat("K0_default", -1.0f));
    if (newK != -1.0f && !p->getInt("K0_entered_by_user", 0)) {
      newK *= p->getFloat("K0_ratio", 5.0f);
      K0 = newK;
    }
  }
  // setConstants
  const float rInit = p->getFloat("r_injection", 1.0f);
  const float thetainj = p->getFloat("theta_injection", 90.0f) * 3.1415926535f / 180.0f;
  const float polarity = (float)p->getInt("polarity", 1);
  const float injectionMax = p->getFloat("uniform_energy_injection_maximum", 101.0f);
  const bool useUniform = p->getInt("use_uniform_injection", 0) != 0;
  const float newDT = p->getFloat("dt", p->getFloat("dt_default", -1.0f));
  if (newDT != -1.0f) dt = newDT;
  const float newK = p->getFloat("K0", p->getFloat("K0_default", -1.0f));
  if (newK != -1.0f && p->getInt("K0_entered_by_user", 0)) K0 = newK;
  const bool isBackward = (name == "1D Bp");
  float newV = isBackward ? p->getFloat("V", p->getFloat("V_default", 1.0f)) * (-1.0f)
                          : p->getFloat("V", p->getFloat("V_default", -1.0f));
  if (newV != -1.0f) V = newV;
  else V = isBackward ? 2.66667e-6f * (-1.0f) : 2.66667e-6f;

  s.K0 = K0;
  s.V = std::fabs(V);              // the engine applies the backward sign itself
  s.dt = dt;
  s.r_injection = rInit;
  s.theta_injection = thetainj;
  s.tilt = alphaM;
  s.polarity = polarity;
  s.ratio = ratio;
  s.delta0 = delta0;
  s.injection_max = injectionMax;
  s.inj_min = 0.01f;
  s.inj_max = 100.0f;
  s.inj_points = 100;
  s.injection = (model >= GELIO_MODEL_2D_SOLARPROP)
                    ? (useUniform ? GELIO_INJ_REFERENCE_UNIFORM : GELIO_INJ_SOLARPROP_GRID)
                    : GELIO_INJ_REFERENCE_UNIFORM;
  const long long millions = p->getInt("millions", 1);
  const long long chunk = 4096;
  s.n_particles = (millions * 1000000LL + chunk - 1) / chunk * chunk;
  const char *seed = std::getenv("GELIO_SEED");
  s.seed = seed ? (uint64_t)std::strtoull(seed, nullptr, 10)
                : ((uint64_t)time(nullptr) << 20) ^ (uint64_t)getpid() ^ ((uint64_t)model << 60);
  return s;
}

// SI momentum of a kinetic energy [GeV], as the evaluators compute it.
static double p_si(double T) {
  const double q = 1.60219e-19, c = 2.99793e8, T0w = 1.67261e-27 * c * c;
  const double Tw = (T * 1e9) * q;
  return (std::sqrt(Tw * (Tw + 2.0 * T0w)) / q * q) / c;
}
static double yamada_1e45(double p) {
  const double m0 = 1.67261e-27, c = 2.99793e8;
  const double w = (m0 * m0 * c * c * c * c) + (p * p * c * c);
  return (std::pow(w, -1.85) / p) / 1e45;
}

std::string logLine(int model, const gelio_exit_record &r, float thetaInjection) {
  char buf[256];
  if (model >= GELIO_MODEL_2D_SOLARPROP) {
    std::snprintf(buf, sizeof buf, "%g %g %g %g %g %g\n", (double)r.t_injection, (double)r.t_exit, (double)r.r,
                  yamada_1e45(p_si(r.t_injection)), (double)thetaInjection, (double)r.theta);
  } else if (model == GELIO_MODEL_1D_BP) {
    std::snprintf(buf, sizeof buf, "%g %g %g %g\n", (double)r.t_exit, (double)r.t_injection, (double)r.r,
                  yamada_1e45(p_si(r.t_exit)));
  } else {
    const double pinj = p_si(r.t_injection);
    std::snprintf(buf, sizeof buf, " %g  %g  %g  %g %g \n", pinj, p_si(r.t_exit), (double)r.r, yamada_1e45(pinj),
                  (double)r.sumac);
  }
  return buf;
}

}  // namespace ghost
