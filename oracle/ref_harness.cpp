// TEST INFRASTRUCTURE: a driver around the reference's own CPU model code,
// compiled from the reference sources where they lie (oracle/Makefile,
// target `ref`; outputs only into oracle/_ref/, which is not committed).
//
// GELIO_REF_MODEL selects the model source compiled into this translation
// unit (0 = OneDimensionFpCpuModel.cpp, 1 = OneDimensionBpCpuModel.cpp,
// 2 = SolarPropLikeCpuModel.cpp, 3 = GeliosphereCpuModel.cpp).  Including the
// source here gives this harness the model's file-static constants and its
// setContants() (CpuImplementations/include/Constants.hpp:188-223), so the
// parameters are resolved by the reference's own code.
//
// usage: ref_model_X key=value ... -- t,n,it,seed [t,n,it,seed ...]
//   keys are ParamsCarrier keys (model is implied); float keys: dt, K0, V,
//   r_injection, theta_injection, tilt_angle, geliosphereRatio,
//   solarPropRatio, C_delta, K0_ratio, uniform_energy_injection_maximum;
//   int keys: polarity, use_uniform_injection, K0_entered_by_user.
// For each block the reference simulation(t, n, it) runs in a fresh thread
// whose generator is seeded with `seed`, and its output queue is printed.
#if GELIO_REF_MODEL == 0
#include "OneDimensionFpCpuModel.cpp"
typedef OneDimensionFpCpuModel Model;
static const char *kModelName = "1D Fp";
#elif GELIO_REF_MODEL == 1
#include "OneDimensionBpCpuModel.cpp"
typedef OneDimensionBpCpuModel Model;
static const char *kModelName = "1D Bp";
#elif GELIO_REF_MODEL == 2
#include "SolarPropLikeCpuModel.cpp"
typedef SolarPropLikeCpuModel Model;
static const char *kModelName = "2D SolarProp-like";
#else
#include "GeliosphereCpuModel.cpp"
typedef GeliosphereCpuModel Model;
static const char *kModelName = "2D Geliosphere";
#endif

#include <chrono>

unsigned gelio_ref::next_seed = 0;

static void print_row(const SimulationOutput &o) {
#if GELIO_REF_MODEL == 0
  printf("%.17g %.17g %.17g %.17g %.17g\n", o.pinj, o.p, o.r, o.w, o.sumac);
#elif GELIO_REF_MODEL == 1
  printf("%.17g %.17g %.17g %.17g\n", o.Tkin, o.Tkininj, o.r, o.w);
#else
  printf("%.17g %.17g %.17g %.17g %.17g %.17g\n", o.Tkininj, o.Tkin, o.r, o.w, o.thetainj, o.theta);
#endif
}

int main(int argc, char **argv) {
  ParamsCarrier *pc = ParamsCarrier::instance();
  pc->putString("model", kModelName);
  int i = 1;
  bool timing = false;
  int timing_threads = 0, timing_iters = 0;
  for (; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--") { ++i; break; }
    if (a == "--time") { timing = true; timing_threads = atoi(argv[++i]); timing_iters = atoi(argv[++i]); continue; }
    const size_t eq = a.find('=');
    if (eq == std::string::npos) { fprintf(stderr, "bad argument %s\n", a.c_str()); return 2; }
    const std::string k = a.substr(0, eq), v = a.substr(eq + 1);
    if (k == "polarity" || k == "use_uniform_injection" || k == "K0_entered_by_user") pc->putInt(k, atoi(v.c_str()));
    else pc->putFloat(k, (float)atof(v.c_str()));
  }
  setContants(pc);
  printf("# V=%.17g dt=%.17g K0=%.17g ratio=%.17g delta0=%.17g alphaM=%.17g polarity=%.17g rInit=%.17g thetainj=%.17g useUniformInjection=%d uniformEnergyInjectionMaximum=%.17g\n",
         V, dt, K0, ratio, delta0, alphaM, polarity, rInit, thetainj, (int)useUniformInjection,
         uniformEnergyInjectionMaximum);
  if (timing) {
    // the reference's threading structure: hardware threads per iteration
    const auto t0 = std::chrono::steady_clock::now();
    long long records = 0;
    for (int it = 0; it < timing_iters; ++it) {
      Model m;
      std::vector<std::thread> th;
      for (int t = 0; t < timing_threads; ++t) {
        gelio_ref::next_seed = 1000u + (unsigned)(it * timing_threads + t);
        th.emplace_back(&Model::simulation, &m, t, (unsigned)timing_threads, it);
      }
      for (auto &x : th) x.join();
      records += (long long)m.outputQueue.size();
    }
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    printf("# seconds=%.6f records=%lld\n", s, records);
    return 0;
  }
  for (; i < argc; ++i) {
    int t, n, it;
    unsigned seed;
    if (sscanf(argv[i], "%d,%d,%d,%u", &t, &n, &it, &seed) != 4) { fprintf(stderr, "bad block %s\n", argv[i]); return 2; }
    Model m;
    gelio_ref::next_seed = seed;
    std::thread th(&Model::simulation, &m, t, (unsigned)n, it);
    th.join();
    printf("# block %d %d %d %u rows=%zu\n", t, n, it, seed, m.outputQueue.size());
    while (!m.outputQueue.empty()) {
      print_row(m.outputQueue.front());
      m.outputQueue.pop();
    }
  }
  return 0;
}
