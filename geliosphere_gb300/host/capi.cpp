// extern "C" surface of the host layer (gelio_host.h).
#include "gelio_host.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unistd.h>
#include <vector>

#include "Algorithms.hpp"
#include "Engine.hpp"
#include "Input.hpp"
#include "Log.hpp"
#include "ParamsCarrier.hpp"
#include "Results.hpp"

static int32_t copy_out(const std::string &s, char *buf, int32_t cap) {
  if (buf && cap > 0) {
    const size_t n = std::min((size_t)cap - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
  }
  return (int32_t)s.size();
}

extern "C" {

int32_t gelio_host_main(int32_t argc, char **argv) {
  if (gelio_host_parse(argc, argv) != 1) return -1;
  ParamsCarrier *p = ParamsCarrier::instance();
  AbstractAlgorithm *a = getAlgorithm(p->getString("model", "1D Fp"));
  if (!a) {
    glog::error("Selected custom model is not defined in factory.");
    return -1;
  }
  ghost::runFailed() = false;
  a->runAlgorithm(p);
  delete a;
  return ghost::runFailed() ? 1 : 0;
}

int32_t gelio_host_parse(int32_t argc, char **argv) { return parseParams(argc, argv, ParamsCarrier::instance()); }

void gelio_host_reset(void) { ParamsCarrier::instance()->eraseAllItems({}); }

int32_t gelio_host_get_int(const char *k, int32_t d) { return ParamsCarrier::instance()->getInt(k, d); }
float gelio_host_get_float(const char *k, float d) { return ParamsCarrier::instance()->getFloat(k, d); }
int32_t gelio_host_get_string(const char *k, const char *d, char *buf, int32_t cap) {
  return copy_out(ParamsCarrier::instance()->getString(k, d ? d : ""), buf, cap);
}
void gelio_host_put_int(const char *k, int32_t v) { ParamsCarrier::instance()->putInt(k, v); }
void gelio_host_put_float(const char *k, float v) { ParamsCarrier::instance()->putFloat(k, v); }
void gelio_host_put_string(const char *k, const char *v) { ParamsCarrier::instance()->putString(k, v ? v : ""); }

int32_t gelio_host_load_settings(const char *path) {
  return (path && loadSettings(path, ParamsCarrier::instance())) ? 1 : 0;
}

int32_t gelio_host_resolve(int32_t model, gelio_sim_params *out) {
  if (!out || model < 0 || model > GELIO_MODEL_2D_GELIOSPHERE) return GELIO_ERR_INVALID_ARGUMENT;
  *out = ghost::resolveSimParams(ParamsCarrier::instance(), model);
  return GELIO_OK;
}

int32_t gelio_host_batch_plan(const char *csv_path, gelio_sim_params *out, int32_t *rows, int32_t cap,
                              int32_t *n) {
  if (!csv_path || !n || cap < 0) return GELIO_ERR_INVALID_ARGUMENT;
  std::vector<gelio_sim_params> sims;
  std::vector<int> rr;
  const int k = batchPlan(ParamsCarrier::instance(), csv_path, sims, rr);
  if (k < 0) return GELIO_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < k && i < cap; ++i) {
    if (out) out[i] = sims[(size_t)i];
    if (rows) rows[i] = rr[(size_t)i];
  }
  *n = k;
  return GELIO_OK;
}

int32_t gelio_host_write_spectra(int32_t model, const gelio_spectra *s, int32_t csv, const char *dir) {
  if (!s || model < 0 || model > GELIO_MODEL_2D_GELIOSPHERE) return GELIO_ERR_INVALID_ARGUMENT;
  char here[4096];
  if (!getcwd(here, sizeof here)) return GELIO_ERR_INVALID_ARGUMENT;
  if (dir && chdir(dir) != 0) return GELIO_ERR_INVALID_ARGUMENT;
  writeModelSpectra(model, *s, csv != 0);
  if (dir && chdir(here) != 0) return GELIO_ERR_INVALID_ARGUMENT;
  return GELIO_OK;
}

int32_t gelio_host_log_line(int32_t model, const gelio_exit_record *r, float theta_injection, char *buf, int32_t cap) {
  if (!r) return -1;
  return copy_out(ghost::logLine(model, *r, theta_injection), buf, cap);
}

int32_t gelio_host_carrington_rotation(int32_t month, int32_t year) {
  return std::atoi(validation::carringtonRotation(month, year).c_str());
}

}  // extern "C"
