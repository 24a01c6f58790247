#include "GpuModels.hpp"

#include <cstdio>
#include <string>
#include <vector>

#include "Engine.hpp"
#include "FileUtils.hpp"
#include "Log.hpp"
#include "ParamsCarrier.hpp"

bool runGpuModel(ParamsCarrier *p, int model) {
  ghost::lastFused().valid = false;
  std::string destination = p->getString("destination", "");
  if (destination.empty()) {
    destination = getDirectoryName(p);
    glog::info("Destination is not specified - using generated name for destination: " + destination);
  }
  if (!createDirectory(ghost::modelDirectory(model), destination)) {
    // as GeliosphereModel.cu:412-416: logged, no simulation, no spectra; the
    // executable then exits 1 (a run that could not happen)
    glog::error("Directory for the simulation cannot be created.");
    ghost::runFailed() = true;
    return false;
  }
  gelio_ctx *ctx = ghost::context();
  if (!ctx) return false;
  const gelio_sim_params sim = ghost::resolveSimParams(p, model);
  const bool keepLog = p->getInt("remove_log_files_after_simulation", 1) == 0;
  gelio_run_opts opts = {};
  std::vector<gelio_exit_record> recs;
  if (keepLog) {
    // B-p / 2D: at most one record per particle; F-p may cross 1 AU repeatedly
    const int64_t cap = sim.n_particles + (model == GELIO_MODEL_1D_FP ? sim.n_particles : 0) + 1024;
    recs.resize((size_t)cap);
    opts.records = recs.data();
    opts.record_capacity = cap;
  }
  auto &fused = ghost::lastFused();
  gelio_run_stats stats = {};
  glog::info("Starting simulation of " + std::to_string((long long)sim.n_particles) + " test particles.");
  const int st = gelio_run(ctx, &sim, 1, &opts, &fused.spectra, &stats);
  if (st != GELIO_OK && st < GELIO_WARN_FIRST) {
    glog::error(std::string("Simulation failed: ") + gelio_status_string(st) + " " + gelio_last_error());
    ghost::runFailed() = true;
    return false;
  }
  if (st >= GELIO_WARN_FIRST) glog::warn(gelio_status_string(st));
  fused.valid = true;
  fused.model = model;
  if (keepLog) {
    FILE *f = std::fopen("log.dat", "w");
    if (f) {
      for (int64_t i = 0; i < stats.n_records_stored; ++i) {
        const std::string ln = ghost::logLine(model, recs[(size_t)i], sim.theta_injection);
        std::fputs(ln.c_str(), f);
      }
      std::fclose(f);
    }
  }
  char msg[160];
  std::snprintf(msg, sizeof msg, "Simulation ended: %lld records, %.3g particle-steps, %.1f ms on the GPU.",
                (long long)stats.n_records, (double)stats.n_steps, stats.kernel_ms);
  glog::info(msg);
  writeSimulationReportFile(p);
  return true;
}

void OneDimensionFpGpuModel::prepareAndRunSimulation(ParamsCarrier *p) { runGpuModel(p, GELIO_MODEL_1D_FP); }
void OneDimensionBpGpuModel::prepareAndRunSimulation(ParamsCarrier *p) { runGpuModel(p, GELIO_MODEL_1D_BP); }
void SolarPropLikeGpuModel::prepareAndRunSimulation(ParamsCarrier *p) { runGpuModel(p, GELIO_MODEL_2D_SOLARPROP); }
void GeliosphereGpuModel::prepareAndRunSimulation(ParamsCarrier *p) { runGpuModel(p, GELIO_MODEL_2D_GELIOSPHERE); }
