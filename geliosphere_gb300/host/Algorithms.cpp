#include "Algorithms.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <set>
#include <string>
#include <unistd.h>
#include <vector>

#include "Engine.hpp"
#include "FileUtils.hpp"
#include "GpuModels.hpp"
#include "Input.hpp"
#include "Log.hpp"
#include "ParamsCarrier.hpp"

// Common body of the four *Algorithm::runAlgorithm (e.g.
// Algorithm/src/GeliosphereAlgorithm.cpp:11-40): simulate unless only the
// evaluation was asked for, bin, write the spectra, drop log.dat unless the
// settings keep it.  There is no CPU model in this engine: --cpu-only is
// reported and nothing runs.  In evaluation-only mode the input log is never
// unlinked (the reference unlinks ./log.dat there too, which deletes the
// file it was asked to evaluate when that is ./log.dat).
static void runModelAlgorithm(ParamsCarrier *p, AbstractGpuSimulation *gpu, AbstractAlgorithm *results) {
  const bool simulate = p->getInt("run_simulation", 1) != 0;
  if (simulate) {
    if (p->getInt("isCpu", 0)) {
      glog::error("CPU-only runs are not provided by the GB300 engine; run without --cpu-only.");
      return;
    }
    gpu->prepareAndRunSimulation(p);
    if (!ghost::lastFused().valid) return;
  }
  results->runAlgorithm(p);
  if (simulate && p->getInt("remove_log_files_after_simulation", 1)) unlink("log.dat");
}

void OneDimensionFpAlgorithm::runAlgorithm(ParamsCarrier *p) {
  OneDimensionFpGpuModel g;
  OneDimensionFpResults r;
  runModelAlgorithm(p, &g, &r);
}
void OneDimensionBpAlgorithm::runAlgorithm(ParamsCarrier *p) {
  OneDimensionBpGpuModel g;
  OneDimensionBpResults r;
  runModelAlgorithm(p, &g, &r);
}
void SolarPropLikeAlgorithm::runAlgorithm(ParamsCarrier *p) {
  SolarPropLikeGpuModel g;
  TwoDimensionBpResults r;
  runModelAlgorithm(p, &g, &r);
}
void GeliosphereAlgorithm::runAlgorithm(ParamsCarrier *p) {
  GeliosphereGpuModel g;
  TwoDimensionBpResults r;
  runModelAlgorithm(p, &g, &r);
}

AbstractAlgorithm *getAlgorithm(const std::string &name) {
  if (name == "1D Fp") return new OneDimensionFpAlgorithm();
  if (name == "1D Bp") return new OneDimensionBpAlgorithm();
  if (name == "2D SolarProp-like") return new SolarPropLikeAlgorithm();
  if (name == "2D Geliosphere") return new GeliosphereAlgorithm();
  if (name == "batch run") return new BatchRun();
  return nullptr;
}

// ---------------------------------------------------------------------------
// Batch mode
// ---------------------------------------------------------------------------
namespace {

struct BatchRow {          // struct batchRunInput (Algorithm/include/BatchRun.hpp:27-40)
  int year = -1, month = -1;
  double r = -1, theta = -1, V = -1, K0 = -1, dt = -1;
  long N = -1;
  std::string model, pathToCustomSettingsFile, name;
};

// BatchRun::getValuesForSingleSimulation (Algorithm/src/BatchRun.cpp:102-193)
void readRow(const CsvTable &t, size_t i, BatchRow &b) {
  auto warn = [](const char *c) { glog::warn(std::string("Column ") + c + " is not defined."); };
  if (t.has("name")) b.name = t.str("name", i); else warn("name");
  if (t.has("month")) b.month = (int)t.num("month", i); else warn("month");
  if (t.has("year")) b.year = (int)t.num("year", i); else warn("year");
  if (t.has("V")) b.V = (float)t.num("V", i); else warn("V");
  if (t.has("K0")) b.K0 = (float)t.num("K0", i); else warn("K0");
  if (t.has("dt")) b.dt = (float)t.num("dt", i); else warn("dt");
  if (t.has("r")) b.r = (float)t.num("r", i); else warn("r");
  if (t.has("theta")) b.theta = (float)t.num("theta", i); else warn("theta");
  if (t.has("N")) b.N = (long)t.num("N", i); else warn("N");
  if (t.has("model")) b.model = t.str("model", i); else warn("model");
  if (t.has("pathToCustomSettingsFile")) b.pathToCustomSettingsFile = t.str("pathToCustomSettingsFile", i);
  else warn("pathToCustomSettingsFile");
}

// BatchRun::validateInputForSimulation (Algorithm/src/BatchRun.cpp:254-280)
bool validateRow(const BatchRow &b) {
  const bool twoD = (b.model == "2D Geliosphere" || b.model == "2D SolarProp-like");
  if (!twoD && b.theta != -1.0) glog::warn("Setting of theta for 1D models does not have any effect on simulation");
  if ((b.month != -1 && b.year == -1) || (b.month == -1 && b.year != -1)) {
    glog::error("Both month and year must be set.");
    return false;
  }
  if (b.month != -1 && b.year != -1 && (b.K0 != -1.0 || b.V != -1.0)) {
    glog::error("Simulation dates cannot be combined with K0 or V.");
    return false;
  }
  if (b.model == "batch run") {
    glog::error("Cannot select batch run as model.");
    return false;
  }
  return true;
}

// BatchRun::parseValues (Algorithm/src/BatchRun.cpp:282-342); the row's settings are
// merged in memory instead of through a file under /tmp.
bool parseRow(ParamsCarrier *p, const BatchRow &b) {
  if (b.dt != -1.0) {
    if (!validation::checkDt((float)b.dt)) { glog::error("dt is out of range!(3-5000)"); return false; }
    validation::setDt(p, (float)b.dt);
  }
  if (b.K0 != -1.0) {
    if (!validation::checkK0((float)b.K0)) { glog::error("K0 is out of range!(>0)"); return false; }
    if (b.K0 < 1e19 || b.K0 > 1e23) glog::warn("K0 is out of recommended range!(1e19-1e23 cm^2/s)");
    validation::setK0(p, (float)b.K0);
  }
  if (b.N != -1) {
    if (!validation::checkN((int)b.N)) { glog::error("Number of test particles must be greater than 0!"); return false; }
    validation::setN(p, (int)b.N);
  }
  if (b.V != -1.0) {
    // the reference returns -1 from a bool function here, i.e. true: the row
    // runs at once, with V unset and without its name, settings or dates
    // (Algorithm/src/BatchRun.cpp:316-321); kept.
    if (!validation::checkV((float)b.V)) {
      glog::error("V is out of range!(100-1500 km/s)");
      return true;
    }
    validation::setV(p, (float)b.V);
  }
  if (!b.name.empty()) {
    if (b.name.find_first_not_of(' ') != std::string::npos) p->putString("destination", b.name);
    else glog::warn("Name containing whitespaces is not valid, using auto generated name instead.");
  }
  TomlMap t;
  if (!readToml(b.pathToCustomSettingsFile, t)) t = batchDefaultSettings();
  char buf[64];
  if (b.r > 0.0) { std::snprintf(buf, sizeof buf, "%.17g", b.r); t["default_values"]["r_injection"] = buf; }
  if (b.theta > 0.0) { std::snprintf(buf, sizeof buf, "%.17g", b.theta); t["2d_models_common_settings"]["theta_injection"] = buf; }
  applySettings(t, p);
  if (b.month != -1 && b.year != -1)
    validation::monthYearCheck(p, b.year, b.month, p->getString("currentApplicationPath", "./"));
  return true;
}

// BatchRun::validateInputBatchFile (Algorithm/src/BatchRun.cpp:344-365)
bool uniqueNames(const CsvTable &t) {
  std::vector<std::string> names;
  for (size_t i = 0; i < t.rows.size(); ++i) {
    const std::string s = t.str("name", i);
    if (!s.empty() && s.find_first_not_of(' ') != std::string::npos) names.push_back(s);
  }
  std::sort(names.begin(), names.end());
  return std::adjacent_find(names.begin(), names.end()) == names.end();
}

std::string cwd() {
  char buf[4096];
  return getcwd(buf, sizeof buf) ? std::string(buf) : std::string(".");
}

struct Planned {
  int row;
  gelio_sim_params sim;
  std::string dir;          // absolute results/<model>/<destination>
  bool keepLog;
  bool csv;
};

}  // namespace

// Rows of the batch CSV at `path` are validated and resolved one by one
// exactly as the reference does (erase, row values, settings, month/year);
// each row that resolves gets its directory and simulation_log.txt here.
// False when the file cannot be used at all (or a CPU-only run is refused).
static bool planBatch(ParamsCarrier *p, const std::string &path, bool refuseCpu, std::vector<Planned> &plan) {
  const std::set<std::string> excluded = {"default_settings_file", "currentApplicationPath", "csv", "isCpu",
                                          "inputBatchFile"};
  CsvTable doc;
  if (!doc.load(path)) {
    glog::error("Cannot open input batch file.");
    return false;
  }
  if (!uniqueNames(doc)) {
    glog::error("Input batch file contains duplicated values. Use unique names for simulations, or leave fields "
                "empty for using autogenerated values.");
    glog::error("Input batch file contains unrecoverable errors.");
    return false;
  }
  if (refuseCpu && p->getInt("isCpu", 0)) {
    glog::error("CPU-only runs are not provided by the GB300 engine; run without --cpu-only.");
    return false;
  }
  const std::string home = cwd();
  std::set<std::string> usedDirs;
  p->eraseAllItems(excluded);
  for (size_t i = 0; i < doc.rows.size(); ++i) {
    BatchRow b;
    readRow(doc, i, b);
    const int row = (int)i + 1;
    if (!validateRow(b)) { glog::error("Skipping incorrect " + std::to_string(row) + ". simulation."); continue; }
    if (!parseRow(p, b)) { glog::error("Unable to parse values for " + std::to_string(row) + ". simulation."); continue; }
    p->putString("model", b.model);
    const int model = ghost::modelFromName(b.model);
    if (model < 0) {
      // as in the reference, a skipped row leaves its values in the map
      // (Algorithm/src/BatchRun.cpp:64-70 continues without eraseAllItems)
      glog::error("Selected model for simulation " + std::to_string(row) + " is not supported in batch mode.");
      continue;
    }
    std::string dest = p->getString("destination", "");
    if (dest.empty()) {
      dest = getDirectoryName(p);
      // rows resolved within the same second with the same dt/K0/V would
      // share a generated name; keep them apart
      std::string full = std::string("results/") + ghost::modelDirectory(model) + "/" + dest;
      if (usedDirs.count(full)) dest += "_" + std::to_string(row);
      glog::info("Destination is not specified - using generated name for destination: " + dest);
    }
    if (!createDirectory(ghost::modelDirectory(model), dest)) {
      glog::error("Directory for the simulation cannot be created.");
      if (chdir(home.c_str()) != 0) return false;
      p->eraseAllItems(excluded);
      continue;
    }
    Planned pl;
    pl.row = row;
    pl.sim = ghost::resolveSimParams(p, model);
    pl.sim.seed += (uint64_t)row * 0x9E3779B97F4A7C15ull;
    pl.dir = cwd();
    pl.keepLog = p->getInt("remove_log_files_after_simulation", 1) == 0;
    pl.csv = p->getInt("csv", 0) != 0;
    writeSimulationReportFile(p);
    usedDirs.insert(std::string("results/") + ghost::modelDirectory(model) + "/" + dest);
    plan.push_back(pl);
    if (chdir(home.c_str()) != 0) {
      glog::error("Could not change directory");
      break;
    }
    p->eraseAllItems(excluded);
  }
  return true;
}

int batchPlan(ParamsCarrier *p, const std::string &path, std::vector<gelio_sim_params> &sims,
              std::vector<int> &rows) {
  std::vector<Planned> plan;
  if (!planBatch(p, path, false, plan)) return -1;
  for (auto &pl : plan) {
    sims.push_back(pl.sim);
    rows.push_back(pl.row);
  }
  return (int)plan.size();
}

// Launch shapes of a large batch picked by gelio_autotune: for each model
// in the batch, its rows with their particle counts scaled down (the sample
// holds about total / 256 particles, between 1 and 4 million, at least 4096
// per row) are timed over the tuner's block sizes, refill intervals and
// exit-queue modes, and the winner is kept in the context for that model.
// Batches below 2e7 particles run in the default shapes (tuning would cost
// more than it could save).
static void tuneBatch(gelio_ctx *ctx, const std::vector<gelio_sim_params> &sims) {
  for (int m = 0; m < 4; ++m) {
    std::vector<gelio_sim_params> rows;
    int64_t total = 0;
    for (const auto &s : sims)
      if (s.model == m && s.n_particles > 0) {
        rows.push_back(s);
        total += s.n_particles;
      }
    if (rows.empty() || total < 20000000) continue;
    const double target = std::min(4.0e6, std::max(1.0e6, (double)total / 256.0));
    const double scale = target / (double)total;
    for (auto &r : rows) r.n_particles = std::max<int64_t>(4096, (int64_t)((double)r.n_particles * scale));
    gelio_run_opts best = {};
    const int st = gelio_autotune(ctx, rows.data(), (int32_t)rows.size(), &best);
    if (st != GELIO_OK)
      glog::warn(std::string("Autotuning skipped: ") + gelio_status_string(st));
    else
      glog::info("Tuned launch for model " + std::to_string(m) + ": block " + std::to_string(best.block_size) +
                 ", refill every " + std::to_string(best.refill_interval) + " steps, exit queue mode " +
                 std::to_string(best.compact) + ".");
  }
}

// Every row that resolves is added to one gelio_run call, so all
// simulations of the batch share one persistent launch per model.  Each
// row's directory then receives its spectra and, when kept, its log.dat.
void BatchRun::runAlgorithm(ParamsCarrier *p) {
  const std::string path = p->getString("inputBatchFile", "../geliosphere_batch_input_paramaters.csv");
  const std::string home = cwd();
  std::vector<Planned> plan;
  if (!planBatch(p, path, true, plan)) return;
  if (plan.empty()) return;
  gelio_ctx *ctx = ghost::context();
  if (!ctx) return;

  std::vector<gelio_sim_params> sims;
  bool anyLog = false;
  int64_t cap = 1024;
  for (auto &pl : plan) {
    sims.push_back(pl.sim);
    anyLog |= pl.keepLog;
    cap += pl.sim.n_particles * (pl.sim.model == GELIO_MODEL_1D_FP ? 2 : 1);
  }
  std::vector<gelio_exit_record> recs;
  gelio_run_opts opts = {};
  tuneBatch(ctx, sims);
  // the whole batch is one graph-captured sequence (upload, prepare, one
  // persistent launch per model, reduce, download) in the tuned shapes
  opts.use_graph = 1;
  if (anyLog) {
    recs.resize((size_t)cap);
    opts.records = recs.data();
    opts.record_capacity = cap;
  }
  std::vector<gelio_spectra> out(plan.size());
  gelio_run_stats stats = {};
  glog::info("Starting " + std::to_string(plan.size()) + " simulations in one launch.");
  const int st = gelio_run(ctx, sims.data(), (int32_t)sims.size(), &opts, out.data(), &stats);
  if (st != GELIO_OK && st < GELIO_WARN_FIRST) {
    glog::error(std::string("Batch simulation failed: ") + gelio_status_string(st) + " " + gelio_last_error());
    ghost::runFailed() = true;
    return;
  }
  if (st >= GELIO_WARN_FIRST) glog::warn(gelio_status_string(st));
  for (size_t k = 0; k < plan.size(); ++k) {
    const Planned &pl = plan[k];
    if (chdir(pl.dir.c_str()) != 0) {
      glog::error("Could not change directory");
      break;
    }
    writeModelSpectra(pl.sim.model, out[k], pl.csv);
    if (pl.keepLog) {
      FILE *f = std::fopen("log.dat", "w");
      if (f) {
        for (int64_t i = 0; i < stats.n_records_stored; ++i)
          if (recs[(size_t)i].sim == (int32_t)k)
            std::fputs(ghost::logLine(pl.sim.model, recs[(size_t)i], pl.sim.theta_injection).c_str(), f);
        std::fclose(f);
      }
    }
    glog::info("Simulation " + std::to_string(pl.row) + " written to " + pl.dir);
  }
  if (chdir(home.c_str()) != 0) glog::error("Could not change directory");
}
