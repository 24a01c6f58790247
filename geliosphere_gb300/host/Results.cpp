#include "Results.hpp"

#include <cstdio>
#include <string>
#include <vector>

#include "Engine.hpp"
#include "Log.hpp"
#include "ParamsCarrier.hpp"
#include "ResultsUtils.hpp"

void writeModelSpectra(int model, const gelio_spectra &s, bool csv) {
  ResultsUtils ru;
  spectrumOutput o;
  o.isCsv = csv;
  if (model >= GELIO_MODEL_2D_SOLARPROP) {
    o.fileName = "Usoskin_2005";
    ru.writeSpectrum(&o, s.sp_n, s.sp_jgr, SPECTRUM_SOLARPROP);
    o.fileName = "Weber";
    ru.writeSpectrum(&o, s.sp_n, s.sp_weber, SPECTRUM_SOLARPROP);
    o.fileName = "Burger";
    ru.writeSpectrum(&o, s.sp_n, s.sp_burger, SPECTRUM_SOLARPROP);
    o.fileName = "Ulysses";
    ru.writeSpectrum(&o, s.uly_n, s.uly_w, SPECTRUM_ULYSSES);
    o.fileName = "Ams";
    ru.writeSpectrum(&o, s.ams_n, s.ams_w, SPECTRUM_AMS);
  } else {
    o.fileName = "output_1e3bin"; o.size = 1000; o.tkinPortion = 10;
    ru.writeSpectrum(&o, s.e3_n, s.e3_w, SPECTRUM_1E3);
    o.fileName = "output_1e2bin"; o.size = 100; o.tkinPortion = 1;
    ru.writeSpectrum(&o, s.e2_n, s.e2_w, SPECTRUM_1E2);
    o.fileName = "output_logbin";
    ru.writeSpectrum(&o, s.log_n, s.log_w, SPECTRUM_LOG);
    o.fileName = "output_4e2bin"; o.size = 400; o.tkinPortion = 4;
    ru.writeSpectrum(&o, s.e4_n, s.e4_w, SPECTRUM_4E2);
  }
}

// Evaluation-only mode: parse log.dat with the reference's formats.
static bool evaluateLog(ParamsCarrier *p, int model, gelio_spectra &out) {
  const std::string path = p->getString("pathToLogFile", "log.dat");
  FILE *in = std::fopen(path.c_str(), "r");
  if (!in) {
    glog::error("Could not read from log.dat file.");
    return false;
  }
  ResultsUtils ru;
  const int n = ru.countLines(in) - 1;
  if (n < 0) {
    glog::info("No trajectory found in log file.");
    glog::warn("Please, consider increase of amount of simulated test particles for current input parameters.");
  } else {
    glog::info("Founded " + std::to_string(n) + " trajectories for analysis.");
  }
  const int ncol = (model >= GELIO_MODEL_2D_SOLARPROP) ? 6 : (model == GELIO_MODEL_1D_BP ? 4 : 5);
  std::vector<double> rows;
  rows.reserve((size_t)(n > 0 ? n : 0) * ncol);
  for (int i = 0; i < n; ++i) {
    double v[6];
    int got;
    if (model >= GELIO_MODEL_2D_SOLARPROP) got = std::fscanf(in, "%lf %lf %lf %lf %lf %lf\n", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5]);
    else if (model == GELIO_MODEL_1D_BP) got = std::fscanf(in, "%lf %lf %lf %lf\n", &v[0], &v[1], &v[2], &v[3]);
    else got = std::fscanf(in, " %lf  %lf  %lf  %lf %lf \n", &v[0], &v[1], &v[2], &v[3], &v[4]);
    if (got == -1) {
      glog::error("Could not read from log.dat file.");
      std::fclose(in);
      return false;
    }
    rows.insert(rows.end(), v, v + ncol);
  }
  std::fclose(in);
  gelio_ctx *ctx = ghost::context();
  if (!ctx) return false;
  const int st = gelio_evaluate(ctx, model, rows.data(), n > 0 ? n : 0, ncol, &out);
  if (st != GELIO_OK) {
    glog::error(std::string("Evaluation failed: ") + gelio_status_string(st));
    ghost::runFailed() = true;
    return false;
  }
  return true;
}

static void runResults(ParamsCarrier *p, int model) {
  auto &fused = ghost::lastFused();
  gelio_spectra s;
  bool fromFused = p->getInt("run_simulation", 1) && fused.valid && fused.model == model;
  if (fromFused) {
    s = fused.spectra;
  } else if (!evaluateLog(p, model, s)) {
    return;
  }
  writeModelSpectra(model, s, p->getInt("csv", 0) != 0);
  glog::info("Spectra have been written to files.");
}

void TwoDimensionBpResults::runAlgorithm(ParamsCarrier *p) {
  const int m = ghost::modelFromName(p->getString("model", "1D Fp"));
  runResults(p, m >= GELIO_MODEL_2D_SOLARPROP ? m : GELIO_MODEL_2D_GELIOSPHERE);
}
void OneDimensionBpResults::runAlgorithm(ParamsCarrier *p) { runResults(p, GELIO_MODEL_1D_BP); }
void OneDimensionFpResults::runAlgorithm(ParamsCarrier *p) { runResults(p, GELIO_MODEL_1D_FP); }
