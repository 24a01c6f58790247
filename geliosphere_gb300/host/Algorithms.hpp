// The model algorithms and batch mode behind the reference's interfaces
// (Algorithm/src/*Algorithm.cpp:11-40, Algorithm/src/BatchRun.cpp:26-365).
#pragma once
#include <string>
#include <vector>

#include "Results.hpp"

class OneDimensionFpAlgorithm : public AbstractAlgorithm { public: void runAlgorithm(ParamsCarrier *p) override; };
class OneDimensionBpAlgorithm : public AbstractAlgorithm { public: void runAlgorithm(ParamsCarrier *p) override; };
class SolarPropLikeAlgorithm : public AbstractAlgorithm { public: void runAlgorithm(ParamsCarrier *p) override; };
class GeliosphereAlgorithm : public AbstractAlgorithm { public: void runAlgorithm(ParamsCarrier *p) override; };

// Batch mode: every valid row of the batch CSV is resolved as the reference
// resolves it row by row, then all rows run in ONE engine call (one
// persistent launch per model); each row's spectra and report are written
// into its own results/<model>/<name>/ directory.
class BatchRun : public AbstractAlgorithm { public: void runAlgorithm(ParamsCarrier *p) override; };

// Rows of a batch CSV resolved as BatchRun resolves them (directories and
// simulation_log.txt included), without running them: the simulations and
// their 1-based row numbers; -1 if the file cannot be used.
int batchPlan(ParamsCarrier *p, const std::string &path, std::vector<gelio_sim_params> &sims,
              std::vector<int> &rows);

// Model name -> algorithm (Factory/src/CosmicFactory.cpp:8-31); nullptr if unknown.
AbstractAlgorithm *getAlgorithm(const std::string &name);
