// The evaluation step behind the reference's AbstractAlgorithm interface
// (Algorithm/include/AbstractAlgorithm.hpp:24-33).  After a simulation in
// this process the spectra come binned from the GPU run; in evaluation-only
// mode (--evaluation <log.dat>) the log is parsed as the reference does
// (countLines() - 1 records, its fscanf formats) and binned on the GPU.
#pragma once
#include "gelio.h"

class ParamsCarrier;

class AbstractAlgorithm {
 public:
  virtual ~AbstractAlgorithm() = default;
  virtual void runAlgorithm(ParamsCarrier *singleTone) = 0;
};

class TwoDimensionBpResults : public AbstractAlgorithm {    // TwoDimensionBpResults.cpp:13-133
 public:
  void runAlgorithm(ParamsCarrier *singleTone) override;
};
class OneDimensionBpResults : public AbstractAlgorithm {    // OneDimensionBpResults.cpp:13-112
 public:
  void runAlgorithm(ParamsCarrier *singleTone) override;
};
class OneDimensionFpResults : public AbstractAlgorithm {    // OneDimensionFpResults.cpp:13-113
 public:
  void runAlgorithm(ParamsCarrier *singleTone) override;
};

// Spectrum files of one model's spectra in the current directory (the file
// names and formats of the three evaluators).
void writeModelSpectra(int model, const gelio_spectra &s, bool csv);
