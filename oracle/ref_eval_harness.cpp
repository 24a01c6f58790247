// TEST INFRASTRUCTURE: runs the reference's own evaluators
// (Algorithm/src/{TwoDimensionBp,OneDimensionBp,OneDimensionFp}Results.cpp,
// compiled from the reference sources by oracle/Makefile, target `ref`) on a
// log.dat file; the spectrum files are written into the current directory.
// usage: ref_eval <fp|bp|2d> <log.dat> <csv 0|1>
#include "OneDimensionBpResults.hpp"
#include "OneDimensionFpResults.hpp"
#include "TwoDimensionBpResults.hpp"
#include "ParamsCarrier.hpp"

unsigned gelio_ref::next_seed = 0;

int main(int argc, char **argv) {
  if (argc < 4) { fprintf(stderr, "usage: ref_eval <fp|bp|2d> <log.dat> <csv>\n"); return 2; }
  ParamsCarrier *pc = ParamsCarrier::instance();
  pc->putString("pathToLogFile", argv[2]);
  pc->putInt("csv", atoi(argv[3]));
  const std::string m = argv[1];
  AbstractAlgorithm *alg = nullptr;
  if (m == "fp") alg = new OneDimensionFpResults();
  else if (m == "bp") alg = new OneDimensionBpResults();
  else alg = new TwoDimensionBpResults();
  alg->runAlgorithm(pc);
  return 0;
}
