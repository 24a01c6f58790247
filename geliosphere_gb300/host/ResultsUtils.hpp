// Spectrum files in the reference's formats (Utils/src/ResultsUtils.cpp:16-131):
// name + ".dat" (space-separated) or ".csv" (comma-separated, with header);
// log spectra "%.14E %.14E", linear spectra "%3.4f %.14E %.14E",
// SolarProp / Ulysses / AMS spectra "%3.4f" x 4.
#pragma once
#include <cstdio>
#include <string>

enum spectrumType {
  SPECTRUM_LOG = 1,
  SPECTRUM_1E2 = 2,
  SPECTRUM_1E3 = 3,
  SPECTRUM_4E2 = 4,
  SPECTRUM_SOLARPROP = 5,
  SPECTRUM_ULYSSES = 6,
  SPECTRUM_AMS = 7
};

struct spectrumOutput {
  std::string fileName;
  int size = 0;
  int tkinPortion = 1;
  bool isCsv = false;
};

class ResultsUtils {
 public:
  // Write `fileName`.dat/.csv in the current directory; 0 on success.
  int writeSpectrum(spectrumOutput *out, const double *spectrumCount, const double *spectrumValue,
                    spectrumType type);
  // Lines in a file (the evaluators read countLines() - 1 records).
  int countLines(FILE *fin);
};
