#include "ResultsUtils.hpp"

#include <cmath>

static const char *sep(bool csv) { return csv ? "," : " "; }

static void header(FILE *f, spectrumType t) {
  if (t == SPECTRUM_LOG) std::fprintf(f, "%s,%s\n", "binc", "spelog/binw");
  else std::fprintf(f, "%s,%s,%s,%s\n", "Tkin", "spe", "speAvg", "speCount");
}

int ResultsUtils::countLines(FILE *fin) {
  char buf[1024];
  int count = 0;
  while (std::fgets(buf, sizeof(buf), fin) != nullptr) ++count;
  std::rewind(fin);
  return count;
}

int ResultsUtils::writeSpectrum(spectrumOutput *out, const double *cnt, const double *val, spectrumType type) {
  const std::string name = out->fileName + (out->isCsv ? ".csv" : ".dat");
  FILE *f = std::fopen(name.c_str(), "w");
  if (!f) return -1;
  const bool csv = out->isCsv;
  const char *s = sep(csv);
  if (csv) header(f, type);
  auto avg = [&](int i) { return (cnt[i] != 0.0) ? val[i] / cnt[i] : 0.0; };
  if (type == SPECTRUM_LOG) {
    // ResultsUtils.cpp:49-65: the 24-bin layout 10^((i+1)/5 - 3)
    double binb[25], binw[24], binc[24];
    for (int i = 0; i < 25; i++) binb[i] = std::exp((((i + 1) / 5.0) - 3.0) * std::log(10));
    for (int i = 0; i < 24; i++) {
      binw[i] = binb[i + 1] - binb[i];
      binc[i] = (binb[i + 1] + binb[i]) / 2.0;
    }
    for (int i = 0; i < 24; i++) std::fprintf(f, "%.14E%s%.14E\n", binc[i], s, val[i] / binw[i]);
  } else if (type == SPECTRUM_SOLARPROP) {
    for (int i = 1; i < 30; i++)
      std::fprintf(f, "%3.4f%s%3.4f%s%3.4f%s%3.4f\n", (double)(0.01f * powf(1.0f + 0.5f, (float)(i - 1))), s, val[i], s,
                   avg(i), s, cnt[i]);
  } else if (type == SPECTRUM_ULYSSES) {
    const double bins[4] = {0.0, 0.125, 0.250, 2.0};
    for (int i = 1; i < 3; i++) std::fprintf(f, "%3.4f%s%3.4f%s%3.4f%s%3.4f\n", bins[i], s, val[i], s, avg(i), s, cnt[i]);
  } else if (type == SPECTRUM_AMS) {
    static const double ams[72] = {4.924000e-01, 6.207000e-01, 7.637000e-01, 9.252000e-01, 1.105000e+00,
      1.303000e+00, 1.523000e+00, 1.765000e+00, 2.034000e+00, 2.329000e+00, 2.652000e+00, 3.005000e+00,
      3.390000e+00, 3.810000e+00, 4.272000e+00, 4.774000e+00, 5.317000e+00, 5.906000e+00, 6.546000e+00,
      7.236000e+00, 7.981000e+00, 8.787000e+00, 9.653000e+00, 1.060000e+01, 1.160000e+01, 1.264000e+01,
      1.379000e+01, 1.504000e+01, 1.639000e+01, 1.784000e+01, 1.938000e+01, 2.103000e+01, 2.283000e+01,
      2.478000e+01, 2.683000e+01, 2.903000e+01, 3.138000e+01, 3.387000e+01, 3.657000e+01, 3.947000e+01,
      4.257000e+01, 4.587000e+01, 4.942000e+01, 5.322000e+01, 5.727000e+01, 6.162000e+01, 6.632000e+01,
      7.137000e+01, 7.677000e+01, 8.257000e+01, 8.882000e+01, 9.557000e+01, 1.031000e+02, 1.111000e+02,
      1.196000e+02, 1.291000e+02, 1.401000e+02, 1.526000e+02, 1.666000e+02, 1.826000e+02, 2.006000e+02,
      2.211000e+02, 2.451000e+02, 2.741000e+02, 3.096000e+02, 3.536000e+02, 4.091000e+02, 4.821000e+02,
      5.831000e+02, 7.316000e+02, 9.751000e+02, 1.464000e+03};
    for (int i = 1; i < 71; i++) std::fprintf(f, "%3.4f%s%3.4f%s%3.4f%s%3.4f\n", ams[i], s, val[i], s, avg(i), s, cnt[i]);
  } else {
    // linear spectra: the format has three conversions, so the count is not printed
    for (int i = 0; i < out->size; i++)
      std::fprintf(f, "%3.4f%s%.14E%s%.14E\n", (double)((float)(i + 1) / out->tkinPortion), s, val[i], s, avg(i));
  }
  std::fclose(f);
  return 0;
}
