#include "Input.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <set>
#include <sstream>
#include <unistd.h>

#include "Log.hpp"
#include "ParamsCarrier.hpp"

// ---------------------------------------------------------------------------
// CSV
// ---------------------------------------------------------------------------
static std::vector<std::string> split_csv(const std::string &line) {
  std::vector<std::string> out;
  std::string cur;
  bool quoted = false;
  for (char ch : line) {
    if (ch == '"') quoted = !quoted;
    else if (ch == ',' && !quoted) { out.push_back(cur); cur.clear(); }
    else if (ch != '\r') cur.push_back(ch);
  }
  out.push_back(cur);
  return out;
}

bool CsvTable::load(const std::string &path) {
  std::ifstream f(path);
  if (!f.good()) return false;
  std::string line;
  if (!std::getline(f, line)) return false;
  columns = split_csv(line);
  while (std::getline(f, line)) {
    if (line.empty() || line == "\r") continue;
    rows.push_back(split_csv(line));
  }
  return true;
}
bool CsvTable::has(const std::string &c) const {
  for (auto &x : columns) if (x == c) return true;
  return false;
}
std::string CsvTable::str(const std::string &c, size_t r) const {
  for (size_t i = 0; i < columns.size(); ++i)
    if (columns[i] == c) return (r < rows.size() && i < rows[r].size()) ? rows[r][i] : std::string();
  return std::string();
}
double CsvTable::num(const std::string &c, size_t r) const {
  const std::string s = str(c, r);
  if (s.empty()) return -1.0;
  char *end = nullptr;
  const double v = std::strtod(s.c_str(), &end);
  return (end && *end == '\0') ? v : -1.0;
}

// ---------------------------------------------------------------------------
// Settings.toml
// ---------------------------------------------------------------------------
static std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return (a == std::string::npos) ? std::string() : s.substr(a, b - a + 1);
}

bool readToml(const std::string &path, TomlMap &out) {
  std::ifstream f(path);
  if (!f.good()) return false;
  std::string line, section;
  while (std::getline(f, line)) {
    const size_t hash = line.find('#');
    if (hash != std::string::npos && line.find('"') == std::string::npos) line = line.substr(0, hash);
    line = trim(line);
    if (line.empty()) continue;
    if (line.front() == '[' && line.back() == ']') { section = trim(line.substr(1, line.size() - 2)); continue; }
    const size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    std::string v = trim(line.substr(eq + 1));
    if (v.size() >= 2 && v.front() == '"' && v.back() == '"') v = v.substr(1, v.size() - 2);
    out[section][trim(line.substr(0, eq))] = v;
  }
  return true;
}

TomlMap batchDefaultSettings() {
  TomlMap t;
  t["default_values"] = {{"uniform_energy_injection_maximum", "101.0"}, {"K0", "5e+22"}, {"V", "400.0"},
                         {"dt", "50.0"}, {"r_injection", "1.0"}};
  t["2d_models_common_settings"] = {{"theta_injection", "90.0"}, {"use_uniform_injection", "true"}};
  t["SolarProp_like_model_settings"] = {{"SolarProp_ratio", "0.02"}};
  t["Geliosphere_model_settings"] = {{"Geliosphere_ratio", "0.2"}, {"K0_ratio", "1.0"}, {"C_delta", "8.7e-05"},
                                     {"default_tilt_angle", "0.1"}};
  t["advanced_settings"] = {{"remove_log_files_after_simulation", "true"}};
  return t;
}

bool loadSettings(const std::string &path, ParamsCarrier *p) {
  TomlMap t;
  if (!readToml(path, t)) return false;
  return applySettings(t, p);
}

// TomlSettings::parseFromSettings (TomlSettings.cpp:9-52)
bool applySettings(const TomlMap &tin, ParamsCarrier *p) {
  TomlMap t = tin;
  auto num = [&](const char *sec, const char *key, double &v) {
    auto s = t.find(sec);
    if (s == t.end() || !s->second.count(key)) { glog::error(std::string("Settings: missing ") + sec + "." + key); return false; }
    v = std::strtod(s->second[key].c_str(), nullptr);
    return true;
  };
  auto boolean = [&](const char *sec, const char *key, bool &v) {
    auto s = t.find(sec);
    if (s == t.end() || !s->second.count(key)) { glog::error(std::string("Settings: missing ") + sec + "." + key); return false; }
    v = (s->second[key] == "true");
    return true;
  };
  double k0, V, dt, rInj, injMax, thetaInj, spRatio, gRatio, k0Ratio, cDelta, tilt;
  bool uniform, removeLogs;
  if (!num("default_values", "K0", k0) || !num("default_values", "V", V) || !num("default_values", "dt", dt) ||
      !num("default_values", "r_injection", rInj) || !num("default_values", "uniform_energy_injection_maximum", injMax) ||
      !num("2d_models_common_settings", "theta_injection", thetaInj) ||
      !boolean("2d_models_common_settings", "use_uniform_injection", uniform) ||
      !num("SolarProp_like_model_settings", "SolarProp_ratio", spRatio) ||
      !num("Geliosphere_model_settings", "Geliosphere_ratio", gRatio) ||
      !num("Geliosphere_model_settings", "K0_ratio", k0Ratio) || !num("Geliosphere_model_settings", "C_delta", cDelta) ||
      !num("Geliosphere_model_settings", "default_tilt_angle", tilt) ||
      !boolean("advanced_settings", "remove_log_files_after_simulation", removeLogs))
    return false;
  p->putFloat("K0_default", (float)(k0 * 4.4683705e-27));
  p->putFloat("V_default", (float)(V * 6.68458712e-9));
  p->putFloat("dt_default", (float)dt);
  p->putFloat("r_injection", (float)rInj);
  p->putFloat("uniform_energy_injection_maximum", (float)injMax);
  p->putFloat("theta_injection", (float)thetaInj);
  p->putInt("use_uniform_injection", uniform ? 1 : 0);
  p->putFloat("solarPropRatio", (float)spRatio);
  p->putFloat("geliosphereRatio", (float)gRatio);
  p->putFloat("K0_ratio", (float)k0Ratio);
  p->putFloat("C_delta", (float)cDelta);
  p->putFloat("default_tilt_angle", (float)tilt);
  p->putInt("remove_log_files_after_simulation", removeLogs ? 1 : 0);
  return true;
}

// ---------------------------------------------------------------------------
// InputValidation / MeasureValuesTransformation
// ---------------------------------------------------------------------------
namespace validation {
bool checkDt(float dt) { return !(dt < 3.0 || dt > 5000.0); }
bool checkK0(float k0) { return !(k0 < 0.0); }
bool checkV(float v) { return !(v < 100.0 || v > 1500.0); }
bool checkN(int n) { return n > 0; }
void setDt(ParamsCarrier *p, float dt) { p->putFloat("dt", dt); }
void setK0(ParamsCarrier *p, float k0) {
  char buf[80];
  std::snprintf(buf, sizeof buf, "%g", k0);
  p->putString("K0input", buf);
  const float newK = k0 * 4.4683705e-27;
  p->putFloat("K0", newK);
  p->putInt("K0_entered_by_user", 1);
}
void setV(ParamsCarrier *p, float v) {
  p->putString("Vinput", std::to_string(v));
  const float newV = v * 6.68458712e-9;
  p->putFloat("V", newV);
}
void setN(ParamsCarrier *p, int n) { p->putInt("millions", n); }

void newSettingsLocationCheck(ParamsCarrier *p, const std::string &settings) {
  if (access(settings.c_str(), F_OK) == 0) loadSettings(settings, p);
  else glog::warn("No settings file exists on entered path.");
}

std::string monthName(int month) {
  static const char *names[] = {"NaN", "04", "12", "20", "29", "37", "45", "54", "62", "70", "79", "87", "95"};
  return (month >= 1 && month <= 12) ? names[month] : "NaN";
}

std::string carringtonRotation(int month, int year) {
  struct tm start = {};
  start.tm_year = 1976 - 1900; start.tm_mon = 5 - 1; start.tm_mday = 27;
  struct tm end = {};
  end.tm_year = year - 1900; end.tm_mon = month - 1; end.tm_mday = 15;
  const double seconds = difftime(mktime(&end), mktime(&start));
  double d = seconds / 2356560.0;
  double whole;
  const double frac = std::modf(d, &whole);
  d = (frac <= 0.5499) ? std::trunc(d) : std::ceil(d);
  return std::to_string((int)d + 1642);
}

void monthYearCheck(ParamsCarrier *p, int year, int month, const std::string &appPath) {
  p->putInt("month_option", month);
  p->putInt("year_option", year);
  const std::string model = p->getString("model", "1D Fp");
  const bool twoD = (model == "2D SolarProp-like" || model == "2D Geliosphere");
  const std::string table = (model == "2D SolarProp-like") ? "SolarProp_K0_phi_table.csv"
                            : (model == "2D Geliosphere") ? "Geliosphere_K0_phi_table.csv" : "K0_phi_table.csv";
  CsvTable t;
  if (!t.load(appPath + table)) {
    glog::error("Measured-value table " + appPath + table + " cannot be read.");
    return;
  }
  const std::string rowId = twoD ? carringtonRotation(month, year) : std::to_string(year) + "." + monthName(month);
  const std::string key = t.columns.empty() ? std::string() : t.columns[0];
  for (size_t r = 0; r < t.rows.size(); ++r) {
    if (t.str(key, r) != rowId) continue;
    p->putFloat("K0", (float)t.num("k0_au2/s", r));
    if (twoD) {
      p->putFloat("tilt_angle", (float)t.num("tilt_angle", r));
      p->putInt("polarity", (int)t.num("polarity", r));
    } else {
      p->putFloat("V", (float)(t.num("V", r) * 6.68458712e-9));
    }
    return;
  }
  glog::error("Combination for entered date was not found in input table.");
}
}  // namespace validation

// ---------------------------------------------------------------------------
// ParseParams (ParseParams.cpp:16-178)
// ---------------------------------------------------------------------------
static std::string applicationPath(char **argv) {
  std::string a = argv[0] ? argv[0] : "";
  const size_t slash = a.find_last_of('/');
  return (slash == std::string::npos) ? std::string("./") : a.substr(0, slash + 1);
}

int parseParams(int argc, char **argv, ParamsCarrier *p) {
  const std::string appPath = applicationPath(argv);
  p->putString("currentApplicationPath", appPath);
  struct Opt { bool set = false; std::string val; };
  std::map<std::string, Opt> o;
  auto canon = [](const std::string &a) -> std::string {
    static const std::map<std::string, std::string> alias = {
      {"-F", "forward"}, {"--forward", "forward"}, {"-B", "backward"}, {"--backward", "backward"},
      {"-E", "solarprop"}, {"--solarprop-like-model", "solarprop"}, {"-T", "geliosphere"},
      {"--geliosphere-2d-model", "geliosphere"}, {"-c", "csv"}, {"--csv", "csv"}, {"--evaluation", "evaluation"},
      {"--cpu-only", "cpu"}, {"-b", "batch"}, {"--batchrun", "batch"}, {"-d", "dt"}, {"--dt", "dt"},
      {"-K", "K0"}, {"--K0", "K0"}, {"-V", "V"}, {"--V", "V"}, {"-p", "path"}, {"--path", "path"},
      {"-N", "N"}, {"--number-of-test-particles", "N"}, {"-m", "month"}, {"--month", "month"},
      {"-y", "year"}, {"--year", "year"}, {"-s", "settings"}, {"--settings", "settings"},
      {"--custom-model", "custom"}};
    auto it = alias.find(a);
    return it == alias.end() ? std::string() : it->second;
  };
  static const std::set<std::string> flags = {"forward", "backward", "solarprop", "geliosphere", "csv", "cpu"};
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i], val;
    const size_t eq = a.find('=');
    if (a.rfind("--", 0) == 0 && eq != std::string::npos) { val = a.substr(eq + 1); a = a.substr(0, eq); }
    const std::string k = canon(a);
    if (k.empty()) { glog::error("The following argument was not expected: " + a); return -1; }
    o[k].set = true;
    if (!flags.count(k)) {
      if (val.empty()) {
        if (i + 1 >= argc) { glog::error(a + " requires an argument"); return -1; }
        val = argv[++i];
      }
      o[k].val = val;
    }
  }
  auto on = [&](const char *k) { return o.count(k) && o[k].set; };
  // exclusions (ParseParams.cpp:51-62)
  const char *models[] = {"forward", "backward", "solarprop", "geliosphere", "custom", "batch"};
  int nmodels = 0;
  for (auto m : models) nmodels += on(m);
  if (nmodels > 1) { glog::error("Model options exclude each other"); return -1; }
  if ((on("K0") || on("V")) && (on("month") || on("year"))) { glog::error("K0 / V exclude month / year"); return -1; }
  if (on("batch") && (on("dt") || on("N") || on("K0") || on("V") || on("month") || on("year"))) {
    glog::error("--batchrun excludes dt, N, K0, V, month and year"); return -1;
  }
  if (on("month") && !on("year")) { glog::error("--month requires --year"); return -1; }
  // The reference's "at least one model" check tests a pointer, so it never
  // fires and no model flag means the default model "1D Fp"
  // (ParseParams.cpp:66); kept.
  if (on("evaluation")) { p->putInt("run_simulation", 0); p->putString("pathToLogFile", o["evaluation"].val); }
  else p->putInt("run_simulation", 1);
  if (on("csv")) p->putInt("csv", 1);
  if (on("dt")) {
    const float dt = std::strtof(o["dt"].val.c_str(), nullptr);
    if (!validation::checkDt(dt)) { glog::error("dt is out of range!(3-5000)"); return false; }
    validation::setDt(p, dt);
  }
  if (on("K0")) {
    const float k0 = std::strtof(o["K0"].val.c_str(), nullptr);
    if (!validation::checkK0(k0)) { glog::error("K0 is out of range!(>0)"); return -1; }
    if (k0 < 1e19 || k0 > 1e23) glog::warn("K0 is out of recommended range!(1e19-1e23 cm^2/s)");
    validation::setK0(p, k0);
  }
  if (on("N")) {
    const int n = std::atoi(o["N"].val.c_str());
    if (!validation::checkN(n)) { glog::error("Number of test particles must be greater than 0!"); return -1; }
    validation::setN(p, n);
  }
  if (on("V")) {
    const float v = std::strtof(o["V"].val.c_str(), nullptr);
    if (!validation::checkV(v)) { glog::error("V is out of range!(100-1500 km/s)"); return -1; }
    validation::setV(p, v);
  }
  // Without -s the reference tests access("") and so never loads the
  // default Settings.toml (ParseParams.cpp:126-134); kept.
  if (on("settings")) validation::newSettingsLocationCheck(p, o["settings"].val);
  else glog::warn("No settings file exists on default path.");
  if (on("cpu")) p->putInt("isCpu", 1);
  if (on("path")) p->putString("destination", o["path"].val);
  if (on("forward")) p->putString("model", "1D Fp");
  else if (on("backward")) p->putString("model", "1D Bp");
  else if (on("solarprop")) p->putString("model", "2D SolarProp-like");
  else if (on("geliosphere")) p->putString("model", "2D Geliosphere");
  else if (on("custom")) p->putString("model", o["custom"].val);
  else if (on("batch")) {
    p->putString("model", "batch run");
    p->putString("inputBatchFile", o["batch"].val);
    return 1;
  }
  if (on("month") && on("year"))
    validation::monthYearCheck(p, std::atoi(o["year"].val.c_str()), std::atoi(o["month"].val.c_str()), appPath);
  glog::info("Chosen model:" + p->getString("model", "1D Fp"));
  return 1;
}
