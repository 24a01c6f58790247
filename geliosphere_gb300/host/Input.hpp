// Input layer with the reference's behaviour (Input/src/ParseParams.cpp:16-178,
// TomlSettings.cpp:9-52, InputValidation.cpp:58-152,
// MeasureValuesTransformation.cpp:14-115) written without CLI11 / toml11 /
// rapidcsv.
#pragma once
#include <map>
#include <string>
#include <vector>

class ParamsCarrier;

// Parse argv into the ParamsCarrier; 1 on success (the reference's contract).
int parseParams(int argc, char **argv, ParamsCarrier *p);

// Settings.toml subset: [section] key = number | true | false | "string".
using TomlMap = std::map<std::string, std::map<std::string, std::string>>;
bool readToml(const std::string &path, TomlMap &out);
// TomlSettings::parseFromSettings over parsed values; false if a key is missing.
bool applySettings(const TomlMap &t, ParamsCarrier *p);
bool loadSettings(const std::string &path, ParamsCarrier *p);
// The settings BatchRun falls back to when a row names no readable file
// (Algorithm/src/BatchRun.cpp:209-236; note K0_ratio 1.0 and uniform injection).
TomlMap batchDefaultSettings();

namespace validation {
bool checkDt(float dt);
bool checkK0(float k0);
bool checkV(float v);
bool checkN(int n);
void setDt(ParamsCarrier *p, float dt);
void setK0(ParamsCarrier *p, float k0);           // cm^2/s -> AU^2/s
void setV(ParamsCarrier *p, float v);             // km/s -> AU/s
void setN(ParamsCarrier *p, int n);
void newSettingsLocationCheck(ParamsCarrier *p, const std::string &settings);
void monthYearCheck(ParamsCarrier *p, int year, int month, const std::string &appPath);
std::string carringtonRotation(int month, int year);
std::string monthName(int month);
}  // namespace validation

// Minimal CSV reader with rapidcsv's conventions used by BatchRun: a header
// row, comma separator, numeric cells that fail to parse read as -1.
struct CsvTable {
  std::vector<std::string> columns;
  std::vector<std::vector<std::string>> rows;
  bool load(const std::string &path);
  bool has(const std::string &col) const;
  std::string str(const std::string &col, size_t row) const;
  double num(const std::string &col, size_t row) const;   // -1 if empty / not a number
};
