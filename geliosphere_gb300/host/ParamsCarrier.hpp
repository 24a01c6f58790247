// Process-wide parameter map with the interface of the reference's
// ParamsCarrier (Input/include/ParamsCarrier.hpp:127-345), so the host code
// around the engine reads like the reference: typed put/get with defaults, a
// singleton, and eraseAllItems for batch mode.  As in the reference,
// putInt / putFloat / putDouble do not overwrite an existing key (std::map
// insert semantics) while putString does.
#pragma once
#include <map>
#include <set>
#include <string>
#include <variant>

class ParamsCarrier {
 public:
  static ParamsCarrier *instance();

  void putString(const std::string &key, const std::string &value);
  void putFloat(const std::string &key, float value);
  void putInt(const std::string &key, int value);
  void putDouble(const std::string &key, double value);

  int getInt(const std::string &key, int defaultValue) const;
  float getFloat(const std::string &key, float defaultValue) const;
  double getDouble(const std::string &key, double defaultValue) const;
  std::string getString(const std::string &key, const std::string &defaultValue) const;

  // Remove every key that is not in `except`.
  void eraseAllItems(const std::set<std::string> &except);
  bool has(const std::string &key) const { return m_.count(key) != 0; }

 private:
  ParamsCarrier() = default;
  using Value = std::variant<std::string, int, float, double>;
  std::map<std::string, Value> m_;
};
