#include "ParamsCarrier.hpp"

ParamsCarrier *ParamsCarrier::instance() {
  static ParamsCarrier *inst = new ParamsCarrier();
  return inst;
}

void ParamsCarrier::putString(const std::string &key, const std::string &value) {
  auto it = m_.find(key);
  if (it != m_.end() && std::holds_alternative<std::string>(it->second)) {
    it->second = value;
    return;
  }
  m_.insert({key, Value(value)});
}
void ParamsCarrier::putFloat(const std::string &key, float value) { m_.insert({key, Value(value)}); }
void ParamsCarrier::putInt(const std::string &key, int value) { m_.insert({key, Value(value)}); }
void ParamsCarrier::putDouble(const std::string &key, double value) { m_.insert({key, Value(value)}); }

template <class T>
static T get_as(const std::map<std::string, std::variant<std::string, int, float, double>> &m,
                const std::string &key, T def) {
  auto it = m.find(key);
  if (it == m.end() || !std::holds_alternative<T>(it->second)) return def;
  return std::get<T>(it->second);
}

int ParamsCarrier::getInt(const std::string &key, int d) const { return get_as<int>(m_, key, d); }
float ParamsCarrier::getFloat(const std::string &key, float d) const { return get_as<float>(m_, key, d); }
double ParamsCarrier::getDouble(const std::string &key, double d) const { return get_as<double>(m_, key, d); }
std::string ParamsCarrier::getString(const std::string &key, const std::string &d) const {
  return get_as<std::string>(m_, key, d);
}

void ParamsCarrier::eraseAllItems(const std::set<std::string> &except) {
  for (auto it = m_.begin(); it != m_.end();) {
    if (except.count(it->first)) ++it;
    else it = m_.erase(it);
  }
}
