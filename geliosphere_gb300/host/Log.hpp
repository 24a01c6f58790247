// Minimal leveled logging for the host layer (the reference uses spdlog's
// info / warn / error, e.g. GeliosphereModel.cu:404-448).
#pragma once
#include <cstdio>
#include <string>

namespace glog {
inline bool &quiet() { static bool q = false; return q; }
inline void info(const std::string &m) { if (!quiet()) std::fprintf(stderr, "[info] %s\n", m.c_str()); }
inline void warn(const std::string &m) { std::fprintf(stderr, "[warning] %s\n", m.c_str()); }
inline void error(const std::string &m) { std::fprintf(stderr, "[error] %s\n", m.c_str()); }
}  // namespace glog
