// TEST INFRASTRUCTURE: no-op stand-in for the spdlog logging header, so the
// reference's CPU models and evaluators compile from source without the
// spdlog dependency (which is not installed and cannot be fetched here).
#pragma once
namespace spdlog {
template <class... A> inline void info(A &&...) {}
template <class... A> inline void warn(A &&...) {}
template <class... A> inline void error(A &&...) {}
template <class... A> inline void debug(A &&...) {}
}  // namespace spdlog
