// TEST INFRASTRUCTURE: force-included before the reference sources built by
// oracle/Makefile (target `ref`).
//
// * std::random_device is replaced by a device that returns a seed chosen by
//   the harness, so the reference CPU models' thread_local std::mt19937
//   generators become reproducible;
// * `private` is opened so the harness can call the models' simulation()
//   blocks and drain their output queues directly.
// The standard headers are included first, so neither macro touches them.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <dirent.h>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>
#include <mutex>
#include <queue>
#include <random>
#include <set>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <sys/types.h>
#include <thread>
#include <unistd.h>
#include <vector>

namespace gelio_ref {
extern unsigned next_seed;
}

namespace std {
struct gelio_seeded_device {
  typedef unsigned int result_type;
  gelio_seeded_device() {}
  explicit gelio_seeded_device(const std::string &) {}
  result_type operator()() { return gelio_ref::next_seed; }
  double entropy() const noexcept { return 0.0; }
  static constexpr result_type min() { return 0u; }
  static constexpr result_type max() { return ~0u; }
};
}  // namespace std

#define random_device gelio_seeded_device
#define private public
