// compat_common.h -- status bookkeeping shared by the compatibility libraries.
#pragma once
#include <atomic>
#include <cstdio>

#include "../../include/advdiff.h"

namespace adv_compat {
inline std::atomic<int>& last_status() {
  static std::atomic<int> s{0};
  return s;
}
// The reference's wrappers return void; a failure is printed once and kept for
// adv_compat_last_status() instead of exiting the process.
inline void note(adv_status s, const char* what) {
  if (s == ADV_OK) return;
  int expected = 0;
  if (last_status().compare_exchange_strong(expected, (int)s))
    std::fprintf(stderr, "advdiff compat: %s failed: %s (%s)\n", what, adv_status_string(s), adv_last_error_string());
}
inline int take_status() { return last_status().exchange(0); }
}  // namespace adv_compat
