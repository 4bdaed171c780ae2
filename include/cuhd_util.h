// Utilities of the reference API (include/cuhd_util.h:20-44): timing,
// comparison, ceiling division.  time() returns microseconds measured with
// CUDA events (the reference truncates to whole milliseconds,
// src/multians_util.cc:59; this one does not).
#ifndef CUHD_UTIL_
#define CUHD_UTIL_

#include <chrono>
#include <cstddef>
#include <functional>
#include <string>
#include <utility>

#include "cuhd_constants.h"

#define SDIV(n, m) (((n) + (m) - 1) / (m))

#define TIMER_START(vec, label) vec.push_back(cuhd::CUHDUtil::time(label, [&]() {
#define TIMER_STOP }));

namespace cuhd {
class CUHDUtil {
public:
    static std::pair<std::string, size_t> time(std::string s, std::function<void()> f);
    static bool equals(SYMBOL_TYPE* a, SYMBOL_TYPE* b, size_t size);
    static size_t optimal_subsequence_size(size_t input_size, size_t output_size, size_t pref,
                                           size_t device_pref);
};
}  // namespace cuhd

#endif
