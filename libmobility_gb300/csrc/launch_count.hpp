// Count of kernels launched by this library (see probes.cu).
#pragma once
#include <atomic>

namespace lmg {
extern std::atomic<unsigned long long> g_launches;
inline void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
}  // namespace lmg
