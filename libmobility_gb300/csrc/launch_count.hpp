// Count of kernels launched by this library, and the process-wide override of
// the all-pairs launch plan used by tuning sweeps and plan-invariance tests
// (both defined in probes.cu).
#pragma once
#include <atomic>

namespace lmg {
extern std::atomic<unsigned long long> g_launches;
inline void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
// 0 = planner's choice
extern std::atomic<int> g_force_tpt, g_force_split;
}  // namespace lmg
