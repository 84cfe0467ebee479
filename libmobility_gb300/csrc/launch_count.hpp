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
// symmetric open-space product: g_sym_mode 0 = used where it applies, 1 = off;
// g_sym_warps > 0 caps the warps its steps are spread over; g_sym_variant is
// its register budget, 2, 3 or 4 resident blocks per SM (0 = default, 2)
extern std::atomic<int> g_sym_mode, g_sym_warps, g_sym_variant;
// T^{1/2} e1 of the single-system Lanczos checks: 0 (default) the exact host
// QL; 1 on the device by quadrature, the host QL where that falls back
extern std::atomic<int> g_lanczos_device_sqrt;
// iterations issued ahead of a check (0 = by batch size: 3 up to 8192 particles, else 1)
extern std::atomic<int> g_lanczos_lookahead;
// device buffer for the symmetric kernel's timeline (null = off)
extern std::atomic<unsigned long long *> g_sym_trace;
}  // namespace lmg
