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
// T^{1/2} e1 of the single-system Lanczos checks: 0 the exact host QL; 1 on
// the device by quadrature; 2 (default) on the host by quadrature; the host
// QL wherever a quadrature falls back
extern std::atomic<int> g_lanczos_device_sqrt;
// iterations issued ahead of a check (0 = by batch size: 3 up to 8192 particles, else 1)
extern std::atomic<int> g_lanczos_lookahead;
// what the check kernel of iteration i waits for on the side stream: 0 the
// end of iteration i; 1 the end of iteration i + 1's matrix-vector product
// where that was issued (it then runs beside iteration i + 1's vector step)
extern std::atomic<int> g_lanczos_check_wait;
// the single-system Lanczos vector step: 0 (default) one thread-block
// cluster, 1 the cooperative grid-wide launch
extern std::atomic<int> g_lanczos_step_mode;
// its cluster shape, (CTAs << 16) | threads per CTA (0 = the largest cluster
// of kClusterThreads-thread CTAs that fits)
extern std::atomic<int> g_lanczos_step_shape;
// network layers of the preconditioner build on the tensor cores (tcgen05,
// TF32): 1 on, 0 the CUDA-core FP32 GEMM
extern std::atomic<int> g_precond_tc;
// device buffer for the symmetric kernel's timeline (null = off)
extern std::atomic<unsigned long long *> g_sym_trace;
}  // namespace lmg
