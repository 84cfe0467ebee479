// Measurement hooks (not part of the public header):
//   * a count of the kernels this library has launched, so a benchmark can
//     state how many of its kernels ran inside a timed region;
//   * an FP32 FMA-chain kernel whose throughput is the FP32 peak the pair
//     kernel's roofline is quoted against (measured on the same GPU, same
//     clocks, in the same run);
//   * a check that the bounded grid barrier of the fused Lanczos step gives
//     up and reports instead of waiting forever.
#include <atomic>
#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

#include "krylov.cuh"
#include "bounds.cuh"
#include "common.hpp"
#include "launch_count.hpp"
#include "mdot_sym.cuh"

namespace lmg {
std::atomic<unsigned long long> g_launches{0};
std::atomic<int> g_force_tpt{0}, g_force_split{0};
std::atomic<int> g_sym_mode{0}, g_sym_warps{0}, g_sym_variant{0};
std::atomic<unsigned long long *> g_sym_trace{nullptr};
std::atomic<int> g_lanczos_device_sqrt{2};
std::atomic<int> g_lanczos_lookahead{0};
std::atomic<int> g_lanczos_check_wait{0};
std::atomic<int> g_precond_tc{0};
std::atomic<int> g_lanczos_step_mode{0};
std::atomic<int> g_lanczos_step_shape{0};
}

namespace {
// 8 independent FMA chains per thread, `iters` rounds of 8 FMAs each
// (2 flops per FMA).  The result is written only if it is the impossible
// value -1 so the compiler must keep the chains.
__global__ void fma_chain_kernel(int iters, float *sink) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = (threadIdx.x + k) * 1e-7f;
  const float b = 0.999999f, c = 1e-8f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int r = 0; r < 8; r++) {
#pragma unroll
      for (int k = 0; k < 8; k++) a[k] = fmaf(a[k], b, c);
    }
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  if (s == -1.0f) sink[threadIdx.x] = s;
}
// Same with packed FP32 (fma.rn.f32x2 through __ffma2_rn): 4 independent
// float2 chains, so the same 8 FMAs per round per thread.
__global__ void fma2_chain_kernel(int iters, float *sink) {
  float2 a[4];
#pragma unroll
  for (int k = 0; k < 4; k++) a[k] = make_float2((threadIdx.x + k) * 1e-7f, k * 1e-7f);
  const float2 b = make_float2(0.999999f, 0.999999f), c = make_float2(1e-8f, 1e-8f);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int r = 0; r < 8; r++) {
#pragma unroll
      for (int k = 0; k < 4; k++) a[k] = __ffma2_rn(a[k], b, c);
    }
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) s += a[k].x + a[k].y;
  if (s == -1.0f) sink[threadIdx.x] = s;
}

// FP64: 8 independent DFMA chains per thread, the same structure.
__global__ void dfma_chain_kernel(int iters, double *sink) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = (threadIdx.x + k) * 1e-7;
  const double b = 0.999999, c = 1e-8;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int r = 0; r < 8; r++) {
#pragma unroll
      for (int k = 0; k < 8; k++) a[k] = fma(a[k], b, c);
    }
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  if (s == -1.0) sink[threadIdx.x] = s;
}

// A check whose condition is false, on an index it never uses: in the
// checked build it records code 99 (nothing is accessed).
__global__ void bounds_probe_kernel(int limit) {
  const int idx = limit + (int)threadIdx.x;
  if (LMG_IN_BOUNDS(idx < limit, 99, idx)) asm volatile("" ::"r"(idx));
}

// Two blocks meet at a barrier whose arrival count starts at 7: neither is
// the last arrival, nothing advances the generation word, so both waits run
// out and report.
__global__ void barrier_timeout_kernel(unsigned *bar, double *flag) {
  if (!lmg::grid_barrier(bar) && threadIdx.x == 0) flag[blockIdx.x] = 1.0;
}
}  // namespace

extern "C" {

unsigned long long lmg_internal_launch_count(void) { return lmg::g_launches.load(); }

// Forces targets-per-thread (1 or 2) and the source split count of every
// all-pairs launch planned after the call; 0 restores the planner's choice.
// Plans cached by existing solvers are re-made on their next call.
int lmg_internal_mdot_plan_override(int tpt, int nsplit) {
  if (tpt < 0 || tpt > 2 || nsplit < 0 || nsplit > 65535) return 1;
  lmg::g_force_tpt.store(tpt);
  lmg::g_force_split.store(nsplit);
  return 0;
}

// Symmetric open-space product of FP32 handles: mode 0 uses it wherever it
// applies (open boundary, forces only, no angular part, 16-byte aligned
// forces, batches of a multiple of 4 particles or a single batch), mode 1
// always takes mdot_kernel; warps > 0 caps the number of warps its rotation
// steps are spread over (tests cut tile pairs at many places with it).
// Modes 2, 3 and 4 instead pick the kernel build for 2, 3 or 4 resident
// blocks per SM (register budget), leaving the rest as it is.  Applies to the
// next product of every handle.
int lmg_internal_sym_override(int mode, int warps) {
  if (mode < 0 || mode > 4 || warps < 0) return 1;
  if (mode >= 2) {
    lmg::g_sym_variant.store(mode);
    return 0;
  }
  lmg::g_sym_mode.store(mode);
  lmg::g_sym_warps.store(warps);
  return 0;
}

// Host tables of the symmetric kernel's schedule for `resident` resident
// blocks (no device needed).  info[0..8] receives nwarps, tile pairs, tiles,
// slots, threads per element of the fold, blocks, rotation steps, tiles per
// batch and slots per tile; the arrays (pairs: 4 ints per pair, pseg: 1 per
// pair, warps: 8 per warp, tused: 1 per tile) are filled when not null.
// Returns 0, or 2 when the shape does not suit the kernel.
int lmg_internal_sym_plan(int N, int nper, long long resident, int force_warps, long long *info,
                          int *pairs, int *pseg, int *warps, int *tused) {
  lmg::SymPlan p;
  const cudaError_t e = lmg::mdot_sym_plan_tables(N, nper, resident, force_warps, p);
  if (e == cudaErrorNotSupported) return 2;
  if (e != cudaSuccess || !info) return 1;
  info[0] = p.nwarps;
  info[1] = (long long)p.pairs.size();
  info[2] = (long long)p.tused.size();
  info[3] = (long long)p.slots;
  info[4] = p.rt;
  info[5] = p.grid;
  info[6] = p.steps;
  info[7] = p.tpb;
  info[8] = p.cmax;
  if (pairs) std::memcpy(pairs, p.pairs.data(), p.pairs.size() * sizeof(int4));
  if (pseg) std::memcpy(pseg, p.pseg.data(), p.pseg.size() * sizeof(int));
  if (warps) std::memcpy(warps, p.warps.data(), p.warps.size() * sizeof(int4));
  if (tused) std::memcpy(tused, p.tused.data(), p.tused.size() * sizeof(int));
  return 0;
}

// Where the single-system Lanczos takes T^{1/2} e1 at its checks: 0 the
// exact QL on the host; 1 on the device by quadrature; 2 (the default) on
// the host by quadrature; the host QL wherever a quadrature does not apply.
// Applies to the next solves of every handle.  (Measured at N = 4096, FP32,
// tolerance 1e-6: 4.7 ms per solve with the host QL, 2.6 ms with the host
// quadrature (18 against 296 us a check at m = 80 on a Grace core), 7.9 ms
// on the device: there the quadrature is a chain of FP64 divisions on
// GB300's narrow FP64 units.)
int lmg_internal_lanczos_device_sqrt(int on) {
  if (on < 0 || on > 2) return 1;
  lmg::g_lanczos_device_sqrt.store(on);
  return 0;
}

// Iterations the single-system Lanczos issues ahead of the check it is
// evaluating: 1..4, or 0 for the default (3 for batches of up to 8192
// particles, else 1).
int lmg_internal_lanczos_lookahead(int n) {
  if (n < 0 || n > 4) return 1;
  lmg::g_lanczos_lookahead.store(n);
  return 0;
}

// What each check kernel of the single-system Lanczos waits for: 0 the end
// of its iteration, 1 the end of the next iteration's matrix-vector product
// (it then shares the GPU with the next vector step instead of the next
// product).  Results are the same either way.
int lmg_internal_lanczos_check_wait(int mode) {
  if (mode != 0 && mode != 1) return 1;
  lmg::g_lanczos_check_wait.store(mode);
  return 0;
}

// The decision behind every buffer check (0 host, 1 current GPU or managed,
// -1 another GPU's memory) for given pointer attributes, so that it can be
// checked without a second GPU.
int lmg_internal_classify_pointer(int type, int ptr_device, int current_device) {
  return lmg::classify_pointer(type, ptr_device, current_device);
}

// Status words of the checked build (compiled with -DLMG_BOUNDS_CHECK; 0 in
// the normal build): the first failed index check of the all-pairs kernels
// (FP32 and FP64) and of the symmetric kernel, as (code << 48) | index;
// reset clears them.
unsigned long long lmg_internal_bounds_status(int which, int reset) {
  switch (which) {
    case 0: return lmg::bounds_status_mdot_float(reset != 0);
    case 1: return lmg::bounds_status_mdot_double(reset != 0);
    case 2: return lmg::bounds_status_sym(reset != 0);
    default: return lmg::bounds_status_here(reset != 0);
  }
}

// Runs a check that fails on purpose without any access (which = 3 then
// reads it back); returns the CUDA status.
int lmg_internal_bounds_probe(void) {
  bounds_probe_kernel<<<1, 32>>>(1000);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return (int)e;
}

// Lanczos vector step of the single-system solver: 0 one cluster (default),
// 1 the cooperative grid-wide launch.
int lmg_internal_lanczos_step_mode(int mode) {
  if (mode != 0 && mode != 1) return 1;
  lmg::g_lanczos_step_mode.store(mode);
  return 0;
}

// Cluster shape of that step: ctas in 1..16 and threads a multiple of 32 in
// 32..1024, or 0, 0 for the default.
int lmg_internal_lanczos_step_shape(int ctas, int threads) {
  if (ctas == 0 && threads == 0) {
    lmg::g_lanczos_step_shape.store(0);
    return 0;
  }
  if (ctas < 1 || ctas > 16 || threads < 32 || threads > 1024 || threads % 32) return 1;
  lmg::g_lanczos_step_shape.store((ctas << 16) | threads);
  return 0;
}

// Timeline of the symmetric kernel's next launches (null: off): buf is a
// device array of at least 2 x warps + 3 x blocks 64-bit values of the
// launch's grid (per warp its start and end in %globaltimer nanoseconds, per
// block the end of its barrier wait and of its fold, per block its SM).
int lmg_internal_sym_trace(void *buf) {
  lmg::g_sym_trace.store(static_cast<unsigned long long *>(buf));
  return 0;
}

// Launches blocks x threads of the FMA chain on `stream`; flops performed =
// blocks * threads * iters * 64 * 2.
int lmg_internal_fma_probe(int blocks, int threads, int iters, void *sink, void *stream) {
  fma_chain_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, (float *)sink);
  return (int)cudaGetLastError();
}

// Packed variant: the same flop count as lmg_internal_fma_probe.
int lmg_internal_fma2_probe(int blocks, int threads, int iters, void *sink, void *stream) {
  fma2_chain_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, (float *)sink);
  return (int)cudaGetLastError();
}

// FP64 variant: flops performed = blocks * threads * iters * 64 * 2.
int lmg_internal_dfma_probe(int blocks, int threads, int iters, void *sink, void *stream) {
  dfma_chain_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, (double *)sink);
  return (int)cudaGetLastError();
}

// Runs barrier_timeout_kernel (about 1-2 s) and returns in *gave_up the
// number of blocks whose wait ran out (2 expected); the return value is the
// CUDA status, so the context is shown usable afterwards.
int lmg_internal_barrier_timeout_probe(int *gave_up) {
  if (!gave_up) return 1;
  *gave_up = -1;
  unsigned *bar = nullptr;
  double *flag = nullptr;
  cudaError_t e = cudaMalloc(&bar, 2 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&flag, 2 * sizeof(double));
  const unsigned init[2] = {7u, 0u};
  if (e == cudaSuccess) e = cudaMemcpy(bar, init, sizeof(init), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(flag, 0, 2 * sizeof(double));
  if (e == cudaSuccess) {
    barrier_timeout_kernel<<<2, 32>>>(bar, flag);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  double h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, flag, sizeof(h), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) *gave_up = (int)(h[0] + h[1]);
  if (bar) cudaFree(bar);
  if (flag) cudaFree(flag);
  return (int)e;
}
}
