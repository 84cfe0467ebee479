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

#include <cuda_runtime.h>

#include "krylov.cuh"
#include "launch_count.hpp"

namespace lmg {
std::atomic<unsigned long long> g_launches{0};
std::atomic<int> g_force_tpt{0}, g_force_split{0};
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
