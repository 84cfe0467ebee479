// Bounded grid-wide barriers for cooperative launches (every block resident).
//
// grid_barrier: bar[0] counts arrivals, bar[1] is the generation.  The last
// block to arrive resets the count and advances the generation; the others
// spin on the generation with a bounded wait (about 1 s), after which the
// barrier reports failure instead of hanging, so the host can turn it into an
// error status.
#pragma once
#include <cuda_runtime.h>

namespace lmg {

constexpr long kBarrierSpins = 1L << 24;  // x >= 64 ns sleep: > 1 s

// Returns false if the wait ran out.
__device__ __forceinline__ bool grid_barrier(unsigned *bar) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      ok = 0;
      for (long it = 0; it < kBarrierSpins; it++) {
        if (*gen != g) {
          ok = 1;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Barrier on a 64-bit arrival count that only grows: every block adds one,
// and the launch's barrier is passed when the count reaches the next
// multiple of gridDim.x.  Launches that share a count must all have the same
// number of blocks and must not overlap (launches on one stream never do),
// so their arrivals never mix.  One atomic per block, no reset; the wait is
// bounded like grid_barrier's.
constexpr long kMonoSpins = 1L << 26;

__device__ __forceinline__ bool grid_barrier_mono(unsigned long long *count) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    // arrival with release semantics at GPU scope (cumulative: it publishes
    // the block's writes ordered before it by the __syncthreads above), polls
    // with acquire semantics (the __syncthreads below extends them to the
    // block): no separate fences on either side
    const unsigned long long g = gridDim.x;
    unsigned long long old;
    asm volatile("atom.release.gpu.add.u64 %0, [%1], 1;" : "=l"(old) : "l"(count) : "memory");
    const unsigned long long target = (old / g + 1) * g;
    int ok = 0;
    for (long it = 0; it < kMonoSpins; it++) {
      unsigned long long v;
      asm volatile("ld.acquire.gpu.u64 %0, [%1];" : "=l"(v) : "l"(count) : "memory");
      if (v >= target) {
        ok = 1;
        break;
      }
      if (it > 4096) __nanosleep(32);
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace lmg
