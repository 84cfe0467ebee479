// Index checks of the checked build (compiled with -DLMG_BOUNDS_CHECK): a
// failed check records a code and the offending index in this file's device
// status word and the access is skipped, so a bad index shows up as a status
// the host reads instead of a fault.  Without the macro every check is the
// constant true and the compiler removes it.
#pragma once
#include <cuda_runtime.h>

namespace lmg {

#ifdef LMG_BOUNDS_CHECK
// first failed check of this translation unit: (code << 48) | index
static __device__ unsigned long long g_bounds_status = 0;

__device__ __forceinline__ bool bounds_ok(bool ok, unsigned code, unsigned long long index) {
  if (!ok)
    atomicCAS(&g_bounds_status, 0ull,
              ((unsigned long long)code << 48) | (index & 0xffffffffffffull));
  return ok;
}
#define LMG_IN_BOUNDS(cond, code, index) \
  ::lmg::bounds_ok((cond), (code), (unsigned long long)(index))

// This translation unit's status word (0: no check failed), cleared if asked.
static inline unsigned long long bounds_status_here(bool reset) {
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, g_bounds_status, sizeof(v)) != cudaSuccess) {
    cudaGetLastError();
    return ~0ull;
  }
  if (reset) {
    const unsigned long long z = 0;
    cudaMemcpyToSymbol(g_bounds_status, &z, sizeof(z));
  }
  return v;
}
#else
#define LMG_IN_BOUNDS(cond, code, index) true
static inline unsigned long long bounds_status_here(bool) { return 0; }
#endif

// status words of the checked kernels' translation units
unsigned long long bounds_status_mdot_float(bool reset);
unsigned long long bounds_status_mdot_double(bool reset);
unsigned long long bounds_status_sym(bool reset);

}  // namespace lmg
