/*
 * Loads the cubin of libMobility's own NBody "fast" kernel
 * (oracle/_ref/ref_nbody_{f,d}.cubin, made by oracle/build.py from
 * solvers/NBody/extra/NbodyRPY.cu) and launches it with the launch shape of the
 * reference launcher computeRPYBatchedFast (NbodyRPY.cu:99-116).
 *
 * TEST INFRASTRUCTURE ONLY.  Used by the GPU parity tests (the reference
 * kernel is the parity target for libmobility_gb300's Mdot on the same GPU)
 * and by oracle/time_reference_gpu.py.  It runs in the CUDA primary context
 * that the calling process (PyTorch) already uses.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>
#include <string>

namespace {
struct KernelPair {
  CUlibrary lib = nullptr;
  CUkernel open = nullptr, wall = nullptr;
  bool loaded = false;
};
KernelPair g_mod[2]; /* [0] float build, [1] double build */
char g_err[512] = "";

template <class R> struct Constants { R t0, r0, rt0, rh; }; /* hydrodynamicKernels.cuh:20-25 */
struct Blocks { bool useUF, useWT, useUT, useWF; };         /* hydrodynamicKernels.cuh:27-32 */

int fail(const char *what, CUresult r) {
  const char *s = nullptr;
  cuGetErrorString(r, &s);
  std::snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
  return 1;
}
} // namespace

extern "C" const char *ref_gpu_last_error() { return g_err; }

/* Loads the cubin for one precision and finds the two fast-kernel
 * instantiations (open boundary, bottom wall) by name. */
extern "C" int ref_gpu_load(int dbl, const char *cubin_path) {
  cudaFree(0); /* make the primary context current, as PyTorch does */
  KernelPair &m = g_mod[dbl ? 1 : 0];
  if (m.loaded) return 0;
  CUresult r = cuLibraryLoadFromFile(&m.lib, cubin_path, nullptr, nullptr, 0,
                                     nullptr, nullptr, 0);
  if (r != CUDA_SUCCESS) return fail("cuLibraryLoadFromFile", r);
  unsigned int count = 0;
  r = cuLibraryGetKernelCount(&count, m.lib);
  if (r != CUDA_SUCCESS) return fail("cuLibraryGetKernelCount", r);
  CUkernel ks[64];
  if (count > 64) count = 64;
  r = cuLibraryEnumerateKernels(ks, count, m.lib);
  if (r != CUDA_SUCCESS) return fail("cuLibraryEnumerateKernels", r);
  for (unsigned int i = 0; i < count; i++) {
    const char *name = nullptr;
    if (cuKernelGetName(&name, ks[i]) != CUDA_SUCCESS || !name) continue;
    std::string s(name);
    if (s.find("computeRPYBatchedFastGPU") == std::string::npos) continue;
    if (s.find("OpenBoundary") != std::string::npos) m.open = ks[i];
    if (s.find("BottomWall") != std::string::npos) m.wall = ks[i];
  }
  if (!m.open || !m.wall) {
    std::snprintf(g_err, sizeof(g_err), "fast kernels not found in %s", cubin_path);
    return 1;
  }
  m.loaded = true;
  return 0;
}

/* One reference Mdot on device buffers (real3 interleaved).  F or T may be
 * NULL (absent); U, W likewise.  Block flags as in callBatchedNBody
 * (NbodyRPY.cu:264-275).  Launch shape of computeRPYBatchedFast. */
extern "C" int ref_gpu_mdot(int dbl, int wall, const void *pos, const void *F,
                            const void *T, void *U, void *W, int Nbatches,
                            int NperBatch, double t0, double r0, double rt0,
                            double a, int includeAngular, void *stream) {
  KernelPair &m = g_mod[dbl ? 1 : 0];
  if (!m.loaded) {
    std::snprintf(g_err, sizeof(g_err), "cubin not loaded");
    return 1;
  }
  Blocks b{false, false, false, false};
  if (F) { b.useUF = true; if (includeAngular) b.useWF = true; }
  if (T && includeAngular) { b.useWT = true; b.useUT = true; }
  const int N = Nbatches * NperBatch;
  const size_t real3size = dbl ? 3 * sizeof(double) : 3 * sizeof(float);
  int nearestWarpMultiple = ((NperBatch + 16) / 32) * 32;
  int minBlockSize = nearestWarpMultiple > 32 ? nearestWarpMultiple : 32;
  int Nthreads = minBlockSize < N ? minBlockSize : N;
  if (Nthreads > 256) Nthreads = 256;
  int Nblocks = (N + Nthreads - 1) / Nthreads;
  int factor = 1 + (F != nullptr) + (T != nullptr);
  unsigned int smem = (unsigned int)(factor * Nthreads * real3size);
  Constants<float> cf{(float)t0, (float)r0, (float)rt0, (float)a};
  Constants<double> cd{t0, r0, rt0, a};
  void *args[9];
  args[0] = (void *)&pos;
  args[1] = (void *)&F;
  args[2] = (void *)&T;
  args[3] = (void *)&U;
  args[4] = (void *)&W;
  args[5] = dbl ? (void *)&cd : (void *)&cf;
  args[6] = (void *)&b;
  args[7] = (void *)&Nbatches;
  args[8] = (void *)&NperBatch;
  CUfunction fn;
  CUresult r = cuKernelGetFunction(&fn, wall ? m.wall : m.open);
  if (r != CUDA_SUCCESS) return fail("cuKernelGetFunction", r);
  r = cuLaunchKernel(fn, Nblocks, 1, 1, Nthreads, 1, 1, smem, (CUstream)stream,
                     args, nullptr);
  if (r != CUDA_SUCCESS) return fail("cuLaunchKernel", r);
  return 0;
}
