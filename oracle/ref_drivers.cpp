/*
 * Thin C drivers around libMobility's OWN source code, compiled for the CPU of
 * this container from the files where they lie in the reference checkout
 * (nothing is copied).  TEST INFRASTRUCTURE ONLY: they exist to pin the
 * oracle (rpy_oracle.c, oracle.py) against the reference itself and to write
 * the golden fixtures under tests/golden/.
 *
 * REF_PAIR    builds the reference pair physics
 *             (solvers/NBody/extra/hydrodynamicKernels.cuh) into an all-pairs
 *             batched product that follows NbodyRPY.cu:119-147 and the block
 *             selection of NbodyRPY.cu:264-275.
 * REF_LANCZOS builds the reference Krylov solver
 *             (include/lanczos/LanczosAlgorithm.{h,cu}) against host stand-ins
 *             for cuBLAS, CBLAS, LAPACKE and thrust (oracle/ref_shim/).
 *
 * `real` is float unless DOUBLE_PRECISION is defined, as in the reference.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>

#ifdef REF_PAIR
#include <algorithm>
#include "cuda_runtime.h"
/* host versions of the device intrinsics the pair code names */
static inline float rsqrt(float x) { return 1.0f / std::sqrt(x); }
static inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
using std::max;
using std::min;
#include "solvers/NBody/extra/hydrodynamicKernels.cuh"

using nbody_rpy::real;
using nbody_rpy::make_real3;
using nbody_rpy::real3;

template <class Kernel>
static void ref_all_pairs(const real *pos, const real *F, const real *T,
                          real *U, real *W, int64_t N, int64_t NperBatch,
                          nbody_rpy::Constants c, nbody_rpy::blocksToCompute b) {
  for (int64_t i = 0; i < N; i++) {
    real3 pi = make_real3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    real3 MF = make_real3(0, 0, 0), MT = make_real3(0, 0, 0);
    int64_t b0 = (i / NperBatch) * NperBatch;
    for (int64_t j = b0; j < b0 + NperBatch && j < N; j++) {
      real3 pj = make_real3(pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]);
      real3 fj = F ? make_real3(F[3 * j], F[3 * j + 1], F[3 * j + 2]) : make_real3(0, 0, 0);
      real3 tj = T ? make_real3(T[3 * j], T[3 * j + 1], T[3 * j + 2]) : make_real3(0, 0, 0);
      nbody_rpy::mdot_result r = Kernel::dotProduct(pi, pj, fj, tj, c, b);
      MF += r.MF;
      MT += r.MT;
    }
    if (U) { U[3 * i] = MF.x; U[3 * i + 1] = MF.y; U[3 * i + 2] = MF.z; }
    if (W) { W[3 * i] = MT.x; W[3 * i + 1] = MT.y; W[3 * i + 2] = MT.z; }
  }
}

/* pos is in the wall frame (wall at z = 0).  F or T may be NULL.  Block flags
 * as in callBatchedNBody, NbodyRPY.cu:264-275. */
extern "C" int ref_pair_mdot(int wall, const real *pos, const real *F,
                             const real *T, real *U, real *W, int64_t N,
                             int64_t NperBatch, double t0, double r0,
                             double rt0, double a, int includeAngular) {
  nbody_rpy::Constants c{real(t0), real(r0), real(rt0), real(a)};
  nbody_rpy::blocksToCompute b;
  if (F) { b.useUF = true; if (includeAngular) b.useWF = true; }
  if (T && includeAngular) { b.useWT = true; b.useUT = true; }
  if (wall)
    ref_all_pairs<nbody_rpy::BottomWall>(pos, F, T, U, W, N, NperBatch, c, b);
  else
    ref_all_pairs<nbody_rpy::OpenBoundary>(pos, F, T, U, W, N, NperBatch, c, b);
  return 0;
}
extern "C" int ref_real_size() { return (int)sizeof(real); }
#endif

#ifdef REF_LANCZOS
#include "lanczos/LanczosAlgorithm.h"
using lanczos::real;

struct ref_lanczos_handle {
  lanczos::Solver solver;
};

extern "C" void *ref_lanczos_new(int hard_limit) {
  auto *h = new ref_lanczos_handle();
  if (hard_limit > 0) h->solver.setIterationHardLimit(hard_limit);
  return h;
}
extern "C" void ref_lanczos_free(void *h) { delete (ref_lanczos_handle *)h; }

/* Runs the reference solver for y = sqrt(M) z with a dense row-major n x n
 * matrix M (in `real`).  The matrix-vector product accumulates in `real`.
 * residuals[k] receives the error reported to the callback at each check (up
 * to max_res entries; checked_iters[k] the iteration).  Returns the iteration
 * index the solver returned, or -1 on an exception (message in err). */
extern "C" int ref_lanczos_solve(void *hp, const real *M, int n, const real *z,
                                 double tol, real *y, double *residuals,
                                 int *checked_iters, int max_res, int *n_res,
                                 char *err, int err_len) {
  auto *h = (ref_lanczos_handle *)hp;
  lanczos::Dot dot = [M, n](real *v, real *w) {
    for (int i = 0; i < n; i++) {
      real s = 0;
      for (int j = 0; j < n; j++) s += M[(int64_t)i * n + j] * v[j];
      w[i] = s;
    }
  };
  int count = 0;
  lanczos::Callback cb = [&](int it, real res) {
    if (count < max_res) {
      residuals[count] = res;
      checked_iters[count] = it;
    }
    count++;
  };
  try {
    int it = h->solver.run(dot, y, z, real(tol), n, cb);
    *n_res = count;
    return it;
  } catch (std::exception &e) {
    *n_res = count;
    if (err && err_len > 0) {
      std::strncpy(err, e.what(), err_len - 1);
      err[err_len - 1] = 0;
    }
    return -1;
  }
}

/* Same, without a callback, so that the solver's adaptive convergence-check
 * schedule (LanczosAlgorithm.cu:179-184,224-232) is exercised. */
extern "C" int ref_lanczos_solve_nocb(void *hp, const real *M, int n,
                                      const real *z, double tol, real *y,
                                      char *err, int err_len) {
  auto *h = (ref_lanczos_handle *)hp;
  lanczos::Dot dot = [M, n](real *v, real *w) {
    for (int i = 0; i < n; i++) {
      real s = 0;
      for (int j = 0; j < n; j++) s += M[(int64_t)i * n + j] * v[j];
      w[i] = s;
    }
  };
  lanczos::Callback cb;
  try {
    return h->solver.run(dot, y, z, real(tol), n, cb);
  } catch (std::exception &e) {
    if (err && err_len > 0) {
      std::strncpy(err, e.what(), err_len - 1);
      err[err_len - 1] = 0;
    }
    return -1;
  }
}
extern "C" int ref_real_size() { return (int)sizeof(real); }
#endif
