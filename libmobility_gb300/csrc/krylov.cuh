// Device side of the Lanczos evaluation of sqrt(M) dW.
//
// Follows the algorithm of libMobility include/lanczos/LanczosAlgorithm.cu
// (Ando, Chow, Saad, Skolnick 2012):
//   v0 = z/|z|                                     setFirstBasisVector :110-118
//   w = M v_i - beta_{i-1} v_{i-1}; alpha_i = w.v_i; w -= alpha_i v_i;
//   beta_i = |w|, zeroed if beta_i < 1e-3 alpha_i/|z| (then v_{i+1} = e1),
//   v_{i+1} = w/beta_i                             nextIteration :120-153
//   y = |z| V_m T_m^{1/2} e1                       computeCurrentResultEstimation :158-167
//   err = |y_i - y_{i-1}| / |y_{i-1}|              computeError :202-222
// GB300 choices: the Krylov vectors stay in the solver precision, every inner
// product and norm accumulates in FP64 and the scalars alpha, beta, |z| live in
// device memory as FP64.  The m x m tridiagonal eigen-problem behind
// T_m^{1/2} e1 (m <= 250) is solved in FP64 by implicit QL (below) on the Grace
// host core, whose scalar FP64 latency is far below that of GB300's narrow FP64
// units; alpha/beta reach it through mapped host memory while the GPU already
// runs the next matrix-vector product.
#pragma once
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "grid_sync.cuh"

namespace lmg {

// ---------------------------------------------------------------------------
// Gaussian noise: Philox4x32-10 counter-based generator (Salmon, Moraes,
// Dror, Shaw, SC'11) + Box-Muller.  Stream = (seed1, seed2), element i.
// ---------------------------------------------------------------------------
struct Philox {
  static __host__ __device__ __forceinline__ void round(uint32_t c[4], uint32_t k[2]) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k[0];
    const uint32_t n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k[0] += 0x9E3779B9u;
    k[1] += 0xBB67AE85u;
  }
  static __host__ __device__ __forceinline__ void gen(uint32_t ctr, uint32_t s1, uint32_t s2,
                                                      uint32_t out[4]) {
    uint32_t c[4] = {ctr, 0x6C6D6736u /* stream tag */, 0u, 0u};
    uint32_t k[2] = {s1, s2};
#pragma unroll
    for (int r = 0; r < 10; r++) round(c, k);
    out[0] = c[0];
    out[1] = c[1];
    out[2] = c[2];
    out[3] = c[3];
  }
};

// Four N(0,1) values per counter; out[4*q + r].
template <class R>
__global__ void gauss_fill_kernel(R *out, size_t n, uint32_t s1, uint32_t s2) {
  const size_t nq = (n + 3) / 4;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nq;
       q += (size_t)gridDim.x * blockDim.x) {
    uint32_t b[4];
    Philox::gen((uint32_t)q, s1, s2, b);
    R z[4];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      // u1 in (0,1], u2 in [0,1) from 32 random bits each
      const double u1 = ((double)b[2 * h] + 1.0) * 2.3283064365386963e-10;
      const double u2 = (double)b[2 * h + 1] * 2.3283064365386963e-10;
      if (sizeof(R) == 4) {
        const float rr = sqrtf(-2.0f * logf((float)u1));
        float sn, cs;
        sincospif(2.0f * (float)u2, &sn, &cs);
        z[2 * h] = (R)(rr * cs);
        z[2 * h + 1] = (R)(rr * sn);
      } else {
        const double rr = sqrt(-2.0 * log(u1));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        z[2 * h] = (R)(rr * cs);
        z[2 * h + 1] = (R)(rr * sn);
      }
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
      if (4 * q + r < n) out[4 * q + r] = z[r];
  }
}

// ---------------------------------------------------------------------------
// FP64 block reduction + "last block finishes" grid reduction
// ---------------------------------------------------------------------------
constexpr int kRedThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums `v` over the block; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double red[NV][kRedThreads / 32];
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = warp_sum(v[q]);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) red[q][wid] = v[q];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
      double x = lane < kRedThreads / 32 ? red[q][lane] : 0.0;
      v[q] = warp_sum(x);
    }
  }
}

// Publishes this block's NV partial sums; returns true in thread 0 of the
// last block to arrive, whose `tot` then holds the grid totals (summed in
// block order, so the result does not depend on arrival order).
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double *partials,
                                         unsigned *ticket, double (&tot)[NV]) {
  __shared__ bool s_last;
  block_sum<NV>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) __stcg(partials + (size_t)q * gridDim.x + blockIdx.x, v[q]);
    __threadfence();
    const unsigned prev = atomicAdd(ticket, 1u);
    s_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  // the last block sums the partials cooperatively
  double acc[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) acc[q] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] += __ldcg(partials + (size_t)q * gridDim.x + b);
  }
  block_sum<NV>(acc);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) tot[q] = acc[q];
    *ticket = 0u;
  }
  return threadIdx.x == 0;
}

// Scalars of one solve, FP64, in device memory.
struct KrylovScalars {
  double normz;       // |z|
  double err;         // last successive-iterate error
  int status;         // 0 ok, 1 QL failure
  int pad;
  double alpha[256];  // diagonal of T
  double beta[256];   // off-diagonal of T (beta[i] couples i and i+1)
};

// |z|^2 -> normz, and v0 = z/|z| (two kernels: the norm is a grid reduction)
template <class R>
__global__ void krylov_norm_kernel(const R *z, size_t n, double *partials, unsigned *ticket,
                                   KrylovScalars *sc) {
  double v[1] = {0.0};
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double x = (double)z[e];
    v[0] += x * x;
  }
  double tot[1];
  if (grid_sum<1>(v, partials, ticket, tot)) sc->normz = sqrt(tot[0]);
}

template <class R>
__global__ void krylov_scale_first_kernel(const R *z, R *v0, size_t n, const KrylovScalars *sc) {
  const R inv = (R)(1.0 / sc->normz);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    v0[e] = z[e] * inv;
}

// ---------------------------------------------------------------------------
// The vector work of one Lanczos iteration after the matvec, in one
// cooperative launch (all blocks resident) with grid barriers between its
// three phases, each a grid-stride pass with an FP64 block-ordered reduction:
//   w -= beta_{i-1} v_{i-1};  alpha_i = w . v_i
//   w -= alpha_i v_i;  beta_i = |w|, zeroed below 1e-3 alpha_i/|z|
//   v_{i+1} = w / beta_i, or e1 after a breakdown
// (one launch instead of three saves two launch gaps per iteration).  Each
// barrier wait is bounded (~1 s): a block that gives up raises err_flag
// (mapped host memory, read by the host at its next check) and returns; the
// host resets the barrier words before every solve.
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(kRedThreads)
krylov_step_kernel(R *w, const R *vi, const R *vprev, R *vnext, size_t n, int i,
                   double *partials, unsigned *ticket, unsigned *bar, KrylovScalars *sc,
                   double *host_ab, double *err_flag) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t e0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  // w -= beta_{i-1} v_{i-1};  alpha_i = w . v_i
  {
    const R bprev = i > 0 ? (R)sc->beta[i - 1] : R(0);
    double v[1] = {0.0};
    for (size_t e = e0; e < n; e += stride) {
      R x = w[e];
      if (i > 0) x -= bprev * vprev[e];
      w[e] = x;
      v[0] += (double)x * (double)vi[e];
    }
    double tot[1];
    if (grid_sum<1>(v, partials, ticket, tot)) sc->alpha[i] = tot[0];
  }
  if (!grid_barrier(bar)) {
    *err_flag = 1.0;
    return;
  }
  // w -= alpha_i v_i;  beta_i = |w| with the breakdown rule
  {
    const R al = (R)__ldcg(&sc->alpha[i]);
    double v[1] = {0.0};
    for (size_t e = e0; e < n; e += stride) {
      const R x = w[e] - al * vi[e];
      w[e] = x;
      v[0] += (double)x * (double)x;
    }
    double tot[1];
    if (grid_sum<1>(v, partials, ticket, tot)) {
      double b = sqrt(tot[0]);
      const double a = __ldcg(&sc->alpha[i]);
      const double tol = 1e-3 * a / sc->normz;  // LanczosAlgorithm.cu:141-143
      if (b < tol) b = 0.0;
      sc->beta[i] = b;
      host_ab[2 * i] = a;
      host_ab[2 * i + 1] = b;
    }
  }
  if (!grid_barrier(bar)) {
    *err_flag = 1.0;
    return;
  }
  // v_{i+1} = w / beta_i, or e1 after a breakdown
  const double b = __ldcg(&sc->beta[i]);
  const R inv = b > 0.0 ? (R)(1.0 / b) : R(0);
  for (size_t e = e0; e < n; e += stride)
    vnext[e] = b > 0.0 ? __ldcg(w + e) * inv : (e == 0 ? R(1) : R(0));
}

// ---------------------------------------------------------------------------
// Thread-block cluster helpers: the CTA's rank in its cluster and the
// cluster's CTA count, the split cluster barrier (arrive with release
// semantics, wait with acquire semantics; every thread of every CTA takes
// part, and the hardware guarantees that the CTAs of a cluster run at the
// same time) and FP64 loads from another CTA's shared memory.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned cluster_ctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_nctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// *local as it is in the shared memory of the cluster's CTA `rank`
__device__ __forceinline__ double ld_dsmem(const double *local, unsigned rank) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(local);
  unsigned ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(ra) : "memory");
  return v;
}

constexpr int kClusterThreads = 1024;

__device__ __forceinline__ float2 ld_dsmem(const float2 *local, unsigned rank) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(local);
  unsigned ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(ra)
               : "memory");
  return v;
}

// Per-thread sums of products for the cluster reductions.  FP64 vectors sum
// in FP64.  FP32 vectors sum as an unevaluated pair of floats s + c
// ("double-float": each product's rounding error from an fma, each
// addition's from Knuth's two-sum; Ogita, Rump and Oishi, SIAM J. Sci.
// Comput. 26, 2005), good to about 2^-48 relative: GB300 runs FP64 at a small
// fraction of its FP32 rate, and FP64 accumulation on the few SMs of one
// cluster would bound these kernels.
template <class R> struct DotAcc {
  double v = 0.0;
  __device__ __forceinline__ void add_prod(R x, R y) { v += (double)x * (double)y; }
  __device__ __forceinline__ void warp_merge() { v = warp_sum(v); }
  __device__ __forceinline__ double value() const { return v; }
};
template <> struct DotAcc<float> {
  float s = 0.f, c = 0.f;
  // s + c += p + pe, where p + pe is exact and |pe| is below an ulp of p
  __device__ __forceinline__ void add(float p, float pe) {
    const float t = __fadd_rn(s, p);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, pe));
  }
  __device__ __forceinline__ void add_prod(float x, float y) {
    const float p = __fmul_rn(x, y);
    add(p, __fmaf_rn(x, y, -p));
  }
  // (s, c) += (s2, c2); the same result for either order of the operands
  __device__ __forceinline__ void merge(float s2, float c2) {
    const float t = __fadd_rn(s, s2);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(s2, bp));
    s = t;
    c = __fadd_rn(__fadd_rn(c, c2), err);
  }
  __device__ __forceinline__ void warp_merge() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      merge(__shfl_xor_sync(0xffffffffu, s, o), __shfl_xor_sync(0xffffffffu, c, o));
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// Shared memory of the cluster reductions: per-warp sums, this CTA's sums
// (one slot per reduction of a launch, read by the other CTAs) and totals.
template <class R> struct ClusterRed {
  double warp[32];
  double part[2];
  double tot[2];
  __device__ __forceinline__ void put_warp(int w, const DotAcc<R> &a) { warp[w] = a.v; }
  __device__ __forceinline__ DotAcc<R> get_warp(int w) const { DotAcc<R> a; a.v = warp[w]; return a; }
  __device__ __forceinline__ void put_part(int q, const DotAcc<R> &a) { part[q] = a.v; }
  __device__ __forceinline__ DotAcc<R> get_part(int q, unsigned rank) const {
    DotAcc<R> a;
    a.v = ld_dsmem(&part[q], rank);
    return a;
  }
};
template <> struct ClusterRed<float> {
  float2 warp[32];
  float2 part[2];
  double tot[2];
  __device__ __forceinline__ void put_warp(int w, const DotAcc<float> &a) {
    warp[w] = make_float2(a.s, a.c);
  }
  __device__ __forceinline__ DotAcc<float> get_warp(int w) const {
    DotAcc<float> a;
    a.s = warp[w].x;
    a.c = warp[w].y;
    return a;
  }
  __device__ __forceinline__ void put_part(int q, const DotAcc<float> &a) {
    part[q] = make_float2(a.s, a.c);
  }
  __device__ __forceinline__ DotAcc<float> get_part(int q, unsigned rank) const {
    const float2 v = ld_dsmem(&part[q], rank);
    DotAcc<float> a;
    a.s = v.x;
    a.c = v.y;
    return a;
  }
};

// The sum over the cluster of every thread's accumulator, the same value in
// every thread of every CTA: xor trees within the warps, over the block's
// warps (warp 0) and over the cluster's CTAs (warp 0, reading the other CTAs'
// partials in distributed shared memory after a cluster barrier), then
// broadcast through shared memory.  Each reduction of a launch uses its own
// partial slot `q`, so no CTA overwrites a partial that another may still
// be reading.
template <class R>
__device__ __forceinline__ double cluster_reduce(DotAcc<R> a, ClusterRed<R> &sh, int q,
                                                 unsigned nct) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  a.warp_merge();
  if (lane == 0) sh.put_warp(wid, a);
  __syncthreads();
  if (wid == 0) {
    DotAcc<R> b;
    if (lane < (int)(blockDim.x >> 5)) b = sh.get_warp(lane);
    b.warp_merge();
    if (lane == 0) sh.put_part(q, b);
  }
  cluster_arrive();
  cluster_wait();
  if (wid == 0) {
    DotAcc<R> b;
    if (lane < (int)nct) b = sh.get_part(q, lane);
    b.warp_merge();
    if (lane == 0) sh.tot[q] = b.value();
  }
  __syncthreads();
  return sh.tot[q];
}

// ---------------------------------------------------------------------------
// The vector work of one Lanczos iteration after the matvec (the same three
// phases and per-element arithmetic as krylov_step_kernel; FP32 vectors
// accumulate their inner products in double-float, see DotAcc) in ONE
// thread-block cluster: the two reductions go through distributed shared memory and the
// hardware cluster barrier instead of global partials, tickets and software
// grid barriers, so the launch has no spin-wait and leaves the rest of the
// GPU free (the convergence check on the side stream runs beside it).  With
// EPT > 0 each thread keeps its EPT elements of w and v_i in registers
// across the phases (n <= EPT x the cluster's threads); EPT = 0 streams them
// through memory (any n).  Launched as one cluster of up to 16 CTAs of up
// to kClusterThreads threads (a multiple of 32).
// ---------------------------------------------------------------------------
template <class R, int EPT>
__global__ void __launch_bounds__(kClusterThreads, 1)
krylov_step_cluster_kernel(R *w, const R *vi, const R *vprev, R *vnext, size_t n, int i,
                           KrylovScalars *sc, double *host_ab) {
  __shared__ ClusterRed<R> red;
  constexpr int E = EPT > 0 ? EPT : 1;
  const unsigned nct = cluster_nctarank(), rank = cluster_ctarank();
  const size_t stride = (size_t)nct * blockDim.x;
  const size_t e0 = (size_t)rank * blockDim.x + threadIdx.x;
  R wr[E], vr[E];
  // w -= beta_{i-1} v_{i-1};  alpha_i = w . v_i
  const R bprev = i > 0 ? (R)sc->beta[i - 1] : R(0);
  DotAcc<R> acc;
  if (EPT > 0) {
#pragma unroll
    for (int k = 0; k < E; k++) {
      const size_t e = e0 + (size_t)k * stride;
      wr[k] = vr[k] = R(0);
      if (e < n) {
        R x = w[e];
        if (i > 0) x -= bprev * vprev[e];
        wr[k] = x;
        vr[k] = vi[e];
        acc.add_prod(x, vr[k]);
      }
    }
  } else {
    for (size_t e = e0; e < n; e += stride) {
      R x = w[e];
      if (i > 0) x -= bprev * vprev[e];
      w[e] = x;
      acc.add_prod(x, vi[e]);
    }
  }
  const double alpha = cluster_reduce<R>(acc, red, 0, nct);
  // w -= alpha_i v_i;  beta_i = |w| with the breakdown rule
  const R al = (R)alpha;
  DotAcc<R> acc2;
  if (EPT > 0) {
#pragma unroll
    for (int k = 0; k < E; k++) {
      if (e0 + (size_t)k * stride < n) {
        const R x = wr[k] - al * vr[k];
        wr[k] = x;
        acc2.add_prod(x, x);
      }
    }
  } else {
    for (size_t e = e0; e < n; e += stride) {
      const R x = w[e] - al * vi[e];
      w[e] = x;
      acc2.add_prod(x, x);
    }
  }
  double b = sqrt(cluster_reduce<R>(acc2, red, 1, nct));
  // no CTA reads another's partials after this point; the matching wait
  // before the exit keeps every CTA's shared memory alive until then
  cluster_arrive();
  const double tol = 1e-3 * alpha / sc->normz;  // LanczosAlgorithm.cu:141-143
  if (b < tol) b = 0.0;
  if (rank == 0 && threadIdx.x == 0) {
    sc->alpha[i] = alpha;
    sc->beta[i] = b;
    host_ab[2 * i] = alpha;
    host_ab[2 * i + 1] = b;
  }
  // v_{i+1} = w / beta_i, or e1 after a breakdown
  const R inv = b > 0.0 ? (R)(1.0 / b) : R(0);
  if (EPT > 0) {
#pragma unroll
    for (int k = 0; k < E; k++) {
      const size_t e = e0 + (size_t)k * stride;
      if (e < n) vnext[e] = b > 0.0 ? wr[k] * inv : (e == 0 ? R(1) : R(0));
    }
  } else {
    for (size_t e = e0; e < n; e += stride)
      vnext[e] = b > 0.0 ? w[e] * inv : (e == 0 ? R(1) : R(0));
  }
  cluster_wait();
}

// ---------------------------------------------------------------------------
// T_m^{1/2} e1 in FP64: implicit QL with Wilkinson shifts on the symmetric
// tridiagonal T_m (the tql1/tql2 family of Bowdler, Martin, Reinsch and
// Wilkinson, Numer. Math. 11, 1968).  Only the first row of the eigenvector
// matrix Q is carried through the sweeps (O(1) per rotation) and every
// rotation is logged; T^{1/2} e1 = Q diag(sqrt(lambda)) Q^T e1 is then
// obtained by applying the logged rotations in reverse order to the vector
// diag(sqrt(lambda)) Q^T e1.  Total work O(m^2) instead of O(m^3).
// Negative eigenvalues give NaN, as the reference's sqrt does
// (LanczosAlgorithm.cu:72-74), which the error test then reports.
// ---------------------------------------------------------------------------
struct RotLog {
  double2 *cs;     // (c, s) per rotation
  int *idx;        // column index i of the rotation on (i, i+1)
  int capacity;
};

inline double pythag(double a, double b) {
  const double r = sqrt(a * a + b * b);
  if (r == 0.0 || isinf(r)) {  // rescale only when the plain form fails
    const double p = fmax(fabs(a), fabs(b));
    if (p == 0.0) return 0.0;
    const double q = fmin(fabs(a), fabs(b)) / p;
    return p * sqrt(1.0 + q * q);
  }
  return r;
}

inline int tridiag_sqrt_e1(const double *alpha, const double *beta, int m,
                                               double *d, double *e, double *q0, RotLog log,
                                               double *out) {
  for (int k = 0; k < m; k++) {
    d[k] = alpha[k];
    e[k] = k + 1 < m ? beta[k] : 0.0;
    q0[k] = k == 0 ? 1.0 : 0.0;
  }
  int nrot = 0;
  const double eps = 2.220446049250313e-16;
  for (int l = 0; l < m; l++) {
    int iter = 0;
    for (;;) {
      int mm = l;
      for (; mm < m - 1; mm++) {
        const double dd = fabs(d[mm]) + fabs(d[mm + 1]);
        if (fabs(e[mm]) <= eps * dd) break;
      }
      if (mm == l) break;
      if (++iter > 60) return 1;
      // Wilkinson-type shift from the leading 2x2 block
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = pythag(g, 1.0);
      g = d[mm] - d[l] + e[l] / (g + (g >= 0.0 ? fabs(r) : -fabs(r)));
      double s = 1.0, c = 1.0, p = 0.0;
      int i = mm - 1;
      bool deflated = false;
      for (; i >= l; i--) {
        double f = s * e[i];
        const double b = c * e[i];
        r = pythag(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // underflow: split the matrix here and restart
          d[i + 1] -= p;
          e[mm] = 0.0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        // rotation on columns (i, i+1):  Q <- Q G,  G = [[c, s], [-s, c]]
        const double a0 = q0[i], a1 = q0[i + 1];
        q0[i] = c * a0 - s * a1;
        q0[i + 1] = s * a0 + c * a1;
        if (nrot >= log.capacity) return 2;
        log.cs[nrot].x = c;
        log.cs[nrot].y = s;
        log.idx[nrot] = i;
        nrot++;
      }
      if (deflated) continue;
      d[l] -= p;
      e[l] = g;
      e[mm] = 0.0;
    }
  }
  // out = Q (sqrt(lambda) * q0), applying the logged rotations in reverse
  for (int k = 0; k < m; k++) out[k] = sqrt(d[k]) * q0[k];
  for (int t = nrot - 1; t >= 0; t--) {
    const double c = log.cs[t].x, s = log.cs[t].y;
    const int i = log.idx[t];
    const double a0 = out[i], a1 = out[i + 1];
    out[i] = c * a0 + s * a1;
    out[i + 1] = -s * a0 + c * a1;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// T^{1/2} e1 by quadrature, for the ensemble's many per-check solves: with
// T symmetric positive definite,
//   T^{-1/2} = (2/pi) int_0^inf (T + t^2 I)^{-1} dt,   T^{1/2} e1 = T T^{-1/2} e1,
// the integral taken by the trapezoidal rule after the double-exponential
// substitution t = exp((pi/2) sinh v) (Takahasi and Mori, 1974), on T scaled
// so that its spectrum is centred on 1; each node is one tridiagonal solve
// (Thomas, stable for SPD), O(m), and the nodes are independent.  Node
// spacing and range are chosen from the condition number so that the scalar
// rule is within about 1e-13 relative of 1/sqrt(lambda) over the whole spectrum
// (checked on a log grid; 54 to 134 nodes for kappa 1e2 to 1e8); the product
// T (T^{-1/2} e1) adds rounding of order sqrt(kappa) eps.  Returns 0,
// or 2 when T is not positive definite, kappa is above 1e8 or a bound fails:
// the caller then uses the exact routine above (which gives NaN for a
// negative eigenvalue, as the reference does).  work: 18 m doubles.
// ---------------------------------------------------------------------------
// number of eigenvalues of T below x (Sturm count of T - x I = L D L^T)
inline int tridiag_count_below(const double *a, const double *b, int m, double x) {
  int c = 0;
  double d = 1.0;
  for (int k = 0; k < m; k++) {
    const double bb = k > 0 ? b[k - 1] * b[k - 1] : 0.0;
    d = (a[k] - x) - (k > 0 ? bb / d : 0.0);
    if (d == 0.0) d = -1e-300;  // x is an eigenvalue: count it as below
    if (d < 0.0) c++;
  }
  return c;
}

inline int tridiag_sqrt_e1_quad(const double *alpha, const double *beta, int m, double *work,
                                double *out) {
  if (m == 1) {
    if (!(alpha[0] > 0.0)) return 2;
    out[0] = sqrt(alpha[0]);
    return 0;
  }
  // upper bound of the spectrum (Gershgorin)
  double hi = 0.0;
  for (int k = 0; k < m; k++) {
    const double r = (k > 0 ? fabs(beta[k - 1]) : 0.0) + (k + 1 < m ? fabs(beta[k]) : 0.0);
    hi = fmax(hi, alpha[k] + r);
  }
  if (!(hi > 0.0) || !std::isfinite(hi)) return 2;
  if (tridiag_count_below(alpha, beta, m, 0.0) > 0) return 2;
  // lower bound of the spectrum: step down by 4 until nothing lies below
  double lo = hi;
  while (tridiag_count_below(alpha, beta, m, lo) > 0) {
    lo *= 0.25;
    if (lo < hi * 1e-8) return 2;
  }
  const double kappa = hi / lo;
  double h, vmax;
  if (kappa <= 1e2) {
    h = 0.15;
    vmax = 4.0;
  } else if (kappa <= 1e4) {
    h = 0.1;
    vmax = 4.0;
  } else if (kappa <= 1e6) {
    h = 0.08;
    vmax = 4.5;
  } else {
    h = 0.06;
    vmax = 4.0;
  }
  const double s = sqrt(lo * hi), is = 1.0 / s;
  const int half = (int)(vmax / h + 0.5);
  // work: acc[m], then 8 nodes at a time: cp[8][m], gp[8][m]
  double *acc = work, *cp = work + m, *gp = work + 9 * m;
  for (int k = 0; k < m; k++) acc[k] = 0.0;
  constexpr double kPi = 3.14159265358979323846;
  for (int j0 = -half; j0 <= half; j0 += 8) {
    const int nq = (half - j0 + 1) < 8 ? (half - j0 + 1) : 8;
    double t2[8], w[8];
    for (int q = 0; q < nq; q++) {
      const double v = (j0 + q) * h;
      const double t = exp(0.5 * kPi * sinh(v));
      t2[q] = t * t;
      w[q] = h * cosh(v) * t;  // (2/pi) h (pi/2) cosh(v) t
    }
    // forward sweep of (T/s + t^2 I) g = e1, nodes interleaved
    for (int q = 0; q < nq; q++) {
      const double den = alpha[0] * is + t2[q];
      const double inv = 1.0 / den;
      cp[q * m] = beta[0] * is * inv;
      gp[q * m] = inv;
    }
    for (int k = 1; k < m; k++) {
      const double ek = beta[k - 1] * is;
      const double ak = alpha[k] * is;
      const double bk = k + 1 < m ? beta[k] * is : 0.0;
      for (int q = 0; q < nq; q++) {
        const double inv = 1.0 / (ak + t2[q] - ek * cp[q * m + k - 1]);
        cp[q * m + k] = bk * inv;
        gp[q * m + k] = -ek * gp[q * m + k - 1] * inv;
      }
    }
    // back substitution, weighted into acc
    for (int q = 0; q < nq; q++) {
      double g = gp[q * m + m - 1];
      acc[m - 1] += w[q] * g;
      for (int k = m - 2; k >= 0; k--) {
        g = gp[q * m + k] - cp[q * m + k] * g;
        acc[k] += w[q] * g;
      }
    }
  }
  // T^{-1/2} e1 = s^{-1/2} acc;  out = T (s^{-1/2} acc)
  const double f = 1.0 / sqrt(s);
  for (int k = 0; k < m; k++) {
    double y = alpha[k] * acc[k];
    if (k > 0) y += beta[k - 1] * acc[k - 1];
    if (k + 1 < m) y += beta[k] * acc[k + 1];
    out[k] = f * y;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// T^{1/2} e1 on the device, by the quadrature of tridiag_sqrt_e1_quad (same
// spectrum bounds, node rule, weights and node order), so that a convergence
// check needs no host eigen-solve and no copy of its coefficients (an
// option: with GB300's narrow FP64 units this chain of FP64 divisions takes
// longer than the host's QL at the sizes measured, ~40 us a check).  One block:
// the positive-definiteness test and the 4^-j lower-bound candidates are one
// Sturm count per thread; then thread q sweeps quadrature node q (forward
// elimination and back substitution of (T/s + t_q^2 I) g = e1, FP64) and
// writes w_q g to scratch; the node sums are folded in node order and T is
// applied.  *flag (mapped host memory) becomes 0, or 1 when T is not
// positive definite or its condition number exceeds 1e8: then `out` is not
// written and the caller takes the exact eigen-solution on the host.
// ---------------------------------------------------------------------------
constexpr int kQuadThreads = 256;  // >= the largest node count (135) and m

__device__ __forceinline__ int sturm_count_below(const double *a, const double *b, int m,
                                                 double x) {
  int c = 0;
  double d = 1.0;
  for (int k = 0; k < m; k++) {
    const double bb = k > 0 ? b[k - 1] * b[k - 1] : 0.0;
    d = (a[k] - x) - (k > 0 ? bb / d : 0.0);
    if (d == 0.0) d = -1e-300;  // x is an eigenvalue: count it as below
    if (d < 0.0) c++;
  }
  return c;
}

static __global__ void __launch_bounds__(kQuadThreads)
tridiag_sqrt_quad_kernel(const KrylovScalars *sc, int m, double *out, double *G,
                         double *flag) {
  __shared__ double a[kQuadThreads], b[kQuadThreads], acc[kQuadThreads];
  __shared__ int cnt[15];
  __shared__ double s_hi, s_lo;
  __shared__ int s_state;  // 0 go on, 1 fall back
  const int t = threadIdx.x;
  for (int k = t; k < m; k += kQuadThreads) {
    a[k] = sc->alpha[k];
    b[k] = sc->beta[k];
  }
  __syncthreads();
  if (m == 1) {
    if (t == 0) {
      if (a[0] > 0.0) {
        out[0] = sqrt(a[0]);
        *flag = 0.0;
      } else {
        *flag = 1.0;
      }
    }
    return;
  }
  if (t == 0) {  // upper bound of the spectrum (Gershgorin)
    double hi = 0.0;
    for (int k = 0; k < m; k++) {
      const double r = (k > 0 ? fabs(b[k - 1]) : 0.0) + (k + 1 < m ? fabs(b[k]) : 0.0);
      hi = fmax(hi, a[k] + r);
    }
    s_hi = hi;
    s_state = (hi > 0.0 && isfinite(hi)) ? 0 : 1;
  }
  __syncthreads();
  if (s_state) {
    if (t == 0) *flag = 1.0;
    return;
  }
  // thread 0: eigenvalues below 0; thread j = 1..14: below hi * 4^-(j-1)
  if (t < 15) cnt[t] = sturm_count_below(a, b, m, t == 0 ? 0.0 : ldexp(s_hi, -2 * (t - 1)));
  __syncthreads();
  if (t == 0) {
    int state = cnt[0] > 0 ? 1 : 0;
    double lo = 0.0;
    if (!state) {
      int j = 0;
      while (j < 14 && cnt[j + 1] > 0) j++;
      if (j == 14) state = 1;  // below hi * 1e-8
      else lo = ldexp(s_hi, -2 * j);
    }
    s_lo = lo;
    s_state = state;
  }
  __syncthreads();
  if (s_state) {
    if (t == 0) *flag = 1.0;
    return;
  }
  const double hi = s_hi, lo = s_lo;
  const double kappa = hi / lo;
  double h, vmax;
  if (kappa <= 1e2) {
    h = 0.15;
    vmax = 4.0;
  } else if (kappa <= 1e4) {
    h = 0.1;
    vmax = 4.0;
  } else if (kappa <= 1e6) {
    h = 0.08;
    vmax = 4.5;
  } else {
    h = 0.06;
    vmax = 4.0;
  }
  const double sq = sqrt(lo * hi), is = 1.0 / sq;
  const int half = (int)(vmax / h + 0.5);
  const int nodes = 2 * half + 1;
  if (t < nodes) {
    constexpr double kPi = 3.14159265358979323846;
    const double v = (t - half) * h;
    const double tt = exp(0.5 * kPi * sinh(v));
    const double t2 = tt * tt;
    const double w = h * cosh(v) * tt;
    double *g = G + (size_t)t * 2 * kQuadThreads;  // gp[m], then cp[m]
    double *cp = g + kQuadThreads;
    {
      const double inv = 1.0 / (a[0] * is + t2);
      cp[0] = b[0] * is * inv;
      g[0] = inv;
    }
    for (int k = 1; k < m; k++) {
      const double ek = b[k - 1] * is;
      const double bk = k + 1 < m ? b[k] * is : 0.0;
      const double inv = 1.0 / (a[k] * is + t2 - ek * cp[k - 1]);
      cp[k] = bk * inv;
      g[k] = -ek * g[k - 1] * inv;
    }
    double x = g[m - 1];
    g[m - 1] = w * x;
    for (int k = m - 2; k >= 0; k--) {
      x = g[k] - cp[k] * x;
      g[k] = w * x;
    }
  }
  __syncthreads();
  for (int k = t; k < m; k += kQuadThreads) {  // node order, as the host sums
    double s = 0.0;
    for (int q = 0; q < nodes; q++) s += G[(size_t)q * 2 * kQuadThreads + k];
    acc[k] = s;
  }
  __syncthreads();
  const double f = 1.0 / sqrt(sq);
  for (int k = t; k < m; k += kQuadThreads) {
    double y = a[k] * acc[k];
    if (k > 0) y += b[k - 1] * acc[k - 1];
    if (k + 1 < m) y += b[k] * acc[k + 1];
    out[k] = f * y;
  }
  if (t == 0) *flag = 0.0;
}

// y = |z| V c over m basis vectors and, when yprev is given, err = |y -
// yprev| / |yprev| (FP64) -> sc->err and the mapped host copy: the estimate
// and the error of one convergence check in one launch (each thread's
// elements of y feed its share of the error sums directly).  V is row-major
// (row k is v_k, ldv elements apart); c may live in mapped host memory.  For
// short vectors (TPE = 4) each element's sum over the basis is shared by four
// threads, so a check is not a chain of m dependent loads.
template <class R, int TPE>
__global__ void krylov_check_kernel(const R *V, size_t ldv, int m, const double *c,
                                    KrylovScalars *sc, R *y, const R *yprev, size_t n,
                                    double *partials, unsigned *ticket, double *host_err) {
  __shared__ R cs[256];
  const double nz = sc->normz;
  for (int k = threadIdx.x; k < m; k += blockDim.x) cs[k] = (R)(nz * c[k]);
  __syncthreads();
  // TPE consecutive threads share an element, thread `part` taking the basis
  // vectors k = part, part + TPE, ...; their sums meet in a fixed xor tree.
  // The pass loop is the same for every thread (the shuffles need the whole
  // warp), elements past n contribute nothing.
  const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int part = (int)(tid % TPE);
  const size_t per_pass = (size_t)gridDim.x * blockDim.x / TPE;
  double v[2] = {0.0, 0.0};
  for (size_t e0 = 0; e0 < n; e0 += per_pass) {
    const size_t e = e0 + tid / TPE;
    const bool ok = e < n;
    R acc = 0;
    if (ok) {
      // eight loads in flight per thread ahead of their products, which are
      // summed in the same order as one at a time
      const R *col = V + e;
      int k = part;
      for (; k + 7 * TPE < m; k += 8 * TPE) {
        R x[8];
#pragma unroll
        for (int u = 0; u < 8; u++) x[u] = col[(size_t)(k + u * TPE) * ldv];
#pragma unroll
        for (int u = 0; u < 8; u++) acc += cs[k + u * TPE] * x[u];
      }
      for (; k < m; k += TPE) acc += cs[k] * col[(size_t)k * ldv];
    }
#pragma unroll
    for (int o = 1; o < TPE; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (ok && part == 0) {
      y[e] = acc;
      if (yprev) {
        const double a = (double)yprev[e], dlt = (double)acc - a;
        v[0] += a * a;
        v[1] += dlt * dlt;
      }
    }
  }
  if (!yprev) return;
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot)) {
    const double err = fabs(sqrt(tot[1]) / sqrt(tot[0]));
    sc->err = err;
    *host_err = err;
  }
}

// ---------------------------------------------------------------------------
// BiCGSTAB pieces for solving P x = b with the sparse preconditioner (the
// last step of the preconditioned square root).  Each reduction writes its
// FP64 results to mapped host memory (out[0], out[1]).
// ---------------------------------------------------------------------------
template <class R>
__global__ void dot2_kernel(const R *a, const R *b, const R *c, const R *d, size_t n,
                            double *partials, unsigned *ticket, double *out) {
  double v[2] = {0.0, 0.0};
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    v[0] += (double)a[e] * (double)b[e];
    v[1] += (double)c[e] * (double)d[e];
  }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot)) {
    out[0] = tot[0];
    out[1] = tot[1];
  }
}

// p = r + beta (p - omega v)
template <class R>
__global__ void bicg_p_kernel(R *p, const R *r, const R *v, double beta, double omega, size_t n) {
  const R b = (R)beta, o = (R)omega;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    p[e] = r[e] + b * (p[e] - o * v[e]);
}

// s = r - alpha v ; out[0] = |s|^2
template <class R>
__global__ void bicg_s_kernel(R *s, const R *r, const R *v, double alpha, size_t n,
                              double *partials, unsigned *ticket, double *out) {
  const R a = (R)alpha;
  double acc[1] = {0.0};
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const R x = r[e] - a * v[e];
    s[e] = x;
    acc[0] += (double)x * (double)x;
  }
  double tot[1];
  if (grid_sum<1>(acc, partials, ticket, tot)) out[0] = tot[0];
}

// x += alpha p + omega s ; r = s - omega t ; out = (|r|^2, rhat . r)
template <class R>
__global__ void bicg_xr_kernel(R *x, const R *p, const R *s, const R *t, R *r, const R *rhat,
                               double alpha, double omega, size_t n, double *partials,
                               unsigned *ticket, double *out) {
  const R a = (R)alpha, o = (R)omega;
  double acc[2] = {0.0, 0.0};
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    x[e] += a * p[e] + o * s[e];
    const R re = s[e] - o * t[e];
    r[e] = re;
    acc[0] += (double)re * (double)re;
    acc[1] += (double)rhat[e] * (double)re;
  }
  double tot[2];
  if (grid_sum<2>(acc, partials, ticket, tot)) {
    out[0] = tot[0];
    out[1] = tot[1];
  }
}

// y = c x
template <class R>
__global__ void scale_kernel(R *y, const R *x, size_t n, R c) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    y[e] = c * x[e];
}

// out += pf * y  (used for both the linear and the angular halves)
template <class R>
__global__ void axpy_kernel(R *out, const R *y, size_t n, R pf) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    out[e] += pf * y[e];
}

}  // namespace lmg
