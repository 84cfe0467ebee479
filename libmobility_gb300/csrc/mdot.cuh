// Tiled all-pairs RPY mobility product M.[F;T] for sm_103a.
//
// Replaces the reference kernels computeRPYBatchedFastGPU / NaiveGPU /
// NaiveBlockGPU and their launchers (libMobility
// solvers/NBody/extra/NbodyRPY.cu:26-252): every pair (i, j) inside the same
// batch contributes, the self pair included, and the outputs are overwritten.
//
// Layout and schedule:
//   * a CTA owns BT = THREADS*TPT consecutive targets (TPT per thread,
//     strided by THREADS so loads and stores coalesce) and one contiguous
//     chunk of their batch's sources (blockIdx.y selects the chunk);
//   * sources are staged through shared memory in tiles of THREADS, already
//     divided by the radius a and, for the wall, clamped (h = max(z, a)/a)
//     and damped (F, T pre-multiplied by b_j); every thread then reads the
//     tile by broadcast;
//   * tiles whose sources all lie in the targets' batch take an unrolled loop
//     without bounds tests; batch edges take a per-pair test;
//   * FP32 partial sums are folded every tile into (sum, compensation) pairs
//     with the two-sum transformation, so the error does not grow with N;
//   * when the source range is split over several CTAs, each writes its
//     (sum, compensation) partials to scratch and the last CTA of a target
//     tile to finish (counted with an atomic ticket) reduces them in order
//     and writes the result; the ticket is reset by that CTA, so the scratch
//     needs no clearing between launches and nothing waits on anything.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "bounds.cuh"
#include "pack2.cuh"
#include "rpy_pair.cuh"

namespace lmg {

enum Geometry : int { kOpen = 0, kWall = 1 };

template <class R> struct alignas(4 * sizeof(R)) Q4 { R x, y, z, w; };

template <class R> struct MdotArgs {
  const R *pos;  // 3N positions, wall frame (wall at z = 0), interleaved
  const R *F;    // 3N forces or nullptr
  const R *T;    // 3N torques or nullptr
  R *U;          // 3N linear velocities (overwritten) or nullptr
  R *W;          // 3N angular velocities (overwritten) or nullptr
  const int *sys_begin;  // optional table of batch starts (nsys+1 entries)
  int nsys;              // number of entries-1 in sys_begin, or 0
  int N;                 // particles
  // targets [tgt_begin, tgt_end) (tgt_end = 0: all N), results written at
  // row i - tgt_begin of U and W (every source of a target's batch counts)
  int tgt_begin, tgt_end;
  int nper;              // equal batch size when sys_begin == nullptr
  int chunk;             // sources per split (multiple of THREADS)
  R inv_a;               // 1/a
  PairConst<R> k;
  WallConst kw;          // fused all-blocks wall constants (FP32 path)
  R *part;               // scratch: [tiles][nsplit][2*NC][BT]
  unsigned *ticket;      // scratch: [tiles]
  size_t part_cap, ticket_cap;  // their sizes (index checks of the checked build)
  // optional per-batch flags (nsys entries, with sys_begin): a tile whose
  // batches are all flagged 0 is skipped by every one of its CTAs (outputs
  // left as they were, scratch and ticket untouched)
  const int *sys_active;
};

// Two-sum fold of t into (S, C): S + C carries the running sum to about
// one rounding of the final value (Knuth's TwoSum).
template <class R> __device__ __forceinline__ void fold(R &S, R &C, R t) {
  const R s = S + t;
  const R bp = s - S;
  C += (S - (s - bp)) + (t - bp);
  S = s;
}

template <class R> __device__ __forceinline__ int system_of(const MdotArgs<R> &a, int i) {
  if (a.sys_begin == nullptr) return i / a.nper;
  int lo = 0, hi = a.nsys;  // sys_begin[lo] <= i < sys_begin[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(a.sys_begin + mid) <= i) lo = mid; else hi = mid;
  }
  return lo;
}
template <class R> __device__ __forceinline__ int system_start(const MdotArgs<R> &a, int s) {
  return a.sys_begin ? __ldg(a.sys_begin + s) : s * a.nper;
}
template <class R> __device__ __forceinline__ int system_end(const MdotArgs<R> &a, int s) {
  int e = a.sys_begin ? __ldg(a.sys_begin + s + 1) : (s + 1) * a.nper;
  return e < a.N ? e : a.N;
}

template <class R, int GEOM, bool HAS_F, bool HAS_T, bool ANG> struct PairKernel {
  static constexpr bool UF = HAS_F;
  static constexpr bool WF = HAS_F && ANG;
  static constexpr bool UT = HAS_T && ANG;
  static constexpr bool WT = HAS_T && ANG;

  static constexpr bool FUSED_WALL =
      GEOM == kWall && UF && UT && WT && WF && sizeof(R) == 4;

  // Adds the contribution of source (p, f, t) to target (x, y, z) and
  // returns the squared scaled distance r^2.  EXACT = false is the fast form
  // used for every pair of a full tile: the RPY coefficients are those of
  // separated pairs taken at max(r^2, 4) (so the value is finite and O(1)
  // for an overlapping or self pair, and exact for r >= 2a), and the wall
  // images take the pair formula even for the self pair.  The caller
  // replaces the fast value by the exact one for the pairs with r^2 < 4
  // (correct() below).
  template <bool EXACT = true>
  static __device__ __forceinline__ R eval(const PairConst<R> &k, const WallConst &kw, R xi,
                                           R yi, R zi, const Q4<R> &p, const Q4<R> &fv,
                                           const Q4<R> &tv, Vec3<R> &u, Vec3<R> &w) {
    if constexpr (FUSED_WALL) {
      wall_pair_fused(k, kw, xi, yi, zi, p.x, p.y, p.z, fv.x, fv.y, fv.z, tv.x, tv.y, tv.z, u,
                      w);
      return R(4);
    }
    const R dx = xi - p.x;
    const R dy = yi - p.y;
    const R dz = zi - p.z;
    const R r2 = fmaR(dx, dx, fmaR(dy, dy, dz * dz));
    R f = 0, G = 0, fw = 0, Gw = 0, c = 0;
    if constexpr (EXACT) {
      rpy_coefficients<R, UF, WT, UT || WF, true>(k, r2, dev_rsqrt<R>(r2), f, G, fw, Gw, c);
    } else {
      const R r2c = r2 > R(4) ? r2 : R(4);
      rpy_coefficients<R, UF, WT, UT || WF, false>(k, r2c, rsqrt_normal<R>(r2c), f, G, fw, Gw,
                                                   c);
    }
    if (UF) {
      const R g = G * fmaR(dx, fv.x, fmaR(dy, fv.y, dz * fv.z));
      u.x = fmaR(f, fv.x, fmaR(g, dx, u.x));
      u.y = fmaR(f, fv.y, fmaR(g, dy, u.y));
      u.z = fmaR(f, fv.z, fmaR(g, dz, u.z));
    }
    if (UT) {  // c (T x d)
      u.x = fmaR(c, fmaR(tv.y, dz, -tv.z * dy), u.x);
      u.y = fmaR(c, fmaR(tv.z, dx, -tv.x * dz), u.y);
      u.z = fmaR(c, fmaR(tv.x, dy, -tv.y * dx), u.z);
    }
    if (WT) {
      const R g = Gw * fmaR(dx, tv.x, fmaR(dy, tv.y, dz * tv.z));
      w.x = fmaR(fw, tv.x, fmaR(g, dx, w.x));
      w.y = fmaR(fw, tv.y, fmaR(g, dy, w.y));
      w.z = fmaR(fw, tv.z, fmaR(g, dz, w.z));
    }
    if (WF) {  // c (F x d)
      w.x = fmaR(c, fmaR(fv.y, dz, -fv.z * dy), w.x);
      w.y = fmaR(c, fmaR(fv.z, dx, -fv.x * dz), w.y);
      w.z = fmaR(c, fmaR(fv.x, dy, -fv.y * dx), w.z);
    }
    if (GEOM == kWall) {
      // image vector R = (dx, dy, h_i + h_j), shared by all blocks
      const R Rz = zi + p.z;
      const R iR = dev_rsqrt<R>(dx * dx + dy * dy + Rz * Rz);
      const R ex = dx * iR, ey = dy * iR, ez = Rz * iR;
      Vec3<R> cu = {0, 0, 0}, cw = {0, 0, 0}, ct = {0, 0, 0}, cf = {0, 0, 0};
      const Vec3<R> F3 = {fv.x, fv.y, fv.z};
      const Vec3<R> T3 = {tv.x, tv.y, tv.z};
      if (!EXACT || r2 > R(0)) {
        const R iRz = dev_div<R>(R(1), Rz);
        const R hj = p.z * iRz;  // h_j / R_z
        if (UF) wall_uf_pair<R>(ex, ey, ez, iR, hj, F3, cu);
        if (WT) wall_wt_pair<R>(ex, ey, ez, iR, T3, cw);
        if (WF) wall_wf_pair<R>(ex, ey, ez, iR, hj, F3, cf);
        if (UT) wall_ut_pair<R>(-ex, -ey, ez, iR, zi * iRz, T3, ct);
      } else {
        const R ih = dev_div<R>(R(1), p.z);
        if (UF) wall_self_uf<R>(ih, F3, cu);
        if (WT) wall_self_wt<R>(ih, T3, cw);
        if (WF) wall_self_wf<R>(ih, F3, cf);
        if (UT) wall_self_ut<R>(ih, T3, ct);
      }
      if (UF) { u.x += k.t0 * cu.x; u.y += k.t0 * cu.y; u.z += k.t0 * cu.z; }
      if (UT) { u.x += k.rt0 * ct.x; u.y += k.rt0 * ct.y; u.z += k.rt0 * ct.z; }
      if (WT) { w.x += k.r0 * cw.x; w.y += k.r0 * cw.y; w.z += k.r0 * cw.z; }
      if (WF) { w.x += k.rt0 * cf.x; w.y += k.rt0 * cf.y; w.z += k.rt0 * cf.z; }
    }
    return r2;
  }

  // For a pair with r^2 < 4 already added in the fast form: adds
  // (exact - fast).  Both are O(1) there, so the difference is accurate.
  static __device__ __forceinline__ void correct(const PairConst<R> &k, const WallConst &kw,
                                                 R xi, R yi, R zi, const Q4<R> &p,
                                                 const Q4<R> &fv, const Q4<R> &tv, Vec3<R> &u,
                                                 Vec3<R> &w) {
    const R dx = xi - p.x, dy = yi - p.y, dz = zi - p.z;
    if (fmaR(dx, dx, fmaR(dy, dy, dz * dz)) < R(4)) {
      Vec3<R> ue = {0, 0, 0}, we = {0, 0, 0}, uf = {0, 0, 0}, wf = {0, 0, 0};
      eval<true>(k, kw, xi, yi, zi, p, fv, tv, ue, we);
      eval<false>(k, kw, xi, yi, zi, p, fv, tv, uf, wf);
      u.x += ue.x - uf.x; u.y += ue.y - uf.y; u.z += ue.z - uf.z;
      w.x += we.x - wf.x; w.y += we.y - wf.y; w.z += we.z - wf.z;
    }
  }
};

template <class R, int GEOM, bool HAS_F, bool HAS_T, bool ANG, int TPT, int THREADS>
__global__ void __launch_bounds__(THREADS)
mdot_kernel(const MdotArgs<R> a) {
  using PK = PairKernel<R, GEOM, HAS_F, HAS_T, ANG>;
  constexpr int BT = THREADS * TPT;
  constexpr bool USE_T = HAS_T && ANG;
  constexpr int NC = ANG ? 6 : 3;  // accumulated components per target
  constexpr bool COMP = sizeof(R) == 4;  // compensated accumulation in FP32

  // The fused FP32 wall evaluation (all blocks) and the FP32 forces-only
  // evaluations (open and wall UF) take two sources at a time in packed f32x2
  // instructions (pack2.cuh); their sources are staged as separate arrays
  // (x, y, z, F, and T for all blocks) so that one float4 read yields a
  // component of four sources.
  constexpr bool PACK = PK::FUSED_WALL;
  constexpr bool PACK_UF = sizeof(R) == 4 && HAS_F && !ANG && THREADS % 32 == 0;
  constexpr int NSV = PACK ? 9 : (PACK_UF ? 6 : 1);
  constexpr bool SOA = PACK || PACK_UF;
  __shared__ Q4<R> sp[SOA ? 1 : THREADS];
  __shared__ Q4<R> sf[HAS_F && !SOA ? THREADS : 1];
  __shared__ Q4<R> st[USE_T && !SOA ? THREADS : 1];
  __shared__ __align__(16) float sv[NSV][SOA ? THREADS : 4];
  __shared__ int s_last;

  const int N = a.N;
  const int t_lo = a.tgt_begin, t_hi = a.tgt_end > 0 ? a.tgt_end : N;
  const int tile = blockIdx.x;
  const int split = blockIdx.y;
  const int nsplit = gridDim.y;
  const int tgt0 = t_lo + tile * BT;
  const R ia = a.inv_a;

  // ---- targets ----
  R xi[TPT], yi[TPT], zi[TPT], bi[TPT];
  int lo[TPT], hi[TPT];
#pragma unroll
  for (int t = 0; t < TPT; t++) {
    int i = tgt0 + threadIdx.x + t * THREADS;
    int ic = i < t_hi ? i : t_hi - 1;
    R x = a.pos[3 * ic], y = a.pos[3 * ic + 1], z = a.pos[3 * ic + 2];
    xi[t] = mul_rn(x, ia);
    yi[t] = mul_rn(y, ia);
    if (GEOM == kWall) {
      R zs = mul_rn(z, ia);
      bi[t] = zs < R(0) ? R(0) : (zs > R(1) ? R(1) : zs);
      zi[t] = zs > R(1) ? zs : R(1);
    } else {
      zi[t] = mul_rn(z, ia);
      bi[t] = R(1);
    }
    int s = system_of(a, ic);
    lo[t] = system_start(a, s);
    hi[t] = system_end(a, s);
  }
  // batch range of the whole CTA
  const int last = (tgt0 + BT < t_hi ? tgt0 + BT : t_hi) - 1;
  const int s_first = system_of(a, tgt0);
  const int s_lastb = system_of(a, last);
  const int src_lo = system_start(a, s_first);
  const int src_hi = system_end(a, s_lastb);
  const bool uniform = (s_first == s_lastb);
  if (a.sys_active != nullptr) {
    int any = 0;
    for (int q = s_first; q <= s_lastb; q++) any |= __ldg(a.sys_active + q);
    if (!any) return;
  }
  const int c_begin = src_lo + split * a.chunk;
  const int c_end = min(src_hi, c_begin + a.chunk);

  Vec3<R> u[TPT], w[TPT];
  R S[TPT][NC], C[TPT][NC];
#pragma unroll
  for (int t = 0; t < TPT; t++) {
    u[t] = {0, 0, 0};
    w[t] = {0, 0, 0};
#pragma unroll
    for (int c = 0; c < NC; c++) { S[t][c] = 0; C[t][c] = 0; }
  }

  for (int ts = c_begin; ts < c_end; ts += THREADS) {
    {  // stage one tile of sources
      const int j = ts + threadIdx.x;
      Q4<R> p = {0, 0, 0, 0}, fv = {0, 0, 0, 0}, tv = {0, 0, 0, 0};
      if (j < c_end && LMG_IN_BOUNDS(j < N, 1, j)) {
        R x = a.pos[3 * j], y = a.pos[3 * j + 1], z = a.pos[3 * j + 2];
        R b = R(1);
        p.x = mul_rn(x, ia);
        p.y = mul_rn(y, ia);
        if (GEOM == kWall) {
          R zs = mul_rn(z, ia);
          b = zs < R(0) ? R(0) : (zs > R(1) ? R(1) : zs);
          p.z = zs > R(1) ? zs : R(1);
        } else {
          p.z = mul_rn(z, ia);
        }
        if (HAS_F) { fv.x = b * a.F[3 * j]; fv.y = b * a.F[3 * j + 1]; fv.z = b * a.F[3 * j + 2]; }
        if (USE_T) { tv.x = b * a.T[3 * j]; tv.y = b * a.T[3 * j + 1]; tv.z = b * a.T[3 * j + 2]; }
      }
      if constexpr (SOA) {
        const float c9[9] = {p.x, p.y, p.z, fv.x, fv.y, fv.z, tv.x, tv.y, tv.z};
#pragma unroll
        for (int c = 0; c < NSV; c++) sv[c][threadIdx.x] = c9[c];
      } else {
        sp[threadIdx.x] = p;
        if (HAS_F) sf[threadIdx.x] = fv;
        if (USE_T) st[threadIdx.x] = tv;
      }
    }
    __syncthreads();
    const int n_here = min(THREADS, c_end - ts);
    if constexpr (PACK) {
      if (uniform && n_here == THREADS) {
        V3p u2[TPT], w2[TPT];
#pragma unroll
        for (int t = 0; t < TPT; t++) {
          u2[t] = {bc(0.f), bc(0.f), bc(0.f)};
          w2[t] = {bc(0.f), bc(0.f), bc(0.f)};
        }
#pragma unroll 1
        for (int jj = 0; jj < THREADS; jj += 4) {
          float4 q[9];
#pragma unroll
          for (int c = 0; c < 9; c++) q[c] = *reinterpret_cast<const float4 *>(&sv[c][jj]);
#pragma unroll
          for (int h = 0; h < 2; h++) {
            F2 v[9];
#pragma unroll
            for (int c = 0; c < 9; c++) v[c] = h ? mk2(q[c].z, q[c].w) : mk2(q[c].x, q[c].y);
#pragma unroll
            for (int t = 0; t < TPT; t++)
              wall_pair_fused_x2(a.k, a.kw, bc(xi[t]), bc(yi[t]), bc(zi[t]), v[0], v[1], v[2],
                                 v[3], v[4], v[5], v[6], v[7], v[8], u2[t], w2[t]);
          }
        }
#pragma unroll
        for (int t = 0; t < TPT; t++) {  // the two lanes hold even and odd sources
          u[t].x += u2[t].x.v.x + u2[t].x.v.y;
          u[t].y += u2[t].y.v.x + u2[t].y.v.y;
          u[t].z += u2[t].z.v.x + u2[t].z.v.y;
          w[t].x += w2[t].x.v.x + w2[t].x.v.y;
          w[t].y += w2[t].y.v.x + w2[t].y.v.y;
          w[t].z += w2[t].z.v.x + w2[t].z.v.y;
        }
      } else {
        for (int jj = 0; jj < n_here; jj++) {
          const int j = ts + jj;
#pragma unroll
          for (int t = 0; t < TPT; t++)
            if (j >= lo[t] && j < hi[t])
              wall_pair_fused(a.k, a.kw, xi[t], yi[t], zi[t], sv[0][jj], sv[1][jj], sv[2][jj],
                              sv[3][jj], sv[4][jj], sv[5][jj], sv[6][jj], sv[7][jj], sv[8][jj],
                              u[t], w[t]);
        }
      }
    } else if constexpr (PACK_UF && GEOM == kWall) {
      if (uniform && n_here == THREADS) {
        // two sources per instruction; close pairs fall back lane by lane
        V3p u2[TPT];
#pragma unroll
        for (int t = 0; t < TPT; t++) u2[t] = {bc(0.f), bc(0.f), bc(0.f)};
#pragma unroll 1
        for (int jj = 0; jj < THREADS; jj += 4) {
          float4 q[6];
#pragma unroll
          for (int c = 0; c < 6; c++) q[c] = *reinterpret_cast<const float4 *>(&sv[c][jj]);
#pragma unroll
          for (int h = 0; h < 2; h++) {
            F2 v[6];
#pragma unroll
            for (int c = 0; c < 6; c++) v[c] = h ? mk2(q[c].z, q[c].w) : mk2(q[c].x, q[c].y);
#pragma unroll
            for (int t = 0; t < TPT; t++)
              wall_uf_pair_x2(a.k, a.kw, bc(xi[t]), bc(yi[t]), bc(zi[t]), v[0], v[1], v[2],
                              v[3], v[4], v[5], u2[t]);
          }
        }
#pragma unroll
        for (int t = 0; t < TPT; t++) {  // the two lanes hold even and odd sources
          u[t].x += u2[t].x.v.x + u2[t].x.v.y;
          u[t].y += u2[t].y.v.x + u2[t].y.v.y;
          u[t].z += u2[t].z.v.x + u2[t].z.v.y;
        }
      } else {
        for (int jj = 0; jj < n_here; jj++) {
          const int j = ts + jj;
          const Q4<R> p = {sv[0][jj], sv[1][jj], sv[2][jj], 0};
          const Q4<R> fv = {sv[3][jj], sv[4][jj], sv[5][jj], 0};
#pragma unroll
          for (int t = 0; t < TPT; t++)
            if (j >= lo[t] && j < hi[t]) PK::eval(a.k, a.kw, xi[t], yi[t], zi[t], p, fv, fv, u[t], w[t]);
        }
      }
    } else if constexpr (PACK_UF) {
      if (uniform && n_here == THREADS) {
        // as the scalar full-tile path below, two sources per instruction
#pragma unroll 1
        for (int j0 = 0; j0 < THREADS; j0 += 32) {
          V3p u2[TPT];
          float2 mr2[TPT];
#pragma unroll
          for (int t = 0; t < TPT; t++) {
            u2[t] = {bc(0.f), bc(0.f), bc(0.f)};
            mr2[t] = make_float2(4.f, 4.f);
          }
#pragma unroll 2
          for (int jj = j0; jj < j0 + 32; jj += 4) {
            float4 q[6];
#pragma unroll
            for (int c = 0; c < 6; c++) q[c] = *reinterpret_cast<const float4 *>(&sv[c][jj]);
#pragma unroll
            for (int h = 0; h < 2; h++) {
              F2 v[6];
#pragma unroll
              for (int c = 0; c < 6; c++) v[c] = h ? mk2(q[c].z, q[c].w) : mk2(q[c].x, q[c].y);
#pragma unroll
              for (int t = 0; t < TPT; t++)
                open_uf_pair_x2(a.k, bc(xi[t]), bc(yi[t]), bc(zi[t]), v[0], v[1], v[2], v[3],
                                v[4], v[5], u2[t], mr2[t]);
            }
          }
          bool near = false;
#pragma unroll
          for (int t = 0; t < TPT; t++) {
            u[t].x += u2[t].x.v.x + u2[t].x.v.y;
            u[t].y += u2[t].y.v.x + u2[t].y.v.y;
            u[t].z += u2[t].z.v.x + u2[t].z.v.y;
            near = near || fminf(mr2[t].x, mr2[t].y) < 4.f;
          }
          if (__any_sync(0xffffffffu, near)) {
#pragma unroll
            for (int t = 0; t < TPT; t++) {
              if (fminf(mr2[t].x, mr2[t].y) < 4.f) {
                for (int jj = j0; jj < j0 + 32; jj++) {
                  const Q4<R> p = {sv[0][jj], sv[1][jj], sv[2][jj], 0};
                  const Q4<R> fv = {sv[3][jj], sv[4][jj], sv[5][jj], 0};
                  PK::correct(a.k, a.kw, xi[t], yi[t], zi[t], p, fv, fv, u[t], w[t]);
                }
              }
            }
          }
        }
      } else {
        for (int jj = 0; jj < n_here; jj++) {
          const int j = ts + jj;
          const Q4<R> p = {sv[0][jj], sv[1][jj], sv[2][jj], 0};
          const Q4<R> fv = {sv[3][jj], sv[4][jj], sv[5][jj], 0};
#pragma unroll
          for (int t = 0; t < TPT; t++)
            if (j >= lo[t] && j < hi[t]) PK::eval(a.k, a.kw, xi[t], yi[t], zi[t], p, fv, fv, u[t], w[t]);
        }
      }
    } else if (uniform && n_here == THREADS) {
      // Fast form for every pair, 32 sources at a time; then, in a warp where
      // some target met a pair closer than 2a among those 32 (its self pair,
      // or an overlap), those targets swap the fast value of such pairs for
      // the exact one.  Targets are tile-aligned, so a warp's self pairs all
      // fall in the same 32 sources.
#pragma unroll 1
      for (int j0 = 0; j0 < THREADS; j0 += 32) {
        R mr2[TPT];
#pragma unroll
        for (int t = 0; t < TPT; t++) mr2[t] = R(4);
#pragma unroll 4
        for (int jj = j0; jj < j0 + 32; jj++) {
          const Q4<R> p = sp[jj];
          const Q4<R> fv = HAS_F ? sf[jj] : Q4<R>{0, 0, 0, 0};
          const Q4<R> tv = USE_T ? st[jj] : Q4<R>{0, 0, 0, 0};
#pragma unroll
          for (int t = 0; t < TPT; t++) {
            const R r2 = PK::template eval<false>(a.k, a.kw, xi[t], yi[t], zi[t], p, fv, tv,
                                                  u[t], w[t]);
            mr2[t] = r2 < mr2[t] ? r2 : mr2[t];  // a min in R (no promotion)
          }
        }
        bool near = false;
#pragma unroll
        for (int t = 0; t < TPT; t++) near = near || mr2[t] < R(4);
        if (__any_sync(0xffffffffu, near)) {
#pragma unroll
          for (int t = 0; t < TPT; t++) {
            if (mr2[t] < R(4)) {
              for (int jj = j0; jj < j0 + 32; jj++) {
                const Q4<R> p = sp[jj];
                const Q4<R> fv = HAS_F ? sf[jj] : Q4<R>{0, 0, 0, 0};
                const Q4<R> tv = USE_T ? st[jj] : Q4<R>{0, 0, 0, 0};
                PK::correct(a.k, a.kw, xi[t], yi[t], zi[t], p, fv, tv, u[t], w[t]);
              }
            }
          }
        }
      }
    } else {
      for (int jj = 0; jj < n_here; jj++) {
        const int j = ts + jj;
        const Q4<R> p = sp[jj];
        const Q4<R> fv = HAS_F ? sf[jj] : Q4<R>{0, 0, 0, 0};
        const Q4<R> tv = USE_T ? st[jj] : Q4<R>{0, 0, 0, 0};
#pragma unroll
        for (int t = 0; t < TPT; t++)
          if (j >= lo[t] && j < hi[t]) PK::eval(a.k, a.kw, xi[t], yi[t], zi[t], p, fv, tv, u[t], w[t]);
      }
    }
    // fold the tile's partial sums
#pragma unroll
    for (int t = 0; t < TPT; t++) {
      R v[6] = {u[t].x, u[t].y, u[t].z, w[t].x, w[t].y, w[t].z};
#pragma unroll
      for (int c = 0; c < NC; c++) {
        if (COMP) fold(S[t][c], C[t][c], v[c]); else S[t][c] += v[c];
      }
      u[t] = {0, 0, 0};
      w[t] = {0, 0, 0};
    }
    __syncthreads();
  }

  if (nsplit == 1) {
#pragma unroll
    for (int t = 0; t < TPT; t++) {
      const int i = tgt0 + threadIdx.x + t * THREADS;
      if (i >= t_hi) continue;
      const int o = i - t_lo;  // output row
      if (a.U && LMG_IN_BOUNDS(i < N, 5, i)) {
        a.U[3 * o] = bi[t] * (S[t][0] + C[t][0]);
        a.U[3 * o + 1] = bi[t] * (S[t][1] + C[t][1]);
        a.U[3 * o + 2] = bi[t] * (S[t][2] + C[t][2]);
      }
      if (ANG && a.W && LMG_IN_BOUNDS(i < N, 5, i)) {
        a.W[3 * o] = bi[t] * (S[t][NC - 3] + C[t][NC - 3]);
        a.W[3 * o + 1] = bi[t] * (S[t][NC - 2] + C[t][NC - 2]);
        a.W[3 * o + 2] = bi[t] * (S[t][NC - 1] + C[t][NC - 1]);
      }
    }
    return;
  }

  // ---- split sources: publish partials, last CTA of the tile reduces ----
  const size_t mine_off = ((size_t)(tile * nsplit + split) * (2 * NC)) * BT;
  R *mine = a.part + mine_off;
#pragma unroll
  for (int t = 0; t < TPT; t++) {
    const int l = threadIdx.x + t * THREADS;
#pragma unroll
    for (int c = 0; c < NC; c++) {
      if (LMG_IN_BOUNDS(mine_off + (size_t)(NC + c) * BT + l < a.part_cap, 2,
                        mine_off + (size_t)(NC + c) * BT + l)) {
        __stcg(mine + (size_t)c * BT + l, S[t][c]);
        __stcg(mine + (size_t)(NC + c) * BT + l, C[t][c]);
      }
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = LMG_IN_BOUNDS((size_t)tile < a.ticket_cap, 4, tile)
                              ? atomicAdd(a.ticket + tile, 1u) : 0u;
    s_last = (prev == (unsigned)(nsplit - 1));
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const R *base = a.part + ((size_t)tile * nsplit * (2 * NC)) * BT;
#pragma unroll
  for (int t = 0; t < TPT; t++) {
    const int l = threadIdx.x + t * THREADS;
    const int i = tgt0 + l;
    R Ss[NC], Cs[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) { Ss[c] = 0; Cs[c] = 0; }
    // UNR splits' partials are loaded before any is folded, so that many L2
    // reads are in flight at once (the fold order stays the split order)
    constexpr int UNR = 24 / NC;
    for (int s0 = 0; s0 < nsplit; s0 += UNR) {
      R sv[UNR][NC], cv[UNR][NC];
#pragma unroll
      for (int u = 0; u < UNR; u++) {
        // past the last split: re-read the last one (a valid address), add 0
        const bool in = s0 + u < nsplit &&
                        LMG_IN_BOUNDS(((size_t)tile * nsplit + s0 + u + 1) * (2 * NC) * BT <=
                                          a.part_cap, 3, tile);
        const R *ps = base + (size_t)(in ? s0 + u : nsplit - 1) * (2 * NC) * BT;
#pragma unroll
        for (int c = 0; c < NC; c++) {
          const R sl = __ldcg(ps + (size_t)c * BT + l);
          const R cl = __ldcg(ps + (size_t)(NC + c) * BT + l);
          sv[u][c] = in ? sl : R(0);
          cv[u][c] = in ? cl : R(0);
        }
      }
#pragma unroll
      for (int u = 0; u < UNR; u++) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
          if (COMP) fold(Ss[c], Cs[c], sv[u][c]); else Ss[c] += sv[u][c];
          Cs[c] += cv[u][c];
        }
      }
    }
    if (i < t_hi) {
      const int o = i - t_lo;  // output row
      if (a.U && LMG_IN_BOUNDS(i < N, 5, i)) {
        a.U[3 * o] = bi[t] * (Ss[0] + Cs[0]);
        a.U[3 * o + 1] = bi[t] * (Ss[1] + Cs[1]);
        a.U[3 * o + 2] = bi[t] * (Ss[2] + Cs[2]);
      }
      if (ANG && a.W && LMG_IN_BOUNDS(i < N, 5, i)) {
        a.W[3 * o] = bi[t] * (Ss[NC - 3] + Cs[NC - 3]);
        a.W[3 * o + 1] = bi[t] * (Ss[NC - 2] + Cs[NC - 2]);
        a.W[3 * o + 2] = bi[t] * (Ss[NC - 1] + Cs[NC - 1]);
      }
    }
  }
  if (threadIdx.x == 0) a.ticket[tile] = 0u;  // ready for the next launch
}

// Host-side launch description chosen by the planner.
struct MdotPlan {
  int threads = 128;
  int tpt = 1;
  int nsplit = 1;
  int chunk = 0;
  int tiles = 0;
  size_t part_elems = 0;  // scratch elements of R needed
  size_t tickets = 0;
};

}  // namespace lmg
