// Symmetric open-space translational all-pairs product (FP32): kernel, plan
// and launch.  The scheme is described in mdot_sym.cuh.
#include <algorithm>
#include <cmath>

#include "bounds.cuh"
#include "grid_sync.cuh"
#include "launch_count.hpp"
#include "mdot.cuh"
#include "mdot_sym.cuh"
#include "pack2.cuh"

namespace lmg {

namespace {

// Largest partial-sum array the planner accepts (floats, 1 GiB).
constexpr size_t kSymMaxPartials = size_t(1) << 28;
// Fewest rotation steps a warp is given (below it, fewer blocks are launched).
constexpr long long kSymMinSteps = 4;
// Padding particles of a partial tile: zero force, placed 4 radii apart on a
// line far from the origin (their own sums are never read).
constexpr float kPadX = 1.0e6f;
constexpr int kElems = 3 * kSymTile;  // floats of one partial slot
constexpr int kFoldH = 2;              // pairs of output elements a thread folds per pass

struct SymArgs {
  const float *pos;
  const float *F;
  float *U;
  int N, nper, tpb, ntiles, nwarps, lg_rt, cmax;
  size_t part_elems;  // floats of part (index checks of the checked build)
  float inv_a;
  // far-field coefficients in both lanes, f = ir (tf0 + tf1 ir^2),
  // G = ir^3 (tg0 + tg1 ir^2), prefactor t0 folded in
  float2 tf0, tf1, tg0, tg1;
  PairConst<float> k;
  SymTables tab;
  float *part;
  unsigned long long *bar;
  int *err;
  // optional timeline (nanoseconds, %globaltimer): per warp [start, end of
  // its steps], then per block [after the barrier, end of the fold], then
  // per block the SM it ran on
  unsigned long long *trace;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ F2 as2(float2 v) { return {v}; }

// Fast form (r^2 clamped at 4) of one target i against two sources j (lanes)
// of a slot: adds M_ij F_j to ui (lanes: the two j) and M_ij F_i to uj.
__device__ __forceinline__ void sym_pair_x2(const SymArgs &a, F2 xi, F2 yi, F2 zi, F2 fxi,
                                            F2 fyi, F2 fzi, F2 xj, F2 yj, F2 zj, F2 fxj,
                                            F2 fyj, F2 fzj, V3p &ui, V3p &uj, float &mr) {
  const F2 dx = xi - xj, dy = yi - yj, dz = zi - zj;
  const F2 r2 = fma2(dx, dx, fma2(dy, dy, dz * dz));
  mr = fminf(mr, fminf(r2.v.x, r2.v.y));
  const F2 ir = mk2(rsqrt_normal<float>(fmaxf(r2.v.x, 4.0f)),
                    rsqrt_normal<float>(fmaxf(r2.v.y, 4.0f)));
  const F2 ir2 = ir * ir;
  const F2 f = ir * fma2(as2(a.tf1), ir2, as2(a.tf0));
  const F2 G = (ir * ir2) * fma2(as2(a.tg1), ir2, as2(a.tg0));
  const F2 gi = G * fma2(dx, fxj, fma2(dy, fyj, dz * fzj));
  ui.x = fma2(f, fxj, fma2(gi, dx, ui.x));
  ui.y = fma2(f, fyj, fma2(gi, dy, ui.y));
  ui.z = fma2(f, fzj, fma2(gi, dz, ui.z));
  const F2 gj = G * fma2(dx, fxi, fma2(dy, fyi, dz * fzi));
  uj.x = fma2(f, fxi, fma2(gj, dx, uj.x));
  uj.y = fma2(f, fyi, fma2(gj, dy, uj.y));
  uj.z = fma2(f, fzi, fma2(gj, dz, uj.z));
}

// Exact coefficients (near field below 2a, self pair at r = 0), as
// rpy_coefficients of the translational block.
__device__ __forceinline__ void exact_coeffs(const PairConst<float> &k, float r2, float &f,
                                             float &G) {
  float fw, Gw, c;
  rpy_coefficients<float, true, false, false, true>(k, r2, dev_rsqrt<float>(r2), f, G, fw, Gw,
                                                    c);
}

// The fast-form coefficients of sym_pair_x2 for one lane (same operations).
__device__ __forceinline__ void fast_coeffs(const SymArgs &a, float r2, float &f, float &G) {
  const float ir = rsqrt_normal<float>(fmaxf(r2, 4.0f));
  const float ir2 = __fmul_rn(ir, ir);
  f = __fmul_rn(ir, fmaf(a.tf1.x, ir2, a.tf0.x));
  G = __fmul_rn(__fmul_rn(ir, ir2), fmaf(a.tg1.x, ir2, a.tg0.x));
}

// Adds c_f F + c_g (d.F) d to (ux, uy, uz).
__device__ __forceinline__ void apply(float cf, float cg, float dx, float dy, float dz, float fx,
                                      float fy, float fz, float &ux, float &uy, float &uz) {
  const float g = cg * fmaf(dx, fx, fmaf(dy, fy, dz * fz));
  ux = fmaf(cf, fx, fmaf(g, dx, ux));
  uy = fmaf(cf, fy, fmaf(g, dy, uy));
  uz = fmaf(cf, fz, fmaf(g, dz, uz));
}

__device__ __forceinline__ void add_lane(F2 &v, int h, float x) {
  if (h) v.v.y += x; else v.v.x += x;
}

// The four particles of slot `lane` of a tile: scaled positions and forces
// (padding past the end of the batch).
struct Slot {
  float x[4], y[4], z[4], fx[4], fy[4], fz[4];
};

// Tile t of the batched layout: first particle and particles in it.
__device__ __forceinline__ int2 tile_desc(const SymArgs &a, int t) {
  const int b = t / a.tpb;
  const int I = t - b * a.tpb;
  return make_int2(b * a.nper + I * kSymTile, min(kSymTile, a.nper - I * kSymTile));
}

__device__ __forceinline__ void load_slot(const SymArgs &a, int2 td, int lane, Slot &s) {
  const int p0 = 4 * lane;
  if (p0 + 3 < td.y && LMG_IN_BOUNDS((size_t)td.x + p0 + 3 < (size_t)a.N, 11, td.x + p0)) {
    // 12 consecutive floats of positions and of forces (16-byte aligned)
    const float4 *P = reinterpret_cast<const float4 *>(a.pos + 3 * ((size_t)td.x + p0));
    const float4 *Fv = reinterpret_cast<const float4 *>(a.F + 3 * ((size_t)td.x + p0));
    const float4 v0 = __ldg(P), v1 = __ldg(P + 1), v2 = __ldg(P + 2);
    const float4 f0 = __ldg(Fv), f1 = __ldg(Fv + 1), f2 = __ldg(Fv + 2);
    s.x[0] = v0.x; s.y[0] = v0.y; s.z[0] = v0.z;
    s.x[1] = v0.w; s.y[1] = v1.x; s.z[1] = v1.y;
    s.x[2] = v1.z; s.y[2] = v1.w; s.z[2] = v2.x;
    s.x[3] = v2.y; s.y[3] = v2.z; s.z[3] = v2.w;
    s.fx[0] = f0.x; s.fy[0] = f0.y; s.fz[0] = f0.z;
    s.fx[1] = f0.w; s.fy[1] = f1.x; s.fz[1] = f1.y;
    s.fx[2] = f1.z; s.fy[2] = f1.w; s.fz[2] = f2.x;
    s.fx[3] = f2.y; s.fy[3] = f2.z; s.fz[3] = f2.w;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      s.x[q] = __fmul_rn(s.x[q], a.inv_a);
      s.y[q] = __fmul_rn(s.y[q], a.inv_a);
      s.z[q] = __fmul_rn(s.z[q], a.inv_a);
    }
  } else {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (p0 + q < td.y && LMG_IN_BOUNDS((size_t)td.x + p0 + q < (size_t)a.N, 11,
                                          td.x + p0 + q)) {
        const size_t g = 3 * ((size_t)td.x + p0 + q);
        s.x[q] = __fmul_rn(__ldg(a.pos + g), a.inv_a);
        s.y[q] = __fmul_rn(__ldg(a.pos + g + 1), a.inv_a);
        s.z[q] = __fmul_rn(__ldg(a.pos + g + 2), a.inv_a);
        s.fx[q] = __ldg(a.F + g);
        s.fy[q] = __ldg(a.F + g + 1);
        s.fz[q] = __ldg(a.F + g + 2);
      } else {
        s.x[q] = kPadX + 4.0f * (float)(p0 + q);
        s.y[q] = s.z[q] = s.fx[q] = s.fy[q] = s.fz[q] = 0.0f;
      }
    }
  }
}

// One rotation step of a lane: its slot (registers) against slot s of the
// warp's staged tile J4 [6][32] float4, j sums in A4 [3][32] float4.  Returns
// true if a pair of the step was closer than 2a (its fast value then needs
// the exact one, see correct_step).
__device__ __forceinline__ bool rotation_step(const SymArgs &a, const Slot &I, V3p (&ui)[4],
                                              const float4 *J4, float4 *A4, int s) {
  const float4 X = J4[s], Y = J4[32 + s], Z = J4[64 + s];
  const float4 FX = J4[96 + s], FY = J4[128 + s], FZ = J4[160 + s];
  const F2 xj[2] = {mk2(X.x, X.y), mk2(X.z, X.w)};
  const F2 yj[2] = {mk2(Y.x, Y.y), mk2(Y.z, Y.w)};
  const F2 zj[2] = {mk2(Z.x, Z.y), mk2(Z.z, Z.w)};
  const F2 fxj[2] = {mk2(FX.x, FX.y), mk2(FX.z, FX.w)};
  const F2 fyj[2] = {mk2(FY.x, FY.y), mk2(FY.z, FY.w)};
  const F2 fzj[2] = {mk2(FZ.x, FZ.y), mk2(FZ.z, FZ.w)};
  V3p aj[2];
#pragma unroll
  for (int h = 0; h < 2; h++) aj[h] = {bc(0.f), bc(0.f), bc(0.f)};
  float mr = 4.0f;
#pragma unroll
  for (int q = 0; q < 4; q++) {
#pragma unroll
    for (int h = 0; h < 2; h++)
      sym_pair_x2(a, bc(I.x[q]), bc(I.y[q]), bc(I.z[q]), bc(I.fx[q]), bc(I.fy[q]), bc(I.fz[q]),
                  xj[h], yj[h], zj[h], fxj[h], fyj[h], fzj[h], ui[q], aj[h], mr);
  }
  const float4 AX = A4[s], AY = A4[32 + s], AZ = A4[64 + s];
  const F2 ax0 = mk2(AX.x, AX.y) + aj[0].x, ax1 = mk2(AX.z, AX.w) + aj[1].x;
  const F2 ay0 = mk2(AY.x, AY.y) + aj[0].y, ay1 = mk2(AY.z, AY.w) + aj[1].y;
  const F2 az0 = mk2(AZ.x, AZ.y) + aj[0].z, az1 = mk2(AZ.z, AZ.w) + aj[1].z;
  A4[s] = make_float4(ax0.v.x, ax0.v.y, ax1.v.x, ax1.v.y);
  A4[32 + s] = make_float4(ay0.v.x, ay0.v.y, ay1.v.x, ay1.v.y);
  A4[64 + s] = make_float4(az0.v.x, az0.v.y, az1.v.x, az1.v.y);
  return mr < 4.0f;
}

// Two rotation steps at once: slot s0 with the j sums A4a and slot s1 with
// A4b (another copy, so the lanes' slots of both steps never collide).
// Returns the near flags of the two steps in bits 0 and 1.
__device__ __forceinline__ unsigned rotation_step2(const SymArgs &a, const Slot &I,
                                                   V3p (&ui)[4], const float4 *J4, float4 *A4a,
                                                   float4 *A4b, int s0, int s1) {
  F2 xj[4], yj[4], zj[4], fxj[4], fyj[4], fzj[4];
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const int s = u ? s1 : s0;
    const float4 X = J4[s], Y = J4[32 + s], Z = J4[64 + s];
    const float4 FX = J4[96 + s], FY = J4[128 + s], FZ = J4[160 + s];
    xj[2 * u] = mk2(X.x, X.y); xj[2 * u + 1] = mk2(X.z, X.w);
    yj[2 * u] = mk2(Y.x, Y.y); yj[2 * u + 1] = mk2(Y.z, Y.w);
    zj[2 * u] = mk2(Z.x, Z.y); zj[2 * u + 1] = mk2(Z.z, Z.w);
    fxj[2 * u] = mk2(FX.x, FX.y); fxj[2 * u + 1] = mk2(FX.z, FX.w);
    fyj[2 * u] = mk2(FY.x, FY.y); fyj[2 * u + 1] = mk2(FY.z, FY.w);
    fzj[2 * u] = mk2(FZ.x, FZ.y); fzj[2 * u + 1] = mk2(FZ.z, FZ.w);
  }
  V3p aj[4];
#pragma unroll
  for (int h = 0; h < 4; h++) aj[h] = {bc(0.f), bc(0.f), bc(0.f)};
  float mr0 = 4.0f, mr1 = 4.0f;
#pragma unroll
  for (int q = 0; q < 4; q++) {
#pragma unroll
    for (int h = 0; h < 4; h++)
      sym_pair_x2(a, bc(I.x[q]), bc(I.y[q]), bc(I.z[q]), bc(I.fx[q]), bc(I.fy[q]), bc(I.fz[q]),
                  xj[h], yj[h], zj[h], fxj[h], fyj[h], fzj[h], ui[q], aj[h], h < 2 ? mr0 : mr1);
  }
#pragma unroll
  for (int u = 0; u < 2; u++) {
    float4 *A4 = u ? A4b : A4a;
    const int s = u ? s1 : s0;
    const float4 AX = A4[s], AY = A4[32 + s], AZ = A4[64 + s];
    const F2 ax0 = mk2(AX.x, AX.y) + aj[2 * u].x, ax1 = mk2(AX.z, AX.w) + aj[2 * u + 1].x;
    const F2 ay0 = mk2(AY.x, AY.y) + aj[2 * u].y, ay1 = mk2(AY.z, AY.w) + aj[2 * u + 1].y;
    const F2 az0 = mk2(AZ.x, AZ.y) + aj[2 * u].z, az1 = mk2(AZ.z, AZ.w) + aj[2 * u + 1].z;
    A4[s] = make_float4(ax0.v.x, ax0.v.y, ax1.v.x, ax1.v.y);
    A4[32 + s] = make_float4(ay0.v.x, ay0.v.y, ay1.v.x, ay1.v.y);
    A4[64 + s] = make_float4(az0.v.x, az0.v.y, az1.v.x, az1.v.y);
  }
  return (mr0 < 4.0f ? 1u : 0u) | (mr1 < 4.0f ? 2u : 0u);
}

__device__ __forceinline__ float comp4(const float4 &v, int r) {
  return r == 0 ? v.x : (r == 1 ? v.y : (r == 2 ? v.z : v.w));
}
__device__ __forceinline__ void set_comp4(float4 &v, int r, float x) {
  if (r == 0) v.x = x; else if (r == 1) v.y = x; else if (r == 2) v.z = x; else v.w = x;
}
__device__ __forceinline__ float sel4(const float (&v)[4], int q) {
  return q == 0 ? v[0] : (q == 1 ? v[1] : (q == 2 ? v[2] : v[3]));
}

// For a step whose pairs were all taken in the fast form: adds (exact - fast)
// for those closer than 2a, to the lane's sums and to slot s's j sums.  The
// distances of the step's 16 pairs give a mask first; only the near pairs
// (rare) are then evaluated, in (q, r) order.
__device__ __forceinline__ void correct_step(const SymArgs &a, const Slot &I, V3p (&ui)[4],
                                             const float4 *J4, float4 *A4, int s) {
  const float4 X = J4[s], Y = J4[32 + s], Z = J4[64 + s];
  unsigned mask = 0u;
#pragma unroll
  for (int q = 0; q < 4; q++) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const float dx = I.x[q] - comp4(X, r), dy = I.y[q] - comp4(Y, r),
                  dz = I.z[q] - comp4(Z, r);
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      if (r2 < 4.0f) mask |= 1u << (4 * q + r);
    }
  }
  if (mask == 0u) return;
  const float4 FX = J4[96 + s], FY = J4[128 + s], FZ = J4[160 + s];
  float4 AX = A4[s], AY = A4[32 + s], AZ = A4[64 + s];
  while (mask) {
    const int b = __ffs(mask) - 1;
    mask &= mask - 1u;
    const int q = b >> 2, r = b & 3;
    const float xj = comp4(X, r), yj = comp4(Y, r), zj = comp4(Z, r);
    const float dx = sel4(I.x, q) - xj, dy = sel4(I.y, q) - yj, dz = sel4(I.z, q) - zj;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float fe, Ge, ff, Gf;
    exact_coeffs(a.k, r2, fe, Ge);
    fast_coeffs(a, 4.0f, ff, Gf);  // the fast form clamps r^2 < 4 to 4
    const float df = fe - ff, dG = Ge - Gf;
    float ux = 0.f, uy = 0.f, uz = 0.f;
    apply(df, dG, dx, dy, dz, comp4(FX, r), comp4(FY, r), comp4(FZ, r), ux, uy, uz);
    float ax = comp4(AX, r), ay = comp4(AY, r), az = comp4(AZ, r);
    apply(df, dG, dx, dy, dz, sel4(I.fx, q), sel4(I.fy, q), sel4(I.fz, q), ax, ay, az);
    set_comp4(AX, r, ax);
    set_comp4(AY, r, ay);
    set_comp4(AZ, r, az);
    const int h = r & 1;
#pragma unroll
    for (int qq = 0; qq < 4; qq++) {
      if (qq == q) {
        add_lane(ui[qq].x, h, ux);
        add_lane(ui[qq].y, h, uy);
        add_lane(ui[qq].z, h, uz);
      }
    }
  }
  A4[s] = AX;
  A4[32 + s] = AY;
  A4[64 + s] = AZ;
}

// Pairs inside the lane's own slot (q < r) and the self pairs, exactly.
__device__ __forceinline__ void own_slot(const SymArgs &a, const Slot &I, V3p (&ui)[4]) {
#pragma unroll
  for (int q = 0; q < 4; q++) {
    add_lane(ui[q].x, 0, a.k.t0 * I.fx[q]);
    add_lane(ui[q].y, 0, a.k.t0 * I.fy[q]);
    add_lane(ui[q].z, 0, a.k.t0 * I.fz[q]);
#pragma unroll
    for (int r = q + 1; r < 4; r++) {
      const float dx = I.x[q] - I.x[r], dy = I.y[q] - I.y[r], dz = I.z[q] - I.z[r];
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      float f, G;
      exact_coeffs(a.k, r2, f, G);
      float ux = 0.f, uy = 0.f, uz = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
      apply(f, G, dx, dy, dz, I.fx[r], I.fy[r], I.fz[r], ux, uy, uz);
      apply(f, G, dx, dy, dz, I.fx[q], I.fy[q], I.fz[q], vx, vy, vz);
      add_lane(ui[q].x, 0, ux); add_lane(ui[q].y, 0, uy); add_lane(ui[q].z, 0, uz);
      add_lane(ui[r].x, 0, vx); add_lane(ui[r].y, 0, vy); add_lane(ui[r].z, 0, vz);
    }
  }
}

__device__ __forceinline__ void store12(float *p, const float (&v)[12]) {
  float4 *q = reinterpret_cast<float4 *>(p);
  __stcg(q, make_float4(v[0], v[1], v[2], v[3]));
  __stcg(q + 1, make_float4(v[4], v[5], v[6], v[7]));
  __stcg(q + 2, make_float4(v[8], v[9], v[10], v[11]));
}

template <int MINB>
__global__ void __launch_bounds__(kSymThreads, MINB) mdot_sym_kernel(const SymArgs a) {
  __shared__ __align__(16) float sj[4][6][kSymTile];     // staged tile J, one per warp
  __shared__ __align__(16) float sa[4][2][3][kSymTile];  // j sums, two copies per warp

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = blockIdx.x * (kSymThreads / 32) + warp;
  float4 *J4 = reinterpret_cast<float4 *>(&sj[warp][0][0]);       // [6][32]
  float4 *A4 = reinterpret_cast<float4 *>(&sa[warp][0][0][0]);    // [3][32]
  float4 *A4b = reinterpret_cast<float4 *>(&sa[warp][1][0][0]);   // second copy

  if (a.trace && lane == 0) a.trace[2 * gw] = global_ns();
  if (gw < a.nwarps) {
    const int4 w0 = __ldg(a.tab.warps + 2 * gw);
    int4 pr = __ldg(a.tab.warps + 2 * gw + 1);  // entry of the first pair
    int p = w0.x, k0 = w0.y, left = w0.z, pseg = w0.w;
    while (left > 0) {
      const bool diag = pr.x == pr.y;
      const int n = min((diag ? 16 : 32) - k0, left);
      // the next pair's entry is fetched while this one runs
      int4 pr_next = pr;
      int pseg_next = pseg;
      if (left > n) {
        pr_next = __ldg(a.tab.pairs + p + 1);
        pseg_next = __ldg(a.tab.pseg + p + 1);
      }
      Slot I;
      {
        Slot Jl;
        load_slot(a, tile_desc(a, pr.y), lane, Jl);
        J4[lane] = make_float4(Jl.x[0], Jl.x[1], Jl.x[2], Jl.x[3]);
        J4[32 + lane] = make_float4(Jl.y[0], Jl.y[1], Jl.y[2], Jl.y[3]);
        J4[64 + lane] = make_float4(Jl.z[0], Jl.z[1], Jl.z[2], Jl.z[3]);
        J4[96 + lane] = make_float4(Jl.fx[0], Jl.fx[1], Jl.fx[2], Jl.fx[3]);
        J4[128 + lane] = make_float4(Jl.fy[0], Jl.fy[1], Jl.fy[2], Jl.fy[3]);
        J4[160 + lane] = make_float4(Jl.fz[0], Jl.fz[1], Jl.fz[2], Jl.fz[3]);
        if (diag) I = Jl; else load_slot(a, tile_desc(a, pr.x), lane, I);
      }
      const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
      A4[lane] = zero4;
      A4[32 + lane] = zero4;
      A4[64 + lane] = zero4;
      A4b[lane] = zero4;
      A4b[32 + lane] = zero4;
      A4b[64 + lane] = zero4;
      __syncwarp();
      V3p ui[4];
#pragma unroll
      for (int q = 0; q < 4; q++) ui[q] = {bc(0.f), bc(0.f), bc(0.f)};
      // steps whose pairs include one closer than 2a (bit k - k0): their
      // fast values are corrected after the loop
      unsigned near = 0u;
      int k = k0;
      if (diag && k == 0) {
        // pairs inside each slot, and slot pairs at distance 16 (once)
        own_slot(a, I, ui);
        if (lane < 16 && rotation_step(a, I, ui, J4, A4, (lane + 16) & 31)) near |= 1u;
        __syncwarp();
        k++;
      }
      // two steps at a time (the second on the other copy of the j sums)
      for (; k + 1 < k0 + n; k += 2) {
        near |= rotation_step2(a, I, ui, J4, A4, A4b, (lane + k) & 31, (lane + k + 1) & 31)
                << (k - k0);
        // the slots are read by other lanes at the next steps
        __syncwarp();
      }
      if (k < k0 + n) {
        if (rotation_step(a, I, ui, J4, A4, (lane + k) & 31)) near |= 1u << (k - k0);
        __syncwarp();
      }
      // the flagged steps of any lane, in step order (at one step the lanes'
      // slots are all different)
      for (unsigned steps = __reduce_or_sync(0xffffffffu, near); steps != 0u;
           steps &= steps - 1u) {
        const int kk = __ffs(steps) - 1;
        if ((near >> kk) & 1u) {
          const int kabs = k0 + kk;
          correct_step(a, I, ui, J4, A4, (lane + (diag && kabs == 0 ? 16 : kabs)) & 31);
        }
        __syncwarp();
      }
      // ---- publish this warp's sums for the pair ----
      const int seg = gw - (pseg >> 8);
      float vi[12];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        vi[3 * q] = ui[q].x.v.x + ui[q].x.v.y;
        vi[3 * q + 1] = ui[q].y.v.x + ui[q].y.v.y;
        vi[3 * q + 2] = ui[q].z.v.x + ui[q].z.v.y;
      }
      float4 AX = A4[lane], AY = A4[32 + lane], AZ = A4[64 + lane];
      {
        const float4 BX = A4b[lane], BY = A4b[32 + lane], BZ = A4b[64 + lane];
        AX = make_float4(AX.x + BX.x, AX.y + BX.y, AX.z + BX.z, AX.w + BX.w);
        AY = make_float4(AY.x + BY.x, AY.y + BY.y, AY.z + BY.z, AY.w + BY.w);
        AZ = make_float4(AZ.x + BZ.x, AZ.y + BZ.y, AZ.z + BZ.z, AZ.w + BZ.w);
      }
      float vj[12] = {AX.x, AY.x, AZ.x, AX.y, AY.y, AZ.y,
                      AX.z, AY.z, AZ.z, AX.w, AY.w, AZ.w};
      const size_t si = (size_t)(pr.z + seg) * kElems, sj = (size_t)(pr.w + seg) * kElems;
      if (diag) {
#pragma unroll
        for (int c = 0; c < 12; c++) vi[c] += vj[c];
        if (LMG_IN_BOUNDS(si + kElems <= a.part_elems, 12, pr.z + seg))
          store12(a.part + si + 12 * lane, vi);
      } else {
        if (LMG_IN_BOUNDS(si + kElems <= a.part_elems, 12, pr.z + seg))
          store12(a.part + si + 12 * lane, vi);
        if (LMG_IN_BOUNDS(sj + kElems <= a.part_elems, 12, pr.w + seg))
          store12(a.part + sj + 12 * lane, vj);
      }
      // the staged tile and the sums are overwritten by the next pair
      __syncwarp();
      left -= n;
      p++;
      k0 = 0;
      pr = pr_next;
      pseg = pseg_next;
    }
  }
  if (a.trace && lane == 0) a.trace[2 * gw + 1] = global_ns();

  // ---- every partial is written: fold them into U ----
  if (!grid_barrier_mono(a.bar)) {
    if (threadIdx.x == 0) *a.err = 1;
    return;
  }
  const size_t tb = 2 * (size_t)gridDim.x * (kSymThreads / 32) + 2 * blockIdx.x;
  if (a.trace && threadIdx.x == 0) {
    a.trace[tb] = global_ns();
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    a.trace[2 * (size_t)gridDim.x * (kSymThreads / 32) + 2 * gridDim.x + blockIdx.x] = smid;
  }
  // kFoldH pairs of adjacent output elements per thread and pass, sixteen
  // float2 loads of each in flight: a warp's lanes read 8 consecutive elements
  // of each of rt slots (whole 32-byte sectors); at N = 4096 one pass covers
  // every element
  const int rt = 1 << a.lg_rt;
  constexpr int kPairs = kElems / 2;
  const unsigned total = (unsigned)a.ntiles * kPairs * rt;
  const unsigned stride = gridDim.x * blockDim.x;
  for (unsigned base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total;
       base += kFoldH * stride) {
    float S[kFoldH][2], C[kFoldH][2];
    int t[kFoldH], e[kFoldH], sub[kFoldH], cnt[kFoldH];
    bool in[kFoldH];
    const float2 *src[kFoldH];
    int cmx = 0;
#pragma unroll
    for (int h = 0; h < kFoldH; h++) {
      S[h][0] = S[h][1] = C[h][0] = C[h][1] = 0.f;
      const unsigned g = base + h * stride + lane;
      in[h] = g < total;
      const unsigned el = in[h] ? g >> a.lg_rt : 0u;  // pair of elements (2 el, 2 el + 1)
      sub[h] = (int)(g & (unsigned)(rt - 1));
      t[h] = (int)(el / kPairs);
      e[h] = 2 * (int)(el - (unsigned)t[h] * kPairs);
      src[h] = reinterpret_cast<const float2 *>(a.part + (size_t)t[h] * a.cmax * kElems + e[h]);
      cnt[h] = in[h] ? a.cmax : 0;
      cmx = max(cmx, cnt[h]);
    }
    // each tile's slot range, in slot order (share `sub` of every rt)
    for (int m0 = 0; m0 < cmx; m0 += 16 * rt) {
      float2 v[kFoldH][16];
#pragma unroll
      for (int h = 0; h < kFoldH; h++)
#pragma unroll
        for (int m = 0; m < 16; m++) {
          const int j = m0 + sub[h] + m * rt;
          v[h][m] = (j < cnt[h] &&
                     LMG_IN_BOUNDS(((size_t)t[h] * a.cmax + j + 1) * kElems <= a.part_elems, 13,
                                   t[h]))
                        ? __ldcg(src[h] + (size_t)j * kPairs) : make_float2(0.f, 0.f);
        }
#pragma unroll
      for (int h = 0; h < kFoldH; h++)
#pragma unroll
        for (int m = 0; m < 16; m++) {
          fold(S[h][0], C[h][0], v[h][m].x);
          fold(S[h][1], C[h][1], v[h][m].y);
        }
    }
#pragma unroll
    for (int h = 0; h < kFoldH; h++) {
#pragma unroll
      for (int c = 0; c < 2; c++) {
        // combine the rt shares (the same value lands in every lane of a group)
        for (int o = 1; o < rt; o <<= 1) {
          const float S2 = __shfl_xor_sync(0xffffffffu, S[h][c], o);
          const float C2 = __shfl_xor_sync(0xffffffffu, C[h][c], o);
          const float sm = S[h][c] + S2;
          const float bp = sm - S[h][c];
          const float err = (S[h][c] - (sm - bp)) + (S2 - bp);  // exact, symmetric in (S, S2)
          C[h][c] = (C[h][c] + C2) + err;
          S[h][c] = sm;
        }
      }
      if (in[h] && sub[h] == 0) {
        const int2 td = tile_desc(a, t[h]);
#pragma unroll
        for (int c = 0; c < 2; c++)
          if (e[h] + c < 3 * td.y &&
              LMG_IN_BOUNDS(3 * (size_t)td.x + e[h] + c < 3 * (size_t)a.N, 14, td.x))
            a.U[3 * (size_t)td.x + e[h] + c] = S[h][c] + C[h][c];
      }
    }
  }
  if (a.trace) {
    __syncthreads();
    if (threadIdx.x == 0) a.trace[tb + 1] = global_ns();
  }
}

// Register budget of the kernel: 2 resident blocks per SM (up to 255
// registers a thread; the default: no spills, the rotation loop keeps the
// broadcast slot values and two steps' sums in registers), 3 (168) or 4
// (128, spills).  Measured at N = 4096 / 16384 / 65536: 22.1 / 192 / 2973 us
// with 2, 25.1 / 193 / 2922 us with 3, 27.1 / 200 / 3008 us with 4.
const void *sym_kernel(int variant) {
  if (variant == 3) return (const void *)mdot_sym_kernel<3>;
  if (variant == 4) return (const void *)mdot_sym_kernel<4>;
  return (const void *)mdot_sym_kernel<2>;
}

}  // namespace

unsigned long long bounds_status_sym(bool reset) { return bounds_status_here(reset); }

cudaError_t mdot_sym_plan(int N, int nper, int num_sms, int force_warps, SymPlan &p) {
  const int v = g_sym_variant.load();
  const int variant = (v == 3 || v == 4) ? v : 2;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sym_kernel(variant),
                                                                kSymThreads, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorNotSupported;
  e = mdot_sym_plan_tables(N, nper, (long long)per_sm * num_sms, force_warps, p);
  p.variant = variant;
  return e;
}

cudaError_t mdot_sym_plan_tables(int N, int nper, long long resident, int force_warps,
                                 SymPlan &p) {
  p = SymPlan{};
  if (N <= 0 || nper <= 0 || N % nper != 0 || resident < 1) return cudaErrorNotSupported;
  p.N = N;
  p.nper = nper;
  p.nbatch = N / nper;
  if (p.nbatch > 1 && nper % 4 != 0) return cudaErrorNotSupported;  // float4 slot loads
  p.tpb = (nper + kSymTile - 1) / kSymTile;
  const int tpb = p.tpb;
  const long long ntiles = (long long)p.nbatch * tpb;
  const long long ppb = (long long)tpb * (tpb + 1) / 2;  // tile pairs per batch
  const long long npairs = p.nbatch * ppb;
  if (ntiles * kElems * 32 >= (1LL << 31) || npairs >= (1LL << 30))
    return cudaErrorNotSupported;
  // steps of the schedule: batch by batch, tile row by tile row, the
  // diagonal tile (16 steps) then the tiles to its right (32 steps each)
  const long long W = p.nbatch * (16LL * tpb + 32LL * (ppb - tpb));
  p.steps = W;
  const long long wpb = kSymThreads / 32;
  const long long want = std::max(1LL, (W + wpb * kSymMinSteps - 1) / (wpb * kSymMinSteps));
  p.grid = (int)std::min(resident, want);
  p.nwarps = (int)std::min<long long>(wpb * p.grid, W);
  if (force_warps > 0 && force_warps < p.nwarps) {
    p.nwarps = force_warps;
    p.grid = (int)((force_warps + wpb - 1) / wpb);
  }
  const long long NW = p.nwarps;
  auto bound = [&](long long w) { return w * W / NW; };             // first step of warp w
  auto warp_of = [&](long long x) { return ((x + 1) * NW - 1) / W; };  // warp holding step x
  auto pidx = [&](long long b, int lo, int hi) {  // pair (lo, hi), lo <= hi, of batch b
    return b * ppb + (long long)lo * tpb - (long long)lo * (lo - 1) / 2 + (hi - lo);
  };
  // warps touching each pair
  p.pseg.resize(npairs);
  std::vector<int> nseg(npairs);
  std::vector<long long> pstart(npairs);
  long long x = 0, pi = 0;
  for (long long b = 0; b < p.nbatch; b++) {
    for (int I = 0; I < tpb; I++) {
      for (int J = I; J < tpb; J++, pi++) {
        const int len = I == J ? 16 : 32;
        const long long first = warp_of(x), last = warp_of(x + len - 1);
        nseg[pi] = (int)(last - first + 1);
        if (nseg[pi] > 255 || first >= (1LL << 23)) return cudaErrorNotSupported;
        p.pseg[pi] = (int)((first << 8) | nseg[pi]);
        pstart[pi] = x;
        x += len;
      }
    }
  }
  // slot ranges: tile by tile, partner by partner, warp by warp; every tile
  // gets the same stride (the largest count)
  p.tused.assign(ntiles, 0);
  for (long long t = 0; t < ntiles; t++) {
    const long long b = t / tpb;
    const int I = (int)(t % tpb);
    long long c = 0;
    for (int s = 0; s < tpb; s++) c += nseg[pidx(b, std::min(I, s), std::max(I, s))];
    if (c >= (1LL << 20)) return cudaErrorNotSupported;
    p.tused[t] = (int)c;
    p.cmax = std::max(p.cmax, (int)c);
  }
  if ((size_t)ntiles * p.cmax >= (size_t(1) << 31)) return cudaErrorNotSupported;
  p.pairs.resize(npairs);
  for (long long t = 0; t < ntiles; t++) {
    const long long b = t / tpb;
    const int I = (int)(t % tpb);
    long long slot = t * p.cmax;
    for (int s = 0; s < tpb; s++) {
      const int lo = std::min(I, s), hi = std::max(I, s);
      const long long q = pidx(b, lo, hi);
      if (s >= I) {  // this tile is the pair's I side (or the diagonal)
        p.pairs[q].x = (int)(b * tpb + lo);
        p.pairs[q].y = (int)(b * tpb + hi);
        p.pairs[q].z = (int)slot;
      } else {
        p.pairs[q].w = (int)slot;
      }
      slot += nseg[q];
    }
  }
  p.slots = (size_t)ntiles * p.cmax;
  p.part_elems = p.slots * kElems;
  if (p.part_elems > kSymMaxPartials) return cudaErrorNotSupported;
  // warps: first pair, step and count, with that pair's entries
  p.warps.resize(2 * NW);
  pi = 0;
  for (long long w = 0; w < NW; w++) {
    const long long b0 = bound(w);
    while (pstart[pi] + (p.pairs[pi].x == p.pairs[pi].y ? 16 : 32) <= b0) pi++;
    p.warps[2 * w] = make_int4((int)pi, (int)(b0 - pstart[pi]), (int)(bound(w + 1) - b0),
                               p.pseg[pi]);
    p.warps[2 * w + 1] = p.pairs[pi];
  }
  // threads per output element in the final fold: at most ~16 slots each
  int rt = 1;
  while (rt < 32 && rt * 16 < p.cmax) rt *= 2;
  p.rt = rt;
  return cudaSuccess;
}

cudaError_t mdot_sym_launch(const SymPlan &p, const SymTables &tab, const float *pos,
                            const float *F, float *U, float inv_a, const PairConst<float> &k,
                            float *part, unsigned long long *bar, int *err,
                            cudaStream_t stream) {
  if (p.grid <= 0) return cudaErrorInvalidValue;
  SymArgs a{};
  a.pos = pos;
  a.F = F;
  a.U = U;
  a.N = p.N;
  a.nper = p.nper;
  a.tpb = p.tpb;
  a.ntiles = p.nbatch * p.tpb;
  a.part_elems = p.part_elems;
  a.nwarps = p.nwarps;
  a.cmax = p.cmax;
  int lg = 0;
  while ((1 << lg) < p.rt) lg++;
  a.lg_rt = lg;
  a.inv_a = inv_a;
  a.tf0 = make_float2(k.tf0, k.tf0);
  a.tf1 = make_float2(k.tf1, k.tf1);
  a.tg0 = make_float2(k.tg0, k.tg0);
  a.tg1 = make_float2(k.tg1, k.tg1);
  a.k = k;
  a.tab = tab;
  a.part = part;
  a.bar = bar;
  a.err = err;
  a.trace = g_sym_trace.load();
  void *params[] = {(void *)&a};
  count_launch();
  return cudaLaunchCooperativeKernel(sym_kernel(p.variant), dim3(p.grid), dim3(kSymThreads),
                                     params, 0, stream);
}

}  // namespace lmg
