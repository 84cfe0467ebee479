// Packed FP32 arithmetic on pairs of targets (fma.rn.f32x2 and friends).
//
// The wall pair kernel is issue-bound: most of its instructions go to the FMA
// pipe.  Evaluating two targets per thread with packed instructions halves the
// issue slots of that arithmetic (the pipe itself runs a packed instruction in
// two passes, so the FP32 peak is unchanged; what is gained is issue
// bandwidth for everything else).
#pragma once
#include <cuda_runtime.h>

#include "rpy_pair.cuh"

namespace lmg {

struct F2 {
  float2 v;
};

__device__ __forceinline__ F2 bc(float a) { return {make_float2(a, a)}; }
__device__ __forceinline__ F2 mk2(float a, float b) { return {make_float2(a, b)}; }
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return {__fadd2_rn(a.v, b.v)}; }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return {__fmul2_rn(a.v, b.v)}; }
// a - b as a fused multiply-add with -1 (exact)
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
  return {__ffma2_rn(b.v, make_float2(-1.f, -1.f), a.v)};
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) { return {__ffma2_rn(a.v, b.v, c.v)}; }
__device__ __forceinline__ F2 neg2(F2 a) { return {__fmul2_rn(a.v, make_float2(-1.f, -1.f))}; }
// c - a b  (fma with -a: exact negation, one rounding)
__device__ __forceinline__ F2 fms2(F2 a, F2 b, F2 c) { return {__ffma2_rn(neg2(a).v, b.v, c.v)}; }
__device__ __forceinline__ F2 rsq2(F2 a) { return mk2(rsqrtf(a.v.x), rsqrtf(a.v.y)); }
__device__ __forceinline__ F2 rcp2(F2 a) {
  return mk2(__fdividef(1.0f, a.v.x), __fdividef(1.0f, a.v.y));
}

struct V3p {
  F2 x, y, z;
};

// Packed version of wall_pair_fused (rpy_pair.cuh) for two targets (lanes of
// xi, yi, hi) and one source whose values arrive already duplicated in both
// lanes (Xj = {xj, xj}, ...).  Same formulas, same order of operations per
// lane; pairs with r = 0 (self) or r < 2a (overlap) in either lane are
// evaluated lane by lane with the scalar code.
__device__ __forceinline__ void wall_pair_fused_x2(
    const PairConst<float> &k, const WallConst &K, F2 xi, F2 yi, F2 hi, F2 Xj, F2 Yj, F2 Hj,
    F2 Fx, F2 Fy, F2 Fz, F2 Tx, F2 Ty, F2 Tz, V3p &u, V3p &w) {
  const F2 dx = xi - Xj, dy = yi - Yj, dz = hi - Hj;
  const F2 sxy = fma2(dx, dx, dy * dy);
  const F2 r2 = fma2(dz, dz, sxy);
  if (r2.v.x < 4.0f || r2.v.y < 4.0f) {
    // rare: overlapping or self pair in a lane -> scalar evaluation per lane
    Vec3<float> u0 = {0, 0, 0}, w0 = {0, 0, 0}, u1 = {0, 0, 0}, w1 = {0, 0, 0};
    wall_pair_fused(k, K, xi.v.x, yi.v.x, hi.v.x, Xj.v.x, Yj.v.x, Hj.v.x, Fx.v.x, Fy.v.x,
                    Fz.v.x, Tx.v.x, Ty.v.x, Tz.v.x, u0, w0);
    wall_pair_fused(k, K, xi.v.y, yi.v.y, hi.v.y, Xj.v.y, Yj.v.y, Hj.v.y, Fx.v.y, Fy.v.y,
                    Fz.v.y, Tx.v.y, Ty.v.y, Tz.v.y, u1, w1);
    u.x = u.x + mk2(u0.x, u1.x);
    u.y = u.y + mk2(u0.y, u1.y);
    u.z = u.z + mk2(u0.z, u1.z);
    w.x = w.x + mk2(w0.x, w1.x);
    w.y = w.y + mk2(w0.y, w1.y);
    w.z = w.z + mk2(w0.z, w1.z);
    return;
  }
  const F2 Rz = hi + Hj;
  // far-field RPY coefficients (rpy_coefficients, r >= 2a)
  const F2 ir = rsq2(r2);
  const F2 ir2 = ir * ir;
  const F2 ir3 = ir2 * ir;
  const F2 f = ir * fma2(bc(k.tf1), ir2, bc(k.tf0));
  const F2 G = ir3 * fma2(bc(k.tg1), ir2, bc(k.tg0));
  const F2 fw = bc(k.rf1) * ir3;
  const F2 Gw = (bc(k.rg1) * ir3) * ir2;
  const F2 c = bc(k.rt0) * ir3;
  const F2 iR = rsq2(fma2(Rz, Rz, sxy));
  const F2 ex = dx * iR, ey = dy * iR, ez = Rz * iR;
  const F2 iRz = rcp2(Rz);
  const F2 hhj = Hj * iRz, hhi = hi * iRz;
  const F2 q = ez * ez;
  const F2 iR2 = iR * iR, iR3 = iR2 * iR, iR5 = iR3 * iR2, iR4 = iR2 * iR2;
  // translational image C2 merged with RPY UF
  const F2 h1q = fms2(hhj, hhj, hhj) * q;
  const F2 A = fma2(iR, fma2(bc(K.a11), h1q, bc(K.a10)),
                    fma2(iR3, fma2(bc(K.a31), q, bc(K.a30)), iR5 * fma2(bc(K.a51), q, bc(K.a50))));
  const F2 B = fma2(iR, fma2(bc(K.b11), h1q, bc(K.b10)),
                    fma2(iR3, fma2(bc(K.b31), q, bc(K.b30)), iR5 * fma2(bc(K.b51), q, bc(K.b50))));
  const F2 C = ez * fma2(iR, fma2(bc(K.c1h), hhj, bc(K.c11) * h1q),
                         fma2(iR3, fma2(bc(K.c31), q, bc(K.c30)),
                              iR5 * fma2(bc(K.c51), q, bc(K.c50))));
  const F2 D = ez * fma2(bc(K.d1) * hhj, iR, bc(K.d5) * iR5);
  const F2 E = fma2(bc(K.e1) * q, fma2(hhj * hhj, iR, iR3), iR5 * fma2(bc(K.e51), q, bc(K.e50)));
  const F2 ev = fma2(ex, Fx, fma2(ey, Fy, ez * Fz));
  const F2 dF = fma2(dx, Fx, fma2(dy, Fy, dz * Fz));
  const F2 fA = f + A;
  const F2 g = G * dF;
  const F2 s = fma2(B, ev, C * Fz);
  u.x = fma2(fA, Fx, fma2(g, dx, fma2(s, ex, u.x)));
  u.y = fma2(fA, Fy, fma2(g, dy, fma2(s, ey, u.y)));
  u.z = fma2(fA, Fz, fma2(g, dz, fma2(s, ez, fma2(D, ev, fma2(E, Fz, u.z)))));
  // rotational image C4 merged with RPY WT
  const F2 evT = fma2(ex, Tx, fma2(ey, Ty, ez * Tz));
  const F2 dT = fma2(dx, Tx, fma2(dy, Ty, dz * Tz));
  const F2 pv = fma2(ex, Ty, neg2(ey * Tx));  // (z x e).T
  const F2 f2w = bc(K.w2) * iR3;
  const F2 f4w = bc(-2.0f) * f2w;
  const F2 fwA = fma2(iR3, fma2(bc(K.w1), q, bc(K.w0)), fw);
  const F2 gw = Gw * dT;
  const F2 sT = f2w * evT;
  const F2 m = f4w * pv;
  w.x = fma2(fwA, Tx, fma2(gw, dx, fma2(sT, ex, fms2(m, ey, w.x))));
  w.y = fma2(fwA, Ty, fma2(gw, dy, fma2(sT, ey, fma2(m, ex, w.y))));
  w.z = fma2(fwA, Tz, fma2(gw, dz, fma2(sT, ez, fma2(f4w * ez, evT, w.z))));
  // couplings and the C3 images (WF with h_j, UT with h_i)
  const F2 f1 = bc(K.g0) * iR2;
  const F2 ga1 = (bc(K.g1) * q) * iR2;
  const F2 ga0 = iR4 * fma2(bc(K.g3), q, bc(K.g2));
  const F2 ezR2 = ez * iR2, ezR4 = ez * iR4;
  const F2 gb1 = bc(K.g4) * ezR2, gb0 = bc(K.g5) * ezR4;
  const F2 gc1 = bc(K.g6) * ezR2, gc0 = bc(K.g7) * ezR4;
  const F2 k1 = fma2(f1, iR, neg2(c));
  const F2 p = f1 * ez;
  const F2 k2 = fms2(c, dz, p);
  const F2 k3 = fma2(c, dz, p);
  const F2 f2j = fma2(ga1, hhj, ga0), f3j = fma2(gb1, hhj, gb0), f4j = fma2(gc1, hhj, gc0);
  const F2 gj = fma2(f3j, ev, f2j * Fz);
  const F2 k1dx = k1 * dx, k1dy = k1 * dy;
  const F2 k2f = k2 + f4j;
  w.x = fma2(k1dy, Fz, fms2(k2f, Fy, fma2(gj, ey, w.x)));
  w.y = fma2(k2f, Fx, fms2(k1dx, Fz, fms2(gj, ex, w.y)));
  w.z = fma2(k1, fma2(dx, Fy, neg2(dy * Fx)), w.z);
  const F2 f2i = fma2(ga1, hhi, ga0), f3i = fma2(gb1, hhi, gb0), f4i = fma2(gc1, hhi, gc0);
  const F2 mp = pv * f3i;
  const F2 k3f = k3 + f4i;
  u.x = fma2(k3f, Ty, fma2(k1dy, Tz, fms2(mp, ex, u.x)));
  u.y = fms2(k3f, Tx, fms2(k1dx, Tz, fms2(mp, ey, u.y)));
  u.z = fms2(k1, fma2(dy, Tx, neg2(dx * Ty)), fma2(mp, ez, fma2(pv, f2i, u.z)));
}

// Packed wall UF pair (forces only): the translational part of
// wall_pair_fused_x2 above (RPY UF merged with the translational image C2),
// same formulas and order of operations.  Pairs closer than 2a in either lane
// (the self pair included) are evaluated lane by lane with the scalar
// wall_pair_fused with zero torques, keeping its u.
__device__ __forceinline__ void wall_uf_pair_x2(const PairConst<float> &k, const WallConst &K,
                                                F2 xi, F2 yi, F2 hi, F2 Xj, F2 Yj, F2 Hj,
                                                F2 Fx, F2 Fy, F2 Fz, V3p &u) {
  const F2 dx = xi - Xj, dy = yi - Yj, dz = hi - Hj;
  const F2 sxy = fma2(dx, dx, dy * dy);
  const F2 r2 = fma2(dz, dz, sxy);
  if (r2.v.x < 4.0f || r2.v.y < 4.0f) {
    Vec3<float> u0 = {0, 0, 0}, w0 = {0, 0, 0}, u1 = {0, 0, 0}, w1 = {0, 0, 0};
    wall_pair_fused(k, K, xi.v.x, yi.v.x, hi.v.x, Xj.v.x, Yj.v.x, Hj.v.x, Fx.v.x, Fy.v.x,
                    Fz.v.x, 0.f, 0.f, 0.f, u0, w0);
    wall_pair_fused(k, K, xi.v.y, yi.v.y, hi.v.y, Xj.v.y, Yj.v.y, Hj.v.y, Fx.v.y, Fy.v.y,
                    Fz.v.y, 0.f, 0.f, 0.f, u1, w1);
    u.x = u.x + mk2(u0.x, u1.x);
    u.y = u.y + mk2(u0.y, u1.y);
    u.z = u.z + mk2(u0.z, u1.z);
    return;
  }
  const F2 Rz = hi + Hj;
  const F2 ir = rsq2(r2);
  const F2 ir2 = ir * ir;
  const F2 ir3 = ir2 * ir;
  const F2 f = ir * fma2(bc(k.tf1), ir2, bc(k.tf0));
  const F2 G = ir3 * fma2(bc(k.tg1), ir2, bc(k.tg0));
  const F2 iR = rsq2(fma2(Rz, Rz, sxy));
  const F2 ex = dx * iR, ey = dy * iR, ez = Rz * iR;
  const F2 hhj = Hj * rcp2(Rz);
  const F2 q = ez * ez;
  const F2 iR2 = iR * iR, iR3 = iR2 * iR, iR5 = iR3 * iR2;
  const F2 h1q = fms2(hhj, hhj, hhj) * q;
  const F2 A = fma2(iR, fma2(bc(K.a11), h1q, bc(K.a10)),
                    fma2(iR3, fma2(bc(K.a31), q, bc(K.a30)), iR5 * fma2(bc(K.a51), q, bc(K.a50))));
  const F2 B = fma2(iR, fma2(bc(K.b11), h1q, bc(K.b10)),
                    fma2(iR3, fma2(bc(K.b31), q, bc(K.b30)), iR5 * fma2(bc(K.b51), q, bc(K.b50))));
  const F2 C = ez * fma2(iR, fma2(bc(K.c1h), hhj, bc(K.c11) * h1q),
                         fma2(iR3, fma2(bc(K.c31), q, bc(K.c30)),
                              iR5 * fma2(bc(K.c51), q, bc(K.c50))));
  const F2 D = ez * fma2(bc(K.d1) * hhj, iR, bc(K.d5) * iR5);
  const F2 E = fma2(bc(K.e1) * q, fma2(hhj * hhj, iR, iR3), iR5 * fma2(bc(K.e51), q, bc(K.e50)));
  const F2 ev = fma2(ex, Fx, fma2(ey, Fy, ez * Fz));
  const F2 dF = fma2(dx, Fx, fma2(dy, Fy, dz * Fz));
  const F2 fA = f + A;
  const F2 g = G * dF;
  const F2 s = fma2(B, ev, C * Fz);
  u.x = fma2(fA, Fx, fma2(g, dx, fma2(s, ex, u.x)));
  u.y = fma2(fA, Fy, fma2(g, dy, fma2(s, ey, u.y)));
  u.z = fma2(fA, Fz, fma2(g, dz, fma2(s, ez, fma2(D, ev, fma2(E, Fz, u.z)))));
}

// Packed open-space UF pair (translational RPY, forces only) in the fast
// form of PairKernel::eval<false> (mdot.cuh): r^2 clamped at 4 for the
// coefficients, so overlapping and self pairs give finite values that the
// caller corrects; the smallest unclamped r^2 of each lane is kept in mr2.
// Same formulas and order of operations per lane as the scalar fast form.
__device__ __forceinline__ void open_uf_pair_x2(const PairConst<float> &k, F2 xi, F2 yi, F2 zi,
                                                F2 Xj, F2 Yj, F2 Zj, F2 Fx, F2 Fy, F2 Fz,
                                                V3p &u, float2 &mr2) {
  const F2 dx = xi - Xj, dy = yi - Yj, dz = zi - Zj;
  const F2 r2 = fma2(dx, dx, fma2(dy, dy, dz * dz));
  mr2.x = fminf(mr2.x, r2.v.x);
  mr2.y = fminf(mr2.y, r2.v.y);
  const F2 ir = mk2(rsqrt_normal<float>(fmaxf(r2.v.x, 4.0f)),
                    rsqrt_normal<float>(fmaxf(r2.v.y, 4.0f)));
  const F2 ir2 = ir * ir;
  const F2 ir3 = ir * ir2;
  const F2 f = ir * fma2(bc(k.tf1), ir2, bc(k.tf0));
  const F2 G = ir3 * fma2(bc(k.tg1), ir2, bc(k.tg0));
  const F2 g = G * fma2(dx, Fx, fma2(dy, Fy, dz * Fz));
  u.x = fma2(f, Fx, fma2(g, dx, u.x));
  u.y = fma2(f, Fy, fma2(g, dy, u.y));
  u.z = fma2(f, Fz, fma2(g, dz, u.z));
}

}  // namespace lmg
