// Pair physics of the NBody Rotne-Prager-Yamakawa mobility, open boundary and
// single bottom wall, written for the tiled all-pairs kernels.
//
// Physics follows libMobility solvers/NBody/extra/hydrodynamicKernels.cuh:
//   RPY_UF :41-57, RPY_WT :63-86, RPY_UT/RPY_WF :89-118 (open-space blocks),
//   wallCorrection_UF :187-249, _WT :253-282, _UT :287-319, _WF :324-359,
//   BottomWall::dotProduct :362-441 (damping b_i b_j, heights clamped at a,
//   image vector r_ij + 2 h_j z, UT evaluated with -r_ij + 2 h_i z).
//
// Representation chosen here (not the reference's entry-by-entry matrices):
//   * all lengths are divided by the hydrodynamic radius a when a source or a
//     target is loaded, so r~ = r/a appears directly;
//   * each 3x3 block is applied in vector form, e.g. the translational wall
//     image tensor C2 is  A I + B e e^T + C e z^T + D z e^T + E z z^T,
//     so   C2.v = A v + B (e.v) e + C v_z e + D (e.v) z + E v_z z;
//   * the antisymmetric couplings are cross products, M_UT T = c (T x d),
//     the wall image C3 of WF is f1 (e x F) + (f3 (e.F) + f2 F_z)(e x z)
//     + f4 (z x F), and UT uses its transpose;
//   * the image vector R = (dx, dy, h_i + h_j) is shared by all four blocks
//     (UT uses (-dx, -dy, h_i + h_j)), so one rsqrt serves every block;
//   * the damping b_i b_j and the block prefactors t0, r0, rt0 are applied
//     outside the pair loop (sources are pre-multiplied by b_j, targets by
//     b_i, prefactors folded into per-launch constants).
#pragma once
#include <cuda_runtime.h>

namespace lmg {

template <class R> struct Vec3 { R x, y, z; };

template <class R> __device__ __forceinline__ R dev_rsqrt(R x);
template <> __device__ __forceinline__ float dev_rsqrt<float>(float x) { return rsqrtf(x); }
template <> __device__ __forceinline__ double dev_rsqrt<double>(double x) { return rsqrt(x); }

// Reciprocal square root for arguments known to be normal numbers (r^2
// clamped at 4): the hardware approximation without the subnormal handling.
template <class R> __device__ __forceinline__ R rsqrt_normal(R x);
template <> __device__ __forceinline__ float rsqrt_normal<float>(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
template <> __device__ __forceinline__ double rsqrt_normal<double>(double x) { return rsqrt(x); }

template <class R> __device__ __forceinline__ R fmaR(R a, R b, R c);
template <> __device__ __forceinline__ float fmaR<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <> __device__ __forceinline__ double fmaR<double>(double a, double b, double c) { return fma(a, b, c); }

// Multiplication that the compiler may not contract into an FMA with a
// following subtraction: targets and sources are scaled by 1/a with it, so a
// particle paired with itself (or with a coincident one) yields exactly d = 0.
template <class R> __device__ __forceinline__ R mul_rn(R a, R b);
template <> __device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }

template <class R> __device__ __forceinline__ R dev_div(R a, R b);
template <> __device__ __forceinline__ float dev_div<float>(float a, float b) { return __fdividef(a, b); }
template <> __device__ __forceinline__ double dev_div<double>(double a, double b) { return a / b; }

// Per-launch constants, prefactors already folded in.
template <class R> struct PairConst {
  // translational RPY, far:  f = ir*(tf0 + tf1*ir2), G = ir3*(tg0 + tg1*ir2)
  R tf0, tf1, tg0, tg1;
  // translational RPY, near: f = t0 - tn1*r, G = tn2*ir
  R t0, tn1, tn2;
  // rotational RPY, far: f = rf1*ir3, G = rg1*ir5
  R rf1, rg1;
  // rotational RPY, near: f = r0 + rn1*r + rn3*r^3, G = rn2*ir + rn4*r
  R r0, rn1, rn3, rn2, rn4;
  // coupling: far c = rt0*ir3, near c = rt0*(1/2 - 3/16 r)
  R rt0, cn0, cn1;
};

template <class R>
inline PairConst<R> make_pair_const(double t0, double r0, double rt0) {
  PairConst<R> c;
  c.tf0 = R(0.75 * t0);
  c.tf1 = R(0.5 * t0);
  c.tg0 = R(0.75 * t0);
  c.tg1 = R(-1.5 * t0);
  c.t0 = R(t0);
  c.tn1 = R(0.28125 * t0);  // 9/32
  c.tn2 = R(0.09375 * t0);  // 3/32
  c.rf1 = R(-0.5 * r0);
  c.rg1 = R(1.5 * r0);
  c.r0 = R(r0);
  c.rn1 = R(-0.84375 * r0);  // 27/32
  c.rn3 = R(0.078125 * r0);  // 5/64
  c.rn2 = R(0.28125 * r0);   // 9/32
  c.rn4 = R(-0.046875 * r0); // 3/64
  c.rt0 = R(rt0);
  c.cn0 = R(0.5 * rt0);
  c.cn1 = R(-0.1875 * rt0);  // 1/2 * 3/8
  return c;
}

// Open-space RPY scalar coefficients for a pair at scaled distance r (r2 =
// r^2, ir = 1/r).  U_UF = f F + G (d.F) d ; W_WT = fw T + Gw (d.T) d ;
// coupling c:  U_UT = c (T x d), W_WF = c (F x d).  Self pair (r2 == 0):
// f = t0, fw = r0, G = Gw = c = 0 (d = 0 makes the coupling vanish anyway).
// NEAR = false evaluates the far-field formulas for every pair (callers that
// detect r < 2a themselves and redo those pairs).
template <class R, bool TT, bool ROT, bool CPL, bool NEAR = true>
__device__ __forceinline__ void rpy_coefficients(const PairConst<R> &k, R r2, R ir,
                                                 R &f, R &G, R &fw, R &Gw, R &c) {
  const R ir2 = ir * ir;
  const R ir3 = ir * ir2;
  if (TT) {
    f = ir * (k.tf0 + k.tf1 * ir2);
    G = ir3 * (k.tg0 + k.tg1 * ir2);
  }
  if (ROT) {
    fw = k.rf1 * ir3;
    Gw = k.rg1 * ir3 * ir2;
  }
  if (CPL) c = k.rt0 * ir3;
  if (NEAR && r2 < R(4)) {  // overlapping pair (r < 2a), rare except the self pair
    const bool self = !(r2 > R(0));
    const R r = self ? R(0) : r2 * ir;
    const R irs = self ? R(0) : ir;
    if (TT) {
      f = k.t0 - k.tn1 * r;
      G = k.tn2 * irs;
    }
    if (ROT) {
      fw = k.r0 + r * (k.rn1 + k.rn3 * r * r);
      Gw = k.rn2 * irs + k.rn4 * r;
      if (self) Gw = R(0);
    }
    if (CPL) c = k.cn0 + k.cn1 * r;
  }
}

// ---------------------------------------------------------------------------
// Bottom wall image corrections (Swan & Brady 2007), scaled units.
// R = (Rx, Ry, Rz) image vector, iR = 1/|R|, hh = h/Rz (h_j for UF/WT/WF,
// h_i for UT).  All results are *added* into the outputs.
// ---------------------------------------------------------------------------

// C2: translational image, wallCorrection_UF :203-247
template <class R>
__device__ __forceinline__ void wall_uf_pair(R ex, R ey, R ez, R iR, R hh,
                                             const Vec3<R> &v, Vec3<R> &out) {
  const R iR2 = iR * iR;
  const R iR3 = iR2 * iR;
  const R iR5 = iR3 * iR2;
  const R ez2 = ez * ez;
  const R h1 = hh * (R(1) - hh);
  // A = -(3(1 + 2 h(1-h) ez2)/R + 2(1-3ez2)/R^3 - 2(1-5ez2)/R^5)/4
  const R A = R(-0.25) * (R(3) * (R(1) + R(2) * h1 * ez2) * iR +
                          R(2) * (R(1) - R(3) * ez2) * iR3 -
                          R(2) * (R(1) - R(5) * ez2) * iR5);
  // B = -(3(1 - 6 h(1-h) ez2)/R - 6(1-5ez2)/R^3 + 10(1-7ez2)/R^5)/4
  const R B = R(-0.25) * (R(3) * (R(1) - R(6) * h1 * ez2) * iR -
                          R(6) * (R(1) - R(5) * ez2) * iR3 +
                          R(10) * (R(1) - R(7) * ez2) * iR5);
  // C = ez (3h(1 - 6(1-h) ez2)/R - 6(1-5ez2)/R^3 + 10(2-7ez2)/R^5)/2
  const R C = R(0.5) * ez * (R(3) * hh * (R(1) - R(6) * (R(1) - hh) * ez2) * iR -
                             R(6) * (R(1) - R(5) * ez2) * iR3 +
                             R(10) * (R(2) - R(7) * ez2) * iR5);
  // D = ez (3h/R - 10/R^5)/2
  const R D = R(0.5) * ez * (R(3) * hh * iR - R(10) * iR5);
  // E = -(3 h^2 ez2/R + 3 ez2/R^3 + (2 - 15 ez2)/R^5)
  const R E = -(R(3) * hh * hh * ez2 * iR + R(3) * ez2 * iR3 + (R(2) - R(15) * ez2) * iR5);
  const R ev = ex * v.x + ey * v.y + ez * v.z;
  const R s = B * ev + C * v.z;  // coefficient of e
  out.x += A * v.x + s * ex;
  out.y += A * v.y + s * ey;
  out.z += A * v.z + s * ez + D * ev + E * v.z;
}

// C4: rotational image, wallCorrection_WT :262-280
template <class R>
__device__ __forceinline__ void wall_wt_pair(R ex, R ey, R ez, R iR,
                                             const Vec3<R> &v, Vec3<R> &out) {
  const R iR3 = iR * iR * iR;
  const R f1 = R(0.5) * (R(1) - R(6) * ez * ez) * iR3;
  const R f2 = R(-1.5) * iR3;
  const R f3 = R(3) * iR3 * ez;
  const R f4 = R(3) * iR3;
  const R ev = ex * v.x + ey * v.y + ez * v.z;
  const R pv = ex * v.y - ey * v.x;  // (z x e).v with z x e = (-ey, ex, 0)
  const R s = f2 * ev;
  out.x += f1 * v.x + s * ex - f4 * pv * ey;
  out.y += f1 * v.y + s * ey + f4 * pv * ex;
  out.z += f1 * v.z + s * ez + f3 * ev;
}

// C3 factors shared by WF (h = h_j) and UT (h = h_i), :296-307 / :333-345
template <class R>
__device__ __forceinline__ void wall_c3_factors(R ez, R iR, R hh, R &f1, R &f2,
                                                R &f3, R &f4) {
  const R iR2 = iR * iR;
  const R iR4 = iR2 * iR2;
  const R ez2 = ez * ez;
  f1 = iR2;
  f2 = R(2) * (R(6) * hh * ez2 * iR2 + (R(1) - R(10) * ez2) * iR4);
  f3 = R(-2) * ez * (R(3) * hh * iR2 - R(5) * iR4);
  f4 = R(-2) * ez * (hh * iR2 - iR4);
}

// C3 F:  f1 (e x F) + (f3 (e.F) + f2 F_z)(e x z) + f4 (z x F),  :347-356
template <class R>
__device__ __forceinline__ void wall_wf_pair(R ex, R ey, R ez, R iR, R hh,
                                             const Vec3<R> &v, Vec3<R> &out) {
  R f1, f2, f3, f4;
  wall_c3_factors(ez, iR, hh, f1, f2, f3, f4);
  const R ev = ex * v.x + ey * v.y + ez * v.z;
  const R g = f3 * ev + f2 * v.z;  // times e x z = (ey, -ex, 0)
  out.x += f1 * (ey * v.z - ez * v.y) + g * ey - f4 * v.y;
  out.y += f1 * (ez * v.x - ex * v.z) - g * ex + f4 * v.x;
  out.z += f1 * (ex * v.y - ey * v.x);
}

// C3^T T:  f1 (T x e) + ((e x z).T)(f3 e + f2 z) + f4 (T x z),  :309-316
// (e here is the unit vector of the UT image (-dx, -dy, h_i + h_j)).
template <class R>
__device__ __forceinline__ void wall_ut_pair(R ex, R ey, R ez, R iR, R hh,
                                             const Vec3<R> &v, Vec3<R> &out) {
  R f1, f2, f3, f4;
  wall_c3_factors(ez, iR, hh, f1, f2, f3, f4);
  const R q = ey * v.x - ex * v.y;  // (e x z).T
  out.x += f1 * (v.y * ez - v.z * ey) + q * f3 * ex + f4 * v.y;
  out.y += f1 * (v.z * ex - v.x * ez) + q * f3 * ey - f4 * v.x;
  out.z += f1 * (v.x * ey - v.y * ex) + q * (f3 * ez + f2);
}

// Self terms B1, B2, B3 (r == 0), :190-202, :256-261, :290-294, :327-331.
// ih = 1/h (scaled).  Adds the UF, WT, UT, WF self corrections.
template <class R>
__device__ __forceinline__ void wall_self_uf(R ih, const Vec3<R> &v, Vec3<R> &out) {
  const R ih3 = ih * ih * ih;
  const R ih5 = ih3 * ih * ih;
  const R cxy = R(-0.0625) * (R(9) * ih - R(2) * ih3 + ih5);
  const R cz = R(-0.125) * (R(9) * ih - R(4) * ih3 + ih5);
  out.x += cxy * v.x;
  out.y += cxy * v.y;
  out.z += cz * v.z;
}
template <class R>
__device__ __forceinline__ void wall_self_wt(R ih, const Vec3<R> &v, Vec3<R> &out) {
  const R ih3 = ih * ih * ih;
  out.x += R(-0.3125) * ih3 * v.x;
  out.y += R(-0.3125) * ih3 * v.y;
  out.z += R(-0.125) * ih3 * v.z;
}
// WF self: (h^-4/8) (z x F);  UT self: -(h^-4/8) (z x T)
template <class R>
__device__ __forceinline__ void wall_self_wf(R ih, const Vec3<R> &v, Vec3<R> &out) {
  const R c = R(0.125) * (ih * ih) * (ih * ih);
  out.x -= c * v.y;
  out.y += c * v.x;
}
template <class R>
__device__ __forceinline__ void wall_self_ut(R ih, const Vec3<R> &v, Vec3<R> &out) {
  const R c = R(0.125) * (ih * ih) * (ih * ih);
  out.x += c * v.y;
  out.y -= c * v.x;
}

// ---------------------------------------------------------------------------
// All four wall blocks (UF, UT, WT, WF) of one pair in one fused evaluation.
//
// Same tensors as the block-by-block functions above, rearranged so the RPY
// and image parts share work:
//   * R = (dx, dy, h_i + h_j) and d share dx^2 + dy^2;
//   * the isotropic RPY and image coefficients of F (f and A) and of T (fw and
//     f1 of C4) are summed before they multiply the source;
//   * the coupling c (F x d) and the f1 (e x F) term of C3 share their cross
//     products: with k1 = f1/|R| - c, k2 = f1 e_z - c d_z, k3 = f1 e_z + c d_z
//       W += (k1 dy Fz - k2 Fy,  k2 Fx - k1 dx Fz,  k1 (dx Fy - dy Fx))
//       U += (k3 Ty + k1 dy Tz, -k3 Tx - k1 dx Tz, -k1 (dy Tx - dx Ty))
//     (the UT image uses e' = (-ex, -ey, ez), hence the signs);
//   * the C3 factors are linear in h/Rz, f2 = a1 h + a0, f3 = b1 h + b0,
//     f4 = c1 h + c0, so the WF (h_j) and UT (h_i) images share a, b, c;
//   * (z x e).T serves both the C4 (WT) and the transposed C3 (UT) images;
//   * t0, r0, rt0 are folded into the polynomial constants.
// Sources carry b_j in F and T; the caller applies b_i to the sums.
// ---------------------------------------------------------------------------
struct WallConst {
  // UF image (times t0): A = iR (a10 + a11 h1q) + iR3 (a30 + a31 q) + iR5 (a50 + a51 q)
  float a10, a11, a30, a31, a50, a51;
  float b10, b11, b30, b31, b50, b51;
  // C = ez [iR (c1h hh + c11 h1q) + iR3 (c30 + c31 q) + iR5 (c50 + c51 q)]
  float c1h, c11, c30, c31, c50, c51;
  // D = ez (d1 hh iR + d5 iR5);  E = e1 q (hh^2 iR + iR3) + iR5 (e50 + e51 q)
  float d1, d5, e1, e50, e51;
  // WT image (times r0): f1 = iR3 (w0 + w1 q), f2 = w2 iR3, f4 = -2 f2, f3 = f4 ez
  float w0, w1, w2;
  // C3 (times rt0): f1 = g0 iR2; a1 = g1 q iR2, a0 = iR4 (g2 + g3 q);
  // b1 = g4 ez iR2, b0 = g5 ez iR4; c1 = g6 ez iR2, c0 = g7 ez iR4
  float g0, g1, g2, g3, g4, g5, g6, g7;
};

inline WallConst make_wall_const(double t0, double r0, double rt0) {
  WallConst w;
  w.a10 = float(-0.75 * t0); w.a11 = float(-1.5 * t0);
  w.a30 = float(-0.5 * t0);  w.a31 = float(1.5 * t0);
  w.a50 = float(0.5 * t0);   w.a51 = float(-2.5 * t0);
  w.b10 = float(-0.75 * t0); w.b11 = float(4.5 * t0);
  w.b30 = float(1.5 * t0);   w.b31 = float(-7.5 * t0);
  w.b50 = float(-2.5 * t0);  w.b51 = float(17.5 * t0);
  w.c1h = float(1.5 * t0);   w.c11 = float(-9.0 * t0);
  w.c30 = float(-3.0 * t0);  w.c31 = float(15.0 * t0);
  w.c50 = float(10.0 * t0);  w.c51 = float(-35.0 * t0);
  w.d1 = float(1.5 * t0);    w.d5 = float(-5.0 * t0);
  w.e1 = float(-3.0 * t0);   w.e50 = float(-2.0 * t0);  w.e51 = float(15.0 * t0);
  w.w0 = float(0.5 * r0);    w.w1 = float(-3.0 * r0);   w.w2 = float(-1.5 * r0);
  w.g0 = float(rt0);         w.g1 = float(12.0 * rt0);
  w.g2 = float(2.0 * rt0);   w.g3 = float(-20.0 * rt0);
  w.g4 = float(-6.0 * rt0);  w.g5 = float(10.0 * rt0);
  w.g6 = float(-2.0 * rt0);  w.g7 = float(2.0 * rt0);
  return w;
}

// Adds the UF+UT contribution to u and WT+WF to w for target (xi, yi, hi) and
// source p = (xj, yj, hj, .), F, T (scaled units, FP32).
__device__ __forceinline__ void wall_pair_fused(const PairConst<float> &k, const WallConst &K,
                                                float xi, float yi, float hi, float xj, float yj,
                                                float hj, float Fx, float Fy, float Fz, float Tx,
                                                float Ty, float Tz, Vec3<float> &u,
                                                Vec3<float> &w) {
  const float dx = xi - xj, dy = yi - yj, dz = hi - hj;
  const float sxy = fmaf(dx, dx, dy * dy);
  const float r2 = fmaf(dz, dz, sxy);
  const float Rz = hi + hj;
  if (r2 > 0.0f) {
    const float ir = rsqrtf(r2);
    float f, G, fw, Gw, c;
    rpy_coefficients<float, true, true, true>(k, r2, ir, f, G, fw, Gw, c);
    const float iR = rsqrtf(fmaf(Rz, Rz, sxy));
    const float ex = dx * iR, ey = dy * iR, ez = Rz * iR;
    const float iRz = __fdividef(1.0f, Rz);
    const float hhj = hj * iRz, hhi = hi * iRz;
    const float q = ez * ez;
    const float iR2 = iR * iR, iR3 = iR2 * iR, iR5 = iR3 * iR2, iR4 = iR2 * iR2;
    // ---- translational image C2 (UF), merged with the RPY UF block ----
    const float h1q = fmaf(-hhj, hhj, hhj) * q;
    const float A = fmaf(iR, fmaf(K.a11, h1q, K.a10),
                         fmaf(iR3, fmaf(K.a31, q, K.a30), iR5 * fmaf(K.a51, q, K.a50)));
    const float B = fmaf(iR, fmaf(K.b11, h1q, K.b10),
                         fmaf(iR3, fmaf(K.b31, q, K.b30), iR5 * fmaf(K.b51, q, K.b50)));
    const float C = ez * fmaf(iR, fmaf(K.c1h, hhj, K.c11 * h1q),
                              fmaf(iR3, fmaf(K.c31, q, K.c30), iR5 * fmaf(K.c51, q, K.c50)));
    const float D = ez * fmaf(K.d1 * hhj, iR, K.d5 * iR5);
    const float E = fmaf(K.e1 * q, fmaf(hhj * hhj, iR, iR3), iR5 * fmaf(K.e51, q, K.e50));
    const float ev = fmaf(ex, Fx, fmaf(ey, Fy, ez * Fz));
    const float dF = fmaf(dx, Fx, fmaf(dy, Fy, dz * Fz));
    const float fA = f + A;
    const float g = G * dF;
    const float s = fmaf(B, ev, C * Fz);
    u.x = fmaf(fA, Fx, fmaf(g, dx, fmaf(s, ex, u.x)));
    u.y = fmaf(fA, Fy, fmaf(g, dy, fmaf(s, ey, u.y)));
    u.z = fmaf(fA, Fz, fmaf(g, dz, fmaf(s, ez, fmaf(D, ev, fmaf(E, Fz, u.z)))));
    // ---- rotational image C4 (WT), merged with the RPY WT block ----
    const float evT = fmaf(ex, Tx, fmaf(ey, Ty, ez * Tz));
    const float dT = fmaf(dx, Tx, fmaf(dy, Ty, dz * Tz));
    const float pv = fmaf(ex, Ty, -ey * Tx);  // (z x e).T
    const float f2w = K.w2 * iR3;
    const float f4w = -2.0f * f2w;
    const float fwA = fmaf(iR3, fmaf(K.w1, q, K.w0), fw);
    const float gw = Gw * dT;
    const float sT = f2w * evT;
    const float m = f4w * pv;
    w.x = fmaf(fwA, Tx, fmaf(gw, dx, fmaf(sT, ex, fmaf(-m, ey, w.x))));
    w.y = fmaf(fwA, Ty, fmaf(gw, dy, fmaf(sT, ey, fmaf(m, ex, w.y))));
    w.z = fmaf(fwA, Tz, fmaf(gw, dz, fmaf(sT, ez, (f4w * ez) * evT + w.z)));
    // ---- couplings: RPY c(F x d), c(T x d) + C3 images (WF with h_j, UT with h_i) ----
    const float f1 = K.g0 * iR2;
    const float ga1 = (K.g1 * q) * iR2;
    const float ga0 = iR4 * fmaf(K.g3, q, K.g2);
    const float ezR2 = ez * iR2, ezR4 = ez * iR4;
    const float gb1 = K.g4 * ezR2, gb0 = K.g5 * ezR4;
    const float gc1 = K.g6 * ezR2, gc0 = K.g7 * ezR4;
    const float k1 = fmaf(f1, iR, -c);
    const float p = f1 * ez;
    const float k2 = fmaf(-c, dz, p);
    const float k3 = fmaf(c, dz, p);
    // WF image with h_j
    const float f2j = fmaf(ga1, hhj, ga0), f3j = fmaf(gb1, hhj, gb0), f4j = fmaf(gc1, hhj, gc0);
    const float gj = fmaf(f3j, ev, f2j * Fz);
    const float k1dx = k1 * dx, k1dy = k1 * dy;
    w.x = fmaf(k1dy, Fz, fmaf(-(k2 + f4j), Fy, fmaf(gj, ey, w.x)));
    w.y = fmaf(k2 + f4j, Fx, fmaf(-k1dx, Fz, fmaf(-gj, ex, w.y)));
    w.z = fmaf(k1, fmaf(dx, Fy, -dy * Fx), w.z);
    // UT image with h_i
    const float f2i = fmaf(ga1, hhi, ga0), f3i = fmaf(gb1, hhi, gb0), f4i = fmaf(gc1, hhi, gc0);
    const float mp = pv * f3i;
    u.x = fmaf(k3 + f4i, Ty, fmaf(k1dy, Tz, fmaf(-mp, ex, u.x)));
    u.y = fmaf(-(k3 + f4i), Tx, fmaf(-k1dx, Tz, fmaf(-mp, ey, u.y)));
    u.z = fmaf(-k1, fmaf(dy, Tx, -dx * Ty), fmaf(mp, ez, fmaf(pv, f2i, u.z)));
  } else {
    // self pair: RPY self mobilities and the wall self terms B1, B2, B3
    const float ih = __fdividef(1.0f, hj);
    const Vec3<float> F3 = {Fx, Fy, Fz}, T3 = {Tx, Ty, Tz};
    Vec3<float> cu = {0, 0, 0}, cw = {0, 0, 0}, ct = {0, 0, 0}, cf = {0, 0, 0};
    wall_self_uf<float>(ih, F3, cu);
    wall_self_wt<float>(ih, T3, cw);
    wall_self_wf<float>(ih, F3, cf);
    wall_self_ut<float>(ih, T3, ct);
    u.x += k.t0 * (Fx + cu.x) + k.rt0 * ct.x;
    u.y += k.t0 * (Fy + cu.y) + k.rt0 * ct.y;
    u.z += k.t0 * (Fz + cu.z) + k.rt0 * ct.z;
    w.x += k.r0 * (Tx + cw.x) + k.rt0 * cf.x;
    w.y += k.r0 * (Ty + cw.y) + k.rt0 * cf.y;
    w.z += k.r0 * (Tz + cw.z) + k.rt0 * cf.z;
  }
}

}  // namespace lmg
