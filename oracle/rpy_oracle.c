/*
 * FP64 CPU oracle for the NBody Rotne-Prager-Yamakawa mobility product.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle for the CUDA path of
 * libmobility_gb300: only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py load it.  The product never links or calls it.
 *
 * It restates, in double precision and in plain C, the pair physics and the
 * batched all-pairs loop of libMobility's NBody solver:
 *
 *   open boundary RPY blocks     solvers/NBody/extra/hydrodynamicKernels.cuh:41-174
 *     RPY_UF                       :41-57     (translation-translation)
 *     RPY_WT                       :63-86     (rotation-rotation)
 *     RPY_UT / RPY_WF              :89-118    (translation-rotation couplings)
 *     OpenBoundary::dotProduct     :124-140
 *   single bottom wall           hydrodynamicKernels.cuh:182-442
 *     wallCorrection_UF (B1, C2)   :187-249
 *     wallCorrection_WT (B3, C4)   :253-282
 *     wallCorrection_UT (B2^T,C3^T):287-319
 *     wallCorrection_WF (B2, C3)   :324-359
 *     BottomWall::dotProduct       :362-390   (damping b_i b_j, z clamped at a)
 *     BottomWall::dotProduct_*     :392-441   (image vector r_ij + 2 h_j z)
 *   batched all-pairs loop       solvers/NBody/extra/NbodyRPY.cu:119-147
 *                                (every pair inside a batch, self pair included)
 *   block selection              NbodyRPY.cu:264-275
 *   wall shift and check         solvers/NBody/mobility.h:124-148
 *
 * The formulas are written out entry by entry, the way the reference writes
 * them, so that this file reads as a restatement that can be checked line by
 * line; the CUDA kernels use an independent vector form of the same tensors.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  double t0;  /* 1/(6 pi eta a)    trans-trans, mobility.h:101-102 */
  double r0;  /* 1/(8 pi eta a^3)  rot-rot,     mobility.h:105-106 */
  double rt0; /* 1/(8 pi eta a^2)  rot-trans,   mobility.h:103-104 */
  double a;   /* hydrodynamic radius */
  int wall;   /* 0: open boundary, 1: single bottom wall at z = 0 */
  int useUF, useUT, useWT, useWF;
} orc_params;

/* ---- open-boundary scalar functions (hydrodynamicKernels.cuh:41-118) ---- */

/* returns f and g/r^2 of the translational RPY tensor, :41-57 */
static void rpy_uf(double r, double a, double *f, double *gr2) {
  double x = r / a;
  if (x >= 2.0) {
    double ix = 1.0 / x;
    double ix2 = ix * ix;
    *f = (0.75 + 0.5 * ix2) * ix;
    *gr2 = (0.75 - 1.5 * ix2) * ix * ix2 / (a * a);
  } else {
    *f = 1.0 - 0.28125 * x;
    *gr2 = (x > 0.0) ? 0.09375 / (x * a * a) : 0.0;
  }
}

/* rotational RPY tensor normalised by 8 pi eta a^3, :63-86 */
static void rpy_wt(double r, double a, double *f, double *gr2) {
  double x = r / a;
  if (x >= 2.0) {
    double ix = 1.0 / x;
    double ix2 = ix * ix;
    double ix3 = ix * ix2;
    *f = -0.5 * ix3;
    *gr2 = 1.5 * ix2 * ix3 / (a * a);
  } else {
    *f = 1.0 - 0.84375 * x + 0.078125 * x * x * x;
    *gr2 = (x > 0.0) ? (0.28125 / x - 0.046875 * x) / (a * a) : 0.0;
  }
}

/* (M_xy, M_xz, M_yz) of the antisymmetric coupling tensor, :89-118 */
static void rpy_coupling(const double d[3], double r, double a, double m[3]) {
  double x = r / a;
  double s[3] = {d[0] / a, d[1] / a, d[2] / a};
  double c = (x >= 2.0) ? 1.0 / (x * x * x) : 0.5 * (1.0 - 0.375 * x);
  m[0] = c * s[2];
  m[1] = -c * s[1];
  m[2] = c * s[0];
}

/* applies the antisymmetric matrix [[0,mxy,mxz],[-mxy,0,myz],[-mxz,-myz,0]],
 * hydrodynamicKernels.cuh:161-173 */
static void apply_coupling(const double m[3], const double v[3], double out[3]) {
  out[0] = m[0] * v[1] + m[1] * v[2];
  out[1] = -m[0] * v[0] + m[2] * v[2];
  out[2] = -m[1] * v[0] - m[2] * v[1];
}

static void apply_isotropic(double f, double gr2, const double d[3], double r,
                            const double v[3], double out[3]) {
  double dv = d[0] * v[0] + d[1] * v[1] + d[2] * v[2];
  for (int k = 0; k < 3; k++)
    out[k] = f * v[k] + ((r > 0.0) ? gr2 * dv * d[k] : 0.0);
}

/* ---- wall corrections, R and h already divided by a (:187-359) ---- */

static void wall_uf(const double R[3], int self, double h, const double v[3],
                    double out[3]) {
  out[0] = out[1] = out[2] = 0.0;
  if (self) { /* B1, :190-202 */
    double iz = 1.0 / h, iz3 = iz * iz * iz, iz5 = iz3 * iz * iz;
    out[0] = -v[0] * (9.0 * iz - 2.0 * iz3 + iz5) / 16.0;
    out[1] = -v[1] * (9.0 * iz - 2.0 * iz3 + iz5) / 16.0;
    out[2] = -v[2] * (9.0 * iz - 4.0 * iz3 + iz5) / 8.0;
    return;
  }
  /* C2, :203-247 */
  double hh = h / R[2];
  double iR = 1.0 / sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  double e[3] = {R[0] * iR, R[1] * iR, R[2] * iR};
  double iR3 = iR * iR * iR, iR5 = iR3 * iR * iR;
  double ez2 = e[2] * e[2];
  double f1 = -(3.0 * (1.0 + 2.0 * hh * (1.0 - hh) * ez2) * iR +
                2.0 * (1.0 - 3.0 * ez2) * iR3 - 2.0 * (1.0 - 5.0 * ez2) * iR5) /
              4.0;
  double f2 = -(3.0 * (1.0 - 6.0 * hh * (1.0 - hh) * ez2) * iR -
                6.0 * (1.0 - 5.0 * ez2) * iR3 + 10.0 * (1.0 - 7.0 * ez2) * iR5) /
              4.0;
  double f3 = e[2] *
              (3.0 * hh * (1.0 - 6.0 * (1.0 - hh) * ez2) * iR -
               6.0 * (1.0 - 5.0 * ez2) * iR3 + 10.0 * (2.0 - 7.0 * ez2) * iR5) /
              2.0;
  double f4 = e[2] * (3.0 * hh * iR - 10.0 * iR5) / 2.0;
  double f5 = -(3.0 * hh * hh * ez2 * iR + 3.0 * ez2 * iR3 +
                (2.0 - 15.0 * ez2) * iR5);
  double M[3][3];
  M[0][0] = f1 + f2 * e[0] * e[0];
  M[0][1] = f2 * e[0] * e[1];
  M[0][2] = f2 * e[0] * e[2] + f3 * e[0];
  M[1][0] = f2 * e[1] * e[0];
  M[1][1] = f1 + f2 * e[1] * e[1];
  M[1][2] = f2 * e[1] * e[2] + f3 * e[1];
  M[2][0] = f2 * e[2] * e[0] + f4 * e[0];
  M[2][1] = f2 * e[2] * e[1] + f4 * e[1];
  M[2][2] = f1 + f2 * e[2] * e[2] + f3 * e[2] + f4 * e[2] + f5;
  for (int k = 0; k < 3; k++)
    out[k] = M[k][0] * v[0] + M[k][1] * v[1] + M[k][2] * v[2];
}

static void wall_wt(const double R[3], int self, double h, const double v[3],
                    double out[3]) {
  out[0] = out[1] = out[2] = 0.0;
  if (self) { /* B3, :256-261 */
    double iz = 1.0 / h, iz3 = iz * iz * iz;
    out[0] = -v[0] * iz3 * 0.3125;
    out[1] = -v[1] * iz3 * 0.3125;
    out[2] = -v[2] * iz3 * 0.125;
    return;
  }
  /* C4, :262-280 */
  double iR = 1.0 / sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  double iR3 = iR * iR * iR;
  double e[3] = {R[0] * iR, R[1] * iR, R[2] * iR};
  double f1 = (1.0 - 6.0 * e[2] * e[2]) * iR3 * 0.5;
  double f2 = -1.5 * iR3;
  double f3 = 3.0 * iR3 * e[2];
  double f4 = 3.0 * iR3;
  double M[3][3];
  M[0][0] = f1 + f2 * e[0] * e[0] + f4 * e[1] * e[1];
  M[0][1] = (f2 - f4) * e[0] * e[1];
  M[0][2] = f2 * e[0] * e[2];
  M[1][0] = (f2 - f4) * e[0] * e[1];
  M[1][1] = f1 + f2 * e[1] * e[1] + f4 * e[0] * e[0];
  M[1][2] = f2 * e[1] * e[2];
  M[2][0] = f2 * e[2] * e[0] + f3 * e[0];
  M[2][1] = f2 * e[2] * e[1] + f3 * e[1];
  M[2][2] = f1 + f2 * e[2] * e[2] + f3 * e[2];
  for (int k = 0; k < 3; k++)
    out[k] = M[k][0] * v[0] + M[k][1] * v[1] + M[k][2] * v[2];
}

/* C3 matrix entries shared by the two couplings (:296-307 and :333-345) */
static void wall_c3(const double R[3], double h, double M[3][3]) {
  double hh = h / R[2];
  double iR = 1.0 / sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  double iR2 = iR * iR, iR4 = iR2 * iR2;
  double e[3] = {R[0] * iR, R[1] * iR, R[2] * iR};
  double f1 = iR2;
  double f2 = (6.0 * hh * e[2] * e[2] * iR2 + (1.0 - 10.0 * e[2] * e[2]) * iR4) * 2.0;
  double f3 = -e[2] * (3.0 * hh * iR2 - 5.0 * iR4) * 2.0;
  double f4 = -e[2] * (hh * iR2 - iR4) * 2.0;
  /* C3 * f as written in wallCorrection_WF, :347-356 (note the minus signs) */
  M[0][0] = -(-f3 * e[0] * e[1]);
  M[0][1] = -(f1 * e[2] - f3 * e[1] * e[1] + f4);
  M[0][2] = -(-f1 * e[1] - f2 * e[1] - f3 * e[1] * e[2]);
  M[1][0] = -(-f1 * e[2] + f3 * e[0] * e[0] - f4);
  M[1][1] = -(f3 * e[0] * e[1]);
  M[1][2] = -(f1 * e[0] + f2 * e[0] + f3 * e[0] * e[2]);
  M[2][0] = -(f1 * e[1]);
  M[2][1] = -(-f1 * e[0]);
  M[2][2] = 0.0;
}

static void wall_wf(const double R[3], int self, double h, const double v[3],
                    double out[3]) {
  out[0] = out[1] = out[2] = 0.0;
  if (self) { /* B2, :327-331 */
    double iz = 1.0 / h, iz4 = iz * iz * iz * iz;
    out[0] = -iz4 * 0.125 * v[1];
    out[1] = iz4 * 0.125 * v[0];
    return;
  }
  double M[3][3];
  wall_c3(R, h, M);
  for (int k = 0; k < 3; k++)
    out[k] = M[k][0] * v[0] + M[k][1] * v[1] + M[k][2] * v[2];
}

/* UT is the transpose of C3 evaluated with R = -r_ij + 2 h_i z, :287-319 */
static void wall_ut(const double R[3], int self, double h, const double v[3],
                    double out[3]) {
  out[0] = out[1] = out[2] = 0.0;
  if (self) { /* B2^T, :290-294 */
    double iz = 1.0 / h, iz4 = iz * iz * iz * iz;
    out[0] = iz4 * 0.125 * v[1];
    out[1] = -iz4 * 0.125 * v[0];
    return;
  }
  double M[3][3];
  wall_c3(R, h, M);
  for (int k = 0; k < 3; k++)
    out[k] = M[0][k] * v[0] + M[1][k] * v[1] + M[2][k] * v[2];
}

/* Contribution of particle j (force fj, torque tj) to the velocities of
 * particle i, added into ui and wi.  Positions are in the wall frame (the
 * wall at z = 0).  OpenBoundary::dotProduct :124-140 and
 * BottomWall::dotProduct :362-441. */
void orc_pair(const orc_params *p, const double *ri, const double *rj,
              const double *fj, const double *tj, double *ui, double *wi) {
  const double a = p->a;
  double pi_[3] = {ri[0], ri[1], ri[2]};
  double pj_[3] = {rj[0], rj[1], rj[2]};
  double bij = 1.0;
  if (p->wall) {
    double bi = fmax(fmin(pi_[2] / a, 1.0), 0.0);
    double bj = fmax(fmin(pj_[2] / a, 1.0), 0.0);
    bij = bi * bj;
    pi_[2] = fmax(pi_[2], a);
    pj_[2] = fmax(pj_[2], a);
  }
  double d[3] = {pi_[0] - pj_[0], pi_[1] - pj_[1], pi_[2] - pj_[2]};
  double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  int self = (r == 0.0);
  double tmp[3], corr[3], f, g, m[3];
  if (p->useUF) {
    rpy_uf(r, a, &f, &g);
    apply_isotropic(f, g, d, r, fj, tmp);
    if (p->wall) {
      double R[3] = {d[0] / a, d[1] / a, (d[2] + 2.0 * pj_[2]) / a};
      wall_uf(R, self, pj_[2] / a, fj, corr);
      for (int k = 0; k < 3; k++) tmp[k] += corr[k];
    }
    for (int k = 0; k < 3; k++) ui[k] += bij * p->t0 * tmp[k];
  }
  if (p->useUT) {
    rpy_coupling(d, r, a, m);
    apply_coupling(m, tj, tmp);
    if (p->wall) {
      double R[3] = {-d[0] / a, -d[1] / a, (-d[2] + 2.0 * pi_[2]) / a};
      wall_ut(R, self, pi_[2] / a, tj, corr);
      for (int k = 0; k < 3; k++) tmp[k] += corr[k];
    }
    for (int k = 0; k < 3; k++) ui[k] += bij * p->rt0 * tmp[k];
  }
  if (p->useWT) {
    rpy_wt(r, a, &f, &g);
    apply_isotropic(f, g, d, r, tj, tmp);
    if (p->wall) {
      double R[3] = {d[0] / a, d[1] / a, (d[2] + 2.0 * pj_[2]) / a};
      wall_wt(R, self, pj_[2] / a, tj, corr);
      for (int k = 0; k < 3; k++) tmp[k] += corr[k];
    }
    for (int k = 0; k < 3; k++) wi[k] += bij * p->r0 * tmp[k];
  }
  if (p->useWF) {
    rpy_coupling(d, r, a, m);
    apply_coupling(m, fj, tmp);
    if (p->wall) {
      double R[3] = {d[0] / a, d[1] / a, (d[2] + 2.0 * pj_[2]) / a};
      wall_wf(R, self, pj_[2] / a, fj, corr);
      for (int k = 0; k < 3; k++) tmp[k] += corr[k];
    }
    for (int k = 0; k < 3; k++) wi[k] += bij * p->rt0 * tmp[k];
  }
}

/* ---- batched all-pairs product, NbodyRPY.cu:119-147 ---- */

typedef struct {
  const orc_params *p;
  const double *pos, *F, *T;
  double *U, *W;
  int64_t NperBatch, row_begin, row_end;
  int64_t N;
  int nthreads, tid;
} orc_job;

static void *orc_rows(void *arg) {
  orc_job *j = (orc_job *)arg;
  const double zero3[3] = {0.0, 0.0, 0.0};
  for (int64_t i = j->row_begin + j->tid; i < j->row_end; i += j->nthreads) {
    double u[3] = {0, 0, 0}, w[3] = {0, 0, 0};
    int64_t b0 = (i / j->NperBatch) * j->NperBatch;
    int64_t b1 = b0 + j->NperBatch;
    if (b1 > j->N) b1 = j->N;
    for (int64_t k = b0; k < b1; k++) {
      orc_pair(j->p, j->pos + 3 * i, j->pos + 3 * k,
               j->F ? j->F + 3 * k : zero3, j->T ? j->T + 3 * k : zero3, u, w);
    }
    int64_t o = i - j->row_begin;
    if (j->U)
      for (int c = 0; c < 3; c++) j->U[3 * o + c] = u[c];
    if (j->W)
      for (int c = 0; c < 3; c++) j->W[3 * o + c] = w[c];
  }
  return NULL;
}

/* U, W receive rows [row_begin, row_end) (3 values per row).  Pass NULL for an
 * absent input or output.  Returns 0 on success. */
int orc_mdot(const orc_params *p, const double *pos, const double *F,
             const double *T, double *U, double *W, int64_t N,
             int64_t NperBatch, int64_t row_begin, int64_t row_end,
             int nthreads) {
  if (N <= 0 || NperBatch <= 0 || row_begin < 0 || row_end > N ||
      row_begin > row_end)
    return 1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  orc_job jobs[256];
  for (int t = 0; t < nthreads; t++) {
    orc_job j = {p, pos, F, T, U, W, NperBatch, row_begin, row_end, N,
                 nthreads, t};
    jobs[t] = j;
  }
  if (nthreads == 1) {
    orc_rows(&jobs[0]);
    return 0;
  }
  for (int t = 0; t < nthreads; t++)
    pthread_create(&th[t], NULL, orc_rows, &jobs[t]);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  return 0;
}

/* Dense grand mobility matrix in the reference layout: rows [U; W], columns
 * [F; T] (tests/utils.py compute_M), of size (k*3N)^2 with k = 1 (UF only) or
 * 2 (all four blocks).  Row-major.  Pairs in different batches are zero. */
int orc_dense(const orc_params *p, const double *pos, int64_t N,
              int64_t NperBatch, int angular, double *M) {
  if (N <= 0 || NperBatch <= 0) return 1;
  int64_t n = (angular ? 6 : 3) * N;
  memset(M, 0, sizeof(double) * n * n);
  orc_params q = *p;
  for (int64_t i = 0; i < N; i++) {
    int64_t b0 = (i / NperBatch) * NperBatch, b1 = b0 + NperBatch;
    if (b1 > N) b1 = N;
    for (int64_t j = b0; j < b1; j++) {
      for (int c = 0; c < 3; c++) {
        double e[3] = {0, 0, 0};
        e[c] = 1.0;
        double u[3] = {0, 0, 0}, w[3] = {0, 0, 0};
        const double zero3[3] = {0, 0, 0};
        /* column for force component c of particle j */
        q.useUF = 1;
        q.useWF = angular;
        q.useUT = 0;
        q.useWT = 0;
        orc_pair(&q, pos + 3 * i, pos + 3 * j, e, zero3, u, w);
        for (int k = 0; k < 3; k++) {
          M[(3 * i + k) * n + 3 * j + c] = u[k];
          if (angular) M[(3 * N + 3 * i + k) * n + 3 * j + c] = w[k];
        }
        if (angular) { /* column for torque component c of particle j */
          double u2[3] = {0, 0, 0}, w2[3] = {0, 0, 0};
          q.useUF = 0;
          q.useWF = 0;
          q.useUT = 1;
          q.useWT = 1;
          orc_pair(&q, pos + 3 * i, pos + 3 * j, zero3, e, u2, w2);
          for (int k = 0; k < 3; k++) {
            M[(3 * i + k) * n + 3 * N + 3 * j + c] = u2[k];
            M[(3 * N + 3 * i + k) * n + 3 * N + 3 * j + c] = w2[k];
          }
        }
      }
    }
  }
  return 0;
}
