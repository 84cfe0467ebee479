/*
 * Host stand-in for the five cuBLAS level-1/2 calls that the reference Lanczos
 * solver makes (include/lanczos/utils/device_blas.h:5-29), so that the
 * reference solver can be compiled and run on the CPU of this container as a
 * parity pin for the oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * Semantics follow the cuBLAS documentation for host pointer mode: results of
 * nrm2 and dot are written through a host pointer; vectors are plain arrays.
 * Accumulation is sequential in the vector's own precision.
 */
#pragma once
#include <cmath>
typedef int cublasStatus_t;
typedef struct lmg_fake_cublas *cublasHandle_t;
typedef enum { CUBLAS_OP_N = 0, CUBLAS_OP_T = 1 } cublasOperation_t;
#define CUBLAS_STATUS_SUCCESS 0
#define CUBLAS_STATUS_NOT_INITIALIZED 1
#define CUBLAS_STATUS_ALLOC_FAILED 3
#define CUBLAS_STATUS_INVALID_VALUE 7
#define CUBLAS_STATUS_ARCH_MISMATCH 8
#define CUBLAS_STATUS_MAPPING_ERROR 11
#define CUBLAS_STATUS_EXECUTION_FAILED 13
#define CUBLAS_STATUS_INTERNAL_ERROR 14
inline cublasStatus_t cublasCreate(cublasHandle_t *h) { *h = nullptr; return 0; }
inline cublasStatus_t cublasDestroy(cublasHandle_t) { return 0; }
template <class T>
inline cublasStatus_t lmg_nrm2(int n, const T *x, int incx, T *r) {
  T s = 0;
  for (int i = 0; i < n; i++) s += x[i * incx] * x[i * incx];
  *r = std::sqrt(s);
  return 0;
}
template <class T>
inline cublasStatus_t lmg_dot(int n, const T *x, int incx, const T *y, int incy, T *r) {
  T s = 0;
  for (int i = 0; i < n; i++) s += x[i * incx] * y[i * incy];
  *r = s;
  return 0;
}
template <class T>
inline cublasStatus_t lmg_axpy(int n, const T *a, const T *x, int incx, T *y, int incy) {
  for (int i = 0; i < n; i++) y[i * incy] += (*a) * x[i * incx];
  return 0;
}
template <class T> inline cublasStatus_t lmg_scal(int n, const T *a, T *x, int incx) {
  for (int i = 0; i < n; i++) x[i * incx] *= (*a);
  return 0;
}
/* y = alpha * A x + beta * y, A column-major m x n with leading dimension lda */
template <class T>
inline cublasStatus_t lmg_gemv(cublasOperation_t, int m, int n, const T *alpha,
                               const T *A, int lda, const T *x, int incx,
                               const T *beta, T *y, int incy) {
  for (int i = 0; i < m; i++) {
    T s = 0;
    for (int j = 0; j < n; j++) s += A[i + (long)j * lda] * x[j * incx];
    y[i * incy] = (*alpha) * s + ((*beta) == T(0) ? T(0) : (*beta) * y[i * incy]);
  }
  return 0;
}
#define LMG_FWD(name, impl)                                                    \
  template <class... A> inline cublasStatus_t name(cublasHandle_t, A... a) {   \
    return impl(a...);                                                         \
  }
LMG_FWD(cublasSnrm2, lmg_nrm2)
LMG_FWD(cublasDnrm2, lmg_nrm2)
LMG_FWD(cublasSdot, lmg_dot)
LMG_FWD(cublasDdot, lmg_dot)
LMG_FWD(cublasSaxpy, lmg_axpy)
LMG_FWD(cublasDaxpy, lmg_axpy)
LMG_FWD(cublasSscal, lmg_scal)
LMG_FWD(cublasDscal, lmg_scal)
LMG_FWD(cublasSgemv, lmg_gemv)
LMG_FWD(cublasDgemv, lmg_gemv)
