/* Maps the CBLAS gemv used by the reference Lanczos solver
 * (include/lanczos/LanczosAlgorithm.cu:80) to the copy of OpenBLAS that SciPy
 * ships, whose exports carry a scipy_ prefix.  TEST INFRASTRUCTURE ONLY. */
#pragma once
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112 };
extern "C" {
void scipy_cblas_sgemv(CBLAS_ORDER, CBLAS_TRANSPOSE, int, int, float,
                       const float *, int, const float *, int, float, float *, int);
void scipy_cblas_dgemv(CBLAS_ORDER, CBLAS_TRANSPOSE, int, int, double,
                       const double *, int, const double *, int, double, double *, int);
}
#define cblas_sgemv scipy_cblas_sgemv
#define cblas_dgemv scipy_cblas_dgemv
