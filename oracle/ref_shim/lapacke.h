/* Maps LAPACKE ?steqr used by the reference Lanczos solver
 * (include/lanczos/LanczosAlgorithm.cu:59) to SciPy's bundled OpenBLAS
 * (scipy_ prefixed exports, 32-bit integers).  TEST INFRASTRUCTURE ONLY. */
#pragma once
#define LAPACK_COL_MAJOR 102
extern "C" {
int scipy_LAPACKE_ssteqr(int, char, int, float *, float *, float *, int);
int scipy_LAPACKE_dsteqr(int, char, int, double *, double *, double *, int);
}
#define LAPACKE_ssteqr scipy_LAPACKE_ssteqr
#define LAPACKE_dsteqr scipy_LAPACKE_dsteqr
