// Tensor-core GEMM for the preconditioner network (sm_103a: tcgen05 + TMA).
//
//   C[M x N] = act(A[M x K] . Bt[N x K]^T + bias)
//
// A and Bt are FP32, row-major with K contiguous (Bt is the weight matrix
// transposed once on the host side of the caller), taken as TF32 by the
// tensor cores (10-bit mantissa, FP32 accumulation in tensor memory); C is
// FP32.  act: 0 none, 1 tanh.  Requirements (checked, cudaErrorInvalidValue
// otherwise): A, Bt 16-byte aligned, lda and ldbt multiples of 4, K >= 1.
#pragma once
#include <cuda_runtime.h>

namespace lmg {

cudaError_t tc_gemm_launch(int M, int N, int K, const float *A, int lda, const float *Bt,
                           int ldbt, float *C, int ldc, const float *bias, int act,
                           cudaStream_t stream);

// Whether this GPU runs the tcgen05 kernel (compute capability 10.x); the
// callers keep their CUDA-core path otherwise.
bool tc_gemm_available();

// Device word that a tcgen05 GEMM launch sets to a non-zero code when one of
// its bounded waits runs out (0: none since the last reset).
int tc_gemm_status(bool reset);

}  // namespace lmg
