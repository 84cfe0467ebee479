// Learned sparse preconditioner for the Lanczos square root.
//
// Lanczos converges in fewer iterations on S = P M P^T when P approximates
// M^{-1/2}; the sample y = P^{-1} S^{1/2} z then has covariance
// P^{-1} S P^{-T} = M exactly, whatever P is (as long as it is nonsingular),
// so P only changes the cost, never the statistics.
//
// P here is sparse: row block i holds 3x3 blocks for particle i and its K = 16
// nearest neighbours, approximating row i of the inverse square root of the
// mobility of that 17-particle neighbourhood.  (A block-diagonal P cannot help
// the RPY mobility: its diagonal blocks of M^{-1/2} are nearly scalar; the
// neighbour blocks carry the gain.)  A small MLP produces the blocks:
//   input   the K neighbours' positions relative to i, sorted by distance, in a
//           canonical frame (x towards the nearest neighbour, y towards the
//           next non-collinear one), divided by a and normalised  -> 48 values
//   layers  48 -> 64 (tanh) -> 64 (tanh) -> 150 (linear)
//   output  normalised entries of the self block (6, symmetric) and of the K
//           neighbour blocks (9 each) in the canonical frame; rotated back to
//           the lab frame and scaled by t0^{-1/2}.
// The network is trained by this project's own GEMM / activation / loss /
// Adam kernels (below) on exact FP64 inverse square roots of small dense
// neighbourhood mobilities.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace lmg {

constexpr int kPrecK = 16;                  // neighbours per particle
constexpr int kPrecIn = 3 * kPrecK;         // 48 inputs
constexpr int kPrecHidden = 64;
constexpr int kPrecOut = 6 + 9 * kPrecK;    // 150 outputs
constexpr int kPrecBlocks = kPrecK + 1;     // blocks per row (self first)

// Network parameters and normalisation, FP32, in one contiguous array:
//   W1[48][64] b1[64] W2[64][64] b2[64] W3[64][150] b3[150]
//   xmean[48] xstd[48] ymean[150] ystd[150]
constexpr int kPrecW1 = 0;
constexpr int kPrecB1 = kPrecW1 + kPrecIn * kPrecHidden;
constexpr int kPrecW2 = kPrecB1 + kPrecHidden;
constexpr int kPrecB2 = kPrecW2 + kPrecHidden * kPrecHidden;
constexpr int kPrecW3 = kPrecB2 + kPrecHidden;
constexpr int kPrecB3 = kPrecW3 + kPrecHidden * kPrecOut;
constexpr int kPrecXm = kPrecB3 + kPrecOut;
constexpr int kPrecXs = kPrecXm + kPrecIn;
constexpr int kPrecYm = kPrecXs + kPrecIn;
constexpr int kPrecYs = kPrecYm + kPrecOut;
constexpr int kPrecParams = kPrecYs + kPrecOut;

// Launchers (precond.cu).  All pointers are device memory; all work goes on
// `stream`.
cudaError_t knn_launch(const float *pos, int N, int nper, int *nb, cudaStream_t stream);
cudaError_t precond_build_launch(const float *pos, const int *nb, int N, const float *params,
                                 float inv_a, float scale, float *blocks, cudaStream_t stream);
// out_i = sum_n B[i][n] x_{nb[i][n]}   (P x), 3 components per particle
cudaError_t precond_apply_launch(const float *blocks, const int *nb, int N, const float *x,
                                 float *out, cudaStream_t stream);
// out_{nb[i][n]} += B[i][n]^T x_i    (P^T x); out must be zeroed first
cudaError_t precond_apply_t_launch(const float *blocks, const int *nb, int N, const float *x,
                                   float *out, cudaStream_t stream);

}  // namespace lmg
