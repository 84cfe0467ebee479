// Learned sparse preconditioner for the Lanczos square root.
//
// Lanczos converges in fewer iterations on S = P M P^T when P approximates
// M^{-1/2}; the sample y = P^{-1} S^{1/2} z then has covariance
// P^{-1} S P^{-T} = M exactly, whatever P is (as long as it is nonsingular),
// so P only changes the cost, never the statistics.
//
// P here is sparse: row block i holds 3x3 blocks for particle i and its K
// nearest neighbours (K = 16, 32 or 48, fixed by the network), approximating
// row i of the inverse square root of the mobility of that (K+1)-particle
// neighbourhood.  (A block-diagonal P cannot help
// the RPY mobility: its diagonal blocks of M^{-1/2} are nearly scalar; the
// neighbour blocks carry the gain.)  A small MLP produces the blocks:
//   input   the K neighbours' positions relative to i, sorted by distance, in a
//           canonical frame (x towards the nearest neighbour, y towards the
//           next non-collinear one), divided by a and normalised  -> 3K values
//   layers  3K -> 64 (tanh) -> 64 (tanh) -> 6 + 9K (linear)
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

// Network shape for K neighbours (K = 16, 32 or 48): parameters and
// normalisation, FP32, in one contiguous array:
//   W1[3K][64] b1[64] W2[64][64] b2[64] W3[64][6+9K] b3[6+9K]
//   xmean[3K] xstd[3K] ymean[6+9K] ystd[6+9K]
template <int K> struct PrecNet {
  static constexpr int Blocks = K + 1;  // blocks per row (self first)
  static constexpr int In = 3 * K;
  static constexpr int Hidden = 64;
  static constexpr int Out = 6 + 9 * K;
  static constexpr int W1 = 0;
  static constexpr int B1 = W1 + In * Hidden;
  static constexpr int W2 = B1 + Hidden;
  static constexpr int B2 = W2 + Hidden * Hidden;
  static constexpr int W3 = B2 + Hidden;
  static constexpr int B3 = W3 + Hidden * Out;
  static constexpr int Xm = B3 + Out;
  static constexpr int Xs = Xm + In;
  static constexpr int Ym = Xs + In;
  static constexpr int Ys = Ym + Out;
  static constexpr int Params = Ys + Out;
};

// The K whose network has n parameters, or 0.
inline int prec_k_for_params(size_t n) {
  if (n == (size_t)PrecNet<16>::Params) return 16;
  if (n == (size_t)PrecNet<32>::Params) return 32;
  if (n == (size_t)PrecNet<48>::Params) return 48;
  return 0;
}

// Launchers (precond.cu) for K = 16, 32 or 48.  All pointers are device
// memory; all work goes on `stream`.  nb holds K + 1 indices per particle
// (itself first, then the K nearest in distance order), blocks K + 1 3x3
// blocks per particle.
cudaError_t knn_launch(int K, const float *pos, int N, int nper, int *nb, cudaStream_t stream);
cudaError_t precond_build_launch(int K, const float *pos, const int *nb, int N,
                                 const float *params, float inv_a, float scale, float *blocks,
                                 cudaStream_t stream);
// out_i = sum_n B[i][n] x_{nb[i][n]}   (P x), 3 components per particle
cudaError_t precond_apply_launch(int K, const float *blocks, const int *nb, int N,
                                 const float *x, float *out, cudaStream_t stream);
// out_{nb[i][n]} += B[i][n]^T x_i    (P^T x); out must be zeroed first
cudaError_t precond_apply_t_launch(int K, const float *blocks, const int *nb, int N,
                                   const float *x, float *out, cudaStream_t stream);

}  // namespace lmg
