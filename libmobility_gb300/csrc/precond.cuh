// Learned sparse preconditioner for the Lanczos square root.
//
// Lanczos converges in fewer iterations on S = P M P^T when P approximates
// M^{-1/2}; the sample y = P^{-1} S^{1/2} z then has covariance
// P^{-1} S P^{-T} = M exactly, whatever P is (as long as it is nonsingular),
// so P only changes the cost, never the statistics.
//
// P here is sparse: row block i holds 3x3 blocks for particle i and its K
// nearest neighbours (K = 16, 32, 48 or 64, fixed by the network), approximating
// row i of the inverse square root of the mobility of that (K+1)-particle
// neighbourhood.  (A block-diagonal P cannot help
// the RPY mobility: its diagonal blocks of M^{-1/2} are nearly scalar; the
// neighbour blocks carry the gain.)  A small MLP produces the blocks:
//   input   the K neighbours' positions relative to i, sorted by distance, in a
//           canonical frame (x towards the nearest neighbour, y towards the
//           next non-collinear one), divided by a and normalised  -> 3K values
//   (wall networks, for a single bottom wall: the frame turns about the wall
//   normal only -- x towards the horizontal offset of the nearest neighbour
//   that has one, z the wall normal -- and the particle's height max(h, a)/a
//   is one more input, 3K + 1 values)
//   layers  3K (+1) -> H (tanh) -> H (tanh) -> 6 + 9K (linear)
//   output  normalised entries of the self block (6, symmetric) and of the K
//           neighbour blocks (9 each) in the canonical frame; rotated back to
//           the lab frame and scaled by t0^{-1/2}.
// The network is trained by this project's own GEMM / activation / loss /
// Adam kernels (below) on exact FP64 inverse square roots of small dense
// neighbourhood mobilities.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.hpp"

namespace lmg {

// Network shape for K neighbours (16, 32, 48 or 64) and hidden width H (64, 128,
// 256, 512 or 1024), In = 3K inputs (3K + 1 for a wall network): parameters
// and normalisation, FP32, in one contiguous array:
//   W1[In][H] b1[H] W2[H][H] b2[H] W3[H][6+9K] b3[6+9K]
//   xmean[In] xstd[In] ymean[6+9K] ystd[6+9K]
// Every (K, H, wall) has a different parameter count, which identifies it.
struct PrecLayout {
  int K = 0, H = 0, In = 0, Out = 0;
  bool wall = false;  // trained on a bottom wall: frame about z, height input
  int W1 = 0, B1 = 0, W2 = 0, B2 = 0, W3 = 0, B3 = 0, Xm = 0, Xs = 0, Ym = 0, Ys = 0;
  int Params = 0;
};

inline PrecLayout prec_layout(int K, int H, bool wall = false) {
  PrecLayout L;
  L.K = K;
  L.H = H;
  L.wall = wall;
  L.In = 3 * K + (wall ? 1 : 0);
  L.Out = 6 + 9 * K;
  L.W1 = 0;
  L.B1 = L.W1 + L.In * H;
  L.W2 = L.B1 + H;
  L.B2 = L.W2 + H * H;
  L.W3 = L.B2 + H;
  L.B3 = L.W3 + H * L.Out;
  L.Xm = L.B3 + L.Out;
  L.Xs = L.Xm + L.In;
  L.Ym = L.Xs + L.In;
  L.Ys = L.Ym + L.Out;
  L.Params = L.Ys + L.Out;
  return L;
}

// The layout whose parameter count is n (K = 0 if there is none).
inline PrecLayout prec_layout_for_params(size_t n) {
  for (bool wall : {false, true})
    for (int K : {16, 32, 48, 64})
      for (int H : {64, 128, 256, 512, 1024}) {
        const PrecLayout L = prec_layout(K, H, wall);
        if ((size_t)L.Params == n) return L;
      }
  return PrecLayout{};
}

// Launchers (precond.cu) for K = 16, 32, 48 or 64.  All pointers are device
// memory; all work goes on `stream`.  Layouts, stored so that consecutive
// particles are consecutive in memory: nb[n][i] (n = 0 the particle itself,
// then its K nearest in distance order), blocks[n][e][i] (element e = 3 r + c
// of block n of row i).
//
// Work arrays of the grid search, kept by the caller between calls (the
// launcher allocates them when they are too small; it reads the bounding box
// back, so it synchronises `stream` once).
struct KnnScratch {
  DeviceBuffer<unsigned> box;
  PinnedBuffer<unsigned> hbox;
  DeviceBuffer<int> key, cnt, start, sidx;
  DeviceBuffer<float4> spos;
};
cudaError_t knn_launch(int K, const float *pos, int N, int nper, int *nb, cudaStream_t stream,
                       KnnScratch *scratch);
// Work arrays of the build: features X [N][3K], frames E [N][9], hidden
// activations H1, H2 [N][H], network outputs Y [N][6+9K].
struct PrecWork {
  DeviceBuffer<float> X, E, H1, H2, Y;
  DeviceBuffer<float> WT;  // weights transposed for the tensor-core layers
};
// P blocks from positions and neighbour lists: features and canonical frames
// (one thread per particle), the three layers as GEMMs of all particles at
// once (bias and tanh fused: the tcgen05 TF32 kernel of tc_gemm.cu where the
// GPU has it and it is switched on, else this library's CUDA-core GEMM),
// then the blocks rotated back to the lab frame and scaled.
cudaError_t precond_build_launch(const PrecLayout &L, const float *pos, const int *nb, int N,
                                 const float *params, float inv_a, float scale, void *blocks,
                                 bool half, PrecWork *work, cudaStream_t stream);
// Blocks are float, or half when `half` (then stored at unit scale and the
// products multiply by `scale`; a float build applies its scale itself and
// the products get 1).
// out_i = scale sum_n B[n][i] x_{nb[n][i]}   (P x), 3 components per particle
cudaError_t precond_apply_launch(int K, const void *blocks, bool half, float scale,
                                 const int *nb, int N, const float *x, float *out,
                                 cudaStream_t stream);
// out_j = scale sum_{(n,i): nb[n][i] = j} B[n][i]^T x_i    (P^T x), through
// the work array pad[N] (float4, 16-byte aligned), which it zeroes first
cudaError_t precond_apply_t_launch(int K, const void *blocks, bool half, float scale,
                                   const int *nb, int N, const float *x, float *out,
                                   float4 *pad, cudaStream_t stream);

}  // namespace lmg
