// Kernels of the learned sparse preconditioner (see precond.cuh) and of its
// training: k-nearest neighbours, feature/MLP/rotation build of P, sparse P
// and P^T products, and the dense GEMM / activation / loss / Adam kernels the
// training loop is made of.
#include <cfloat>
#include <cstdint>

#include "launch_count.hpp"
#include "precond.cuh"

namespace lmg {

// ---------------------------------------------------------------------------
// k nearest neighbours within each batch (self first), brute force through
// shared-memory tiles: O(N * batch) distance tests, ~1 ms at N = 65536.
// ---------------------------------------------------------------------------
constexpr int kKnnThreads = 128;

template <int KB>
__global__ void __launch_bounds__(kKnnThreads)
knn_kernel(const float *__restrict__ pos, int N, int nper, int *__restrict__ nb) {
  __shared__ float sx[kKnnThreads], sy[kKnnThreads], sz[kKnnThreads];
  const int i = blockIdx.x * kKnnThreads + threadIdx.x;
  const int ic = i < N ? i : N - 1;
  const float xi = pos[3 * ic], yi = pos[3 * ic + 1], zi = pos[3 * ic + 2];
  const int b0 = (ic / nper) * nper;
  const int b1 = min(N, b0 + nper);
  const int first = blockIdx.x * kKnnThreads;
  const int last = min(N, first + kKnnThreads) - 1;
  const int s0 = (first / nper) * nper;
  const int s1 = min(N, (last / nper + 1) * nper);
  float bd[KB];
  int bj[KB];
#pragma unroll
  for (int q = 0; q < KB; q++) {
    bd[q] = FLT_MAX;
    bj[q] = ic;
  }
  for (int ts = s0; ts < s1; ts += kKnnThreads) {
    const int j = ts + threadIdx.x;
    if (j < s1) {
      sx[threadIdx.x] = pos[3 * j];
      sy[threadIdx.x] = pos[3 * j + 1];
      sz[threadIdx.x] = pos[3 * j + 2];
    }
    __syncthreads();
    const int nh = min(kKnnThreads, s1 - ts);
    for (int jj = 0; jj < nh; jj++) {
      const int j2 = ts + jj;
      const float dx = sx[jj] - xi, dy = sy[jj] - yi, dz = sz[jj] - zi;
      const float d = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      if (d < bd[KB - 1] && j2 >= b0 && j2 < b1) {
        // insertion into the sorted list, unrolled so it stays in registers;
        // the particle itself (d = 0) lands in slot 0
        float cd = (j2 == ic) ? -1.0f : d;
        int cj = j2;
        bool placed = false;
#pragma unroll
        for (int q = KB - 1; q >= 1; q--) {
          if (!placed) {
            if (bd[q - 1] > cd) {
              bd[q] = bd[q - 1];
              bj[q] = bj[q - 1];
            } else {
              bd[q] = cd;
              bj[q] = cj;
              placed = true;
            }
          }
        }
        if (!placed) {
          bd[0] = cd;
          bj[0] = cj;
        }
      }
    }
    __syncthreads();
  }
  if (i < N) {
#pragma unroll
    for (int q = 0; q < KB; q++) nb[(size_t)i * KB + q] = bj[q];
  }
}

cudaError_t knn_launch(int K, const float *pos, int N, int nper, int *nb, cudaStream_t stream) {
  const int blocks = (N + kKnnThreads - 1) / kKnnThreads;
  if (K != 16 && K != 32 && K != 48) return cudaErrorInvalidValue;
  count_launch();
  if (K == 16) knn_kernel<17><<<blocks, kKnnThreads, 0, stream>>>(pos, N, nper, nb);
  if (K == 32) knn_kernel<33><<<blocks, kKnnThreads, 0, stream>>>(pos, N, nper, nb);
  if (K == 48) knn_kernel<49><<<blocks, kKnnThreads, 0, stream>>>(pos, N, nper, nb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// P rows: canonical frame, features, MLP, rotation back to the lab frame.
// One thread per particle; the network parameters sit in shared memory and
// are read by broadcast; activations stay in registers (fully unrolled).
// ---------------------------------------------------------------------------
constexpr int kBuildThreads = 128;

template <int K>
__global__ void __launch_bounds__(kBuildThreads)
precond_build_kernel(const float *__restrict__ pos, const int *__restrict__ nb, int N,
                     const float *__restrict__ params, float inv_a, float scale,
                     float *__restrict__ blocks) {
  using S = PrecNet<K>;
  constexpr int kPrecK = K, KB_ = S::Blocks, kPrecIn = S::In, kPrecHidden = S::Hidden,
                kPrecOut = S::Out, kPrecParams = S::Params, kPrecW1 = S::W1, kPrecB1 = S::B1,
                kPrecW2 = S::W2, kPrecB2 = S::B2, kPrecW3 = S::W3, kPrecB3 = S::B3,
                kPrecXm = S::Xm, kPrecXs = S::Xs, kPrecYm = S::Ym, kPrecYs = S::Ys;
  extern __shared__ float sw[];
  for (int t = threadIdx.x; t < kPrecParams; t += kBuildThreads) sw[t] = params[t];
  __syncthreads();
  const int i = blockIdx.x * kBuildThreads + threadIdx.x;
  if (i >= N) return;
  const int *nbi = nb + (size_t)i * KB_;
  const float xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
  float rel[kPrecK][3];
#pragma unroll
  for (int n = 0; n < kPrecK; n++) {
    const int j = nbi[n + 1];
    rel[n][0] = (pos[3 * j] - xi) * inv_a;
    rel[n][1] = (pos[3 * j + 1] - yi) * inv_a;
    rel[n][2] = (pos[3 * j + 2] - zi) * inv_a;
  }
  // canonical frame: x to the nearest neighbour, y to the first neighbour
  // that is not collinear with it, z = x cross y
  float e[3][3];
  {
    const float l = rsqrtf(fmaxf(rel[0][0] * rel[0][0] + rel[0][1] * rel[0][1] +
                                 rel[0][2] * rel[0][2], 1e-30f));
    e[0][0] = rel[0][0] * l;
    e[0][1] = rel[0][1] * l;
    e[0][2] = rel[0][2] * l;
    float y0 = 0.f, y1 = 1.f, y2 = 0.f;
    bool found = false;
#pragma unroll
    for (int n = 1; n < kPrecK; n++) {
      if (!found) {
        const float p = rel[n][0] * e[0][0] + rel[n][1] * e[0][1] + rel[n][2] * e[0][2];
        const float a0 = rel[n][0] - p * e[0][0], a1 = rel[n][1] - p * e[0][1],
                    a2 = rel[n][2] - p * e[0][2];
        const float nn = a0 * a0 + a1 * a1 + a2 * a2;
        if (nn > 1e-12f) {
          const float li = rsqrtf(nn);
          y0 = a0 * li;
          y1 = a1 * li;
          y2 = a2 * li;
          found = true;
        }
      }
    }
    e[1][0] = y0;
    e[1][1] = y1;
    e[1][2] = y2;
    e[2][0] = e[0][1] * y2 - e[0][2] * y1;
    e[2][1] = e[0][2] * y0 - e[0][0] * y2;
    e[2][2] = e[0][0] * y1 - e[0][1] * y0;
  }
  float x[kPrecIn];
#pragma unroll
  for (int n = 0; n < kPrecK; n++) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float v = rel[n][0] * e[c][0] + rel[n][1] * e[c][1] + rel[n][2] * e[c][2];
      x[3 * n + c] = (v - sw[kPrecXm + 3 * n + c]) / sw[kPrecXs + 3 * n + c];
    }
  }
  float h1[kPrecHidden];
#pragma unroll
  for (int j = 0; j < kPrecHidden; j++) {
    float acc = sw[kPrecB1 + j];
#pragma unroll
    for (int k = 0; k < kPrecIn; k++) acc = fmaf(x[k], sw[kPrecW1 + k * kPrecHidden + j], acc);
    h1[j] = tanhf(acc);
  }
  float h2[kPrecHidden];
#pragma unroll
  for (int j = 0; j < kPrecHidden; j++) {
    float acc = sw[kPrecB2 + j];
#pragma unroll
    for (int k = 0; k < kPrecHidden; k++)
      acc = fmaf(h1[k], sw[kPrecW2 + k * kPrecHidden + j], acc);
    h2[j] = tanhf(acc);
  }
  float *out = blocks + (size_t)i * KB_ * 9;
  // output unit o, de-normalised
  auto unit = [&](int o) {
    float acc = sw[kPrecB3 + o];
#pragma unroll
    for (int k = 0; k < kPrecHidden; k++) acc = fmaf(h2[k], sw[kPrecW3 + k * kPrecOut + o], acc);
    return acc * sw[kPrecYs + o] + sw[kPrecYm + o];
  };
#pragma unroll 1
  for (int n = 0; n < KB_; n++) {
    float b[3][3];
    if (n == 0) {  // symmetric self block from 6 units: 00 01 02 11 12 22
      const float u0 = unit(0), u1 = unit(1), u2 = unit(2), u3 = unit(3), u4 = unit(4),
                  u5 = unit(5);
      b[0][0] = u0; b[0][1] = u1; b[0][2] = u2;
      b[1][0] = u1; b[1][1] = u3; b[1][2] = u4;
      b[2][0] = u2; b[2][1] = u4; b[2][2] = u5;
    } else {
      const int o = 6 + 9 * (n - 1);
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) b[r][c] = unit(o + 3 * r + c);
    }
    // lab block = E^T b E  (E rows are the canonical axes)
#pragma unroll
    for (int r = 0; r < 3; r++) {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        float acc = 0.f;
#pragma unroll
        for (int p = 0; p < 3; p++) {
          const float t = b[p][0] * e[0][c] + b[p][1] * e[1][c] + b[p][2] * e[2][c];
          acc = fmaf(e[p][r], t, acc);
        }
        out[9 * n + 3 * r + c] = acc * scale;
      }
    }
  }
}

template <int K>
cudaError_t precond_build_k(const float *pos, const int *nb, int N, const float *params,
                            float inv_a, float scale, float *blocks, cudaStream_t stream) {
  const size_t smem = PrecNet<K>::Params * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(precond_build_kernel<K>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int nblk = (N + kBuildThreads - 1) / kBuildThreads;
  count_launch();
  precond_build_kernel<K><<<nblk, kBuildThreads, smem, stream>>>(pos, nb, N, params, inv_a,
                                                                 scale, blocks);
  return cudaGetLastError();
}

cudaError_t precond_build_launch(int K, const float *pos, const int *nb, int N,
                                 const float *params, float inv_a, float scale, float *blocks,
                                 cudaStream_t stream) {
  if (K == 16) return precond_build_k<16>(pos, nb, N, params, inv_a, scale, blocks, stream);
  if (K == 32) return precond_build_k<32>(pos, nb, N, params, inv_a, scale, blocks, stream);
  if (K == 48) return precond_build_k<48>(pos, nb, N, params, inv_a, scale, blocks, stream);
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Sparse products with P (rows of K+1 3x3 blocks)
// ---------------------------------------------------------------------------
template <int KB>
__global__ void precond_apply_kernel(const float *__restrict__ B, const int *__restrict__ nb,
                                     int N, const float *__restrict__ x, float *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const float *b = B + (size_t)i * KB * 9;
  const int *nbi = nb + (size_t)i * KB;
  float o0 = 0.f, o1 = 0.f, o2 = 0.f;
#pragma unroll
  for (int n = 0; n < KB; n++) {
    const int j = nbi[n];
    const float v0 = x[3 * j], v1 = x[3 * j + 1], v2 = x[3 * j + 2];
    o0 = fmaf(b[9 * n + 0], v0, fmaf(b[9 * n + 1], v1, fmaf(b[9 * n + 2], v2, o0)));
    o1 = fmaf(b[9 * n + 3], v0, fmaf(b[9 * n + 4], v1, fmaf(b[9 * n + 5], v2, o1)));
    o2 = fmaf(b[9 * n + 6], v0, fmaf(b[9 * n + 7], v1, fmaf(b[9 * n + 8], v2, o2)));
  }
  out[3 * i] = o0;
  out[3 * i + 1] = o1;
  out[3 * i + 2] = o2;
}

template <int KB>
__global__ void precond_apply_t_kernel(const float *__restrict__ B, const int *__restrict__ nb,
                                       int N, const float *__restrict__ x, float *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const float *b = B + (size_t)i * KB * 9;
  const int *nbi = nb + (size_t)i * KB;
  const float v0 = x[3 * i], v1 = x[3 * i + 1], v2 = x[3 * i + 2];
#pragma unroll
  for (int n = 0; n < KB; n++) {
    const int j = nbi[n];
    atomicAdd(out + 3 * j, b[9 * n + 0] * v0 + b[9 * n + 3] * v1 + b[9 * n + 6] * v2);
    atomicAdd(out + 3 * j + 1, b[9 * n + 1] * v0 + b[9 * n + 4] * v1 + b[9 * n + 7] * v2);
    atomicAdd(out + 3 * j + 2, b[9 * n + 2] * v0 + b[9 * n + 5] * v1 + b[9 * n + 8] * v2);
  }
}

cudaError_t precond_apply_launch(int K, const float *blocks, const int *nb, int N,
                                 const float *x, float *out, cudaStream_t stream) {
  const int g = (N + 255) / 256;
  if (K != 16 && K != 32 && K != 48) return cudaErrorInvalidValue;
  count_launch();
  if (K == 16) precond_apply_kernel<17><<<g, 256, 0, stream>>>(blocks, nb, N, x, out);
  if (K == 32) precond_apply_kernel<33><<<g, 256, 0, stream>>>(blocks, nb, N, x, out);
  if (K == 48) precond_apply_kernel<49><<<g, 256, 0, stream>>>(blocks, nb, N, x, out);
  return cudaGetLastError();
}

cudaError_t precond_apply_t_launch(int K, const float *blocks, const int *nb, int N,
                                   const float *x, float *out, cudaStream_t stream) {
  const int g = (N + 255) / 256;
  if (K != 16 && K != 32 && K != 48) return cudaErrorInvalidValue;
  count_launch();
  if (K == 16) precond_apply_t_kernel<17><<<g, 256, 0, stream>>>(blocks, nb, N, x, out);
  if (K == 32) precond_apply_t_kernel<33><<<g, 256, 0, stream>>>(blocks, nb, N, x, out);
  if (K == 48) precond_apply_t_kernel<49><<<g, 256, 0, stream>>>(blocks, nb, N, x, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Training kernels
// ---------------------------------------------------------------------------
// C[M x N] = op(A)[M x K] op(B)[K x N] (+ bias[N]) (+ beta C), optional tanh.
// Row-major; op(A)[i][k] = TA ? A[k * lda + i] : A[i * lda + k].
constexpr int kGT = 64, kGK = 16;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
gemm_kernel(int M, int N, int K, const float *__restrict__ A, int lda,
            const float *__restrict__ B, int ldb, float *__restrict__ C, int ldc,
            const float *__restrict__ bias, int act, float beta) {
  __shared__ float sa[kGK][kGT + 1];
  __shared__ float sb[kGK][kGT + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int row0 = blockIdx.y * kGT, col0 = blockIdx.x * kGT;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kGK) {
    for (int t = threadIdx.x; t < kGK * kGT; t += 256) {
      const int kk = t / kGT, mm = t % kGT;
      const int gi = row0 + mm, gk = k0 + kk;
      float va = 0.f;
      if (gi < M && gk < K) va = TA ? A[(size_t)gk * lda + gi] : A[(size_t)gi * lda + gk];
      sa[kk][mm] = va;
      const int gj = col0 + mm;
      float vb = 0.f;
      if (gj < N && gk < K) vb = TB ? B[(size_t)gj * ldb + gk] : B[(size_t)gk * ldb + gj];
      sb[kk][mm] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; r++) a[r] = sa[kk][ty * 4 + r];
#pragma unroll
      for (int c = 0; c < 4; c++) b[c] = sb[kk][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const int gi = row0 + ty * 4 + r;
    if (gi >= M) continue;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int gj = col0 + tx * 4 + c;
      if (gj >= N) continue;
      float v = acc[r][c];
      if (bias) v += bias[gj];
      if (beta != 0.f) v += beta * C[(size_t)gi * ldc + gj];
      if (act == 1) v = tanhf(v);
      C[(size_t)gi * ldc + gj] = v;
    }
  }
}

// g *= 1 - h^2  (tanh derivative from its output)
__global__ void tanh_backward_kernel(size_t n, const float *h, float *g) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    g[e] *= 1.f - h[e] * h[e];
}

// g = scale (y - t); loss += sum (y - t)^2  (FP64 accumulation)
__global__ void mse_grad_kernel(size_t n, const float *y, const float *t, float *g, float scale,
                                double *loss) {
  double acc = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const float d = y[e] - t[e];
    g[e] = scale * d;
    acc += (double)d * d;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, acc);
}

// db[j] = sum_i dY[i][j]
__global__ void colsum_kernel(int rows, int cols, const float *dY, float *db) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  float s = 0.f;
  for (int i = 0; i < rows; i++) s += dY[(size_t)i * cols + j];
  db[j] = s;
}

// Adam (Kingma & Ba 2015) with bias correction
__global__ void adam_kernel(size_t n, float *w, const float *g, float *m, float *v, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[e];
    const float mi = b1 * m[e] + (1.f - b1) * gi;
    const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
    m[e] = mi;
    v[e] = vi;
    w[e] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

}  // namespace lmg

using namespace lmg;

extern "C" {

// Internal entry points used by the training driver (libmobility_gb300/
// precond.py) and the tests; all pointers are device memory.
int lmg_internal_gemm(int ta, int tb, int M, int N, int K, const float *A, int lda,
                      const float *B, int ldb, float *C, int ldc, const float *bias, int act,
                      float beta, void *stream) {
  dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT);
  cudaStream_t s = (cudaStream_t)stream;
  count_launch();
  if (!ta && !tb) gemm_kernel<false, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
  else if (ta && !tb) gemm_kernel<true, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
  else if (!ta && tb) gemm_kernel<false, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
  else gemm_kernel<true, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
  return (int)cudaGetLastError();
}

int lmg_internal_tanh_backward(size_t n, const float *h, float *g, void *stream) {
  count_launch();
  tanh_backward_kernel<<<(int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0,
                         (cudaStream_t)stream>>>(n, h, g);
  return (int)cudaGetLastError();
}

int lmg_internal_mse_grad(size_t n, const float *y, const float *t, float *g, float scale,
                          double *loss, void *stream) {
  count_launch();
  mse_grad_kernel<<<(int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0,
                    (cudaStream_t)stream>>>(n, y, t, g, scale, loss);
  return (int)cudaGetLastError();
}

int lmg_internal_colsum(int rows, int cols, const float *dY, float *db, void *stream) {
  count_launch();
  colsum_kernel<<<(cols + 127) / 128, 128, 0, (cudaStream_t)stream>>>(rows, cols, dY, db);
  return (int)cudaGetLastError();
}

int lmg_internal_adam(size_t n, float *w, const float *g, float *m, float *v, float lr, float b1,
                      float b2, float eps, int step, void *stream) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  count_launch();
  adam_kernel<<<(int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0,
                (cudaStream_t)stream>>>(n, w, g, m, v, lr, b1, b2, eps, c1, c2);
  return (int)cudaGetLastError();
}

int lmg_internal_knn_k(int K, const float *pos, int N, int nper, int *nb, void *stream) {
  return (int)knn_launch(K, pos, N, nper, nb, (cudaStream_t)stream);
}

int lmg_internal_precond_build_k(int K, const float *pos, const int *nb, int N,
                                 const float *params, float inv_a, float scale, float *blocks,
                                 void *stream) {
  return (int)precond_build_launch(K, pos, nb, N, params, inv_a, scale, blocks,
                                   (cudaStream_t)stream);
}

int lmg_internal_precond_apply_k(int K, const float *blocks, const int *nb, int N,
                                 const float *x, float *out, int transpose, void *stream) {
  if (transpose) {
    cudaMemsetAsync(out, 0, 3 * (size_t)N * sizeof(float), (cudaStream_t)stream);
    return (int)precond_apply_t_launch(K, blocks, nb, N, x, out, (cudaStream_t)stream);
  }
  return (int)precond_apply_launch(K, blocks, nb, N, x, out, (cudaStream_t)stream);
}

// K = 16 forms
int lmg_internal_knn(const float *pos, int N, int nper, int *nb, void *stream) {
  return lmg_internal_knn_k(16, pos, N, nper, nb, stream);
}

int lmg_internal_precond_build(const float *pos, const int *nb, int N, const float *params,
                               float inv_a, float scale, float *blocks, void *stream) {
  return lmg_internal_precond_build_k(16, pos, nb, N, params, inv_a, scale, blocks, stream);
}

int lmg_internal_precond_apply(const float *blocks, const int *nb, int N, const float *x,
                               float *out, int transpose, void *stream) {
  return lmg_internal_precond_apply_k(16, blocks, nb, N, x, out, transpose, stream);
}

}  // extern "C"
