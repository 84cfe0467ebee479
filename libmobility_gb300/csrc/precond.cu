// Kernels of the learned sparse preconditioner (see precond.cuh) and of its
// training: k-nearest neighbours, feature/MLP/rotation build of P, sparse P
// and P^T products, and the dense GEMM / activation / loss / Adam kernels the
// training loop is made of.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>

#include <cuda_fp16.h>

#include "launch_count.hpp"
#include "precond.cuh"
#include "tc_gemm.cuh"

namespace lmg {

// P blocks are stored as float or as half (unit scale; products apply the
// scale): loads and stores through these two overloads
__device__ __forceinline__ float ldf(const float *p) { return *p; }
__device__ __forceinline__ float ldf(const __half *p) { return __half2float(*p); }
__device__ __forceinline__ void stf(float *p, float v) { *p = v; }
__device__ __forceinline__ void stf(__half *p, float v) { *p = __float2half_rn(v); }

// ---------------------------------------------------------------------------
// k nearest neighbours within each batch (self first) on a uniform grid.
// The bounding box sets a cell side h for a few particles per cell on average;
// particles are counted into cells keyed by (batch, cell), the counts are
// scanned and the particles sorted by cell; then each particle searches the
// cells around its own in shells of Chebyshev distance 0, 1, 2, ... and stops
// once its K-th nearest squared distance is at most (s h)^2: every point
// closer than s h lies in a cell at Chebyshev distance <= s, so the list is
// exact.  Cost O(N x particles in the searched cells) instead of O(N^2).
// ---------------------------------------------------------------------------
constexpr int kKnnThreads = 128;
constexpr int kScanThreads = 1024;

// order-preserving map of floats to unsigned (for atomic min / max)
__device__ __forceinline__ unsigned ord_key(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float ord_float(unsigned u) {
  u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
  float f;
  std::memcpy(&f, &u, sizeof(f));
  return f;
}

// box[0..2] = keys of the minima (start 0xffffffff), box[3..5] of the maxima (start 0)
__global__ void knn_box_kernel(const float *__restrict__ pos, int N, unsigned *box) {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      lo[c] = fminf(lo[c], pos[3 * i + c]);
      hi[c] = fmaxf(hi[c], pos[3 * i + c]);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(box + c, ord_key(lo[c]));
      atomicMax(box + 3 + c, ord_key(hi[c]));
    }
  }
}

struct KnnGridShape {
  float x0, y0, z0, inv_h, h;
  int nx, ny, nz, cells;  // cells per batch
  int nper;
};

__device__ __forceinline__ int cell_coord(float v, float v0, float inv_h, int n) {
  const int c = (int)((v - v0) * inv_h);
  return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

__global__ void knn_key_kernel(const float *__restrict__ pos, int N, KnnGridShape g, int *key,
                               int *cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int ix = cell_coord(pos[3 * i], g.x0, g.inv_h, g.nx);
  const int iy = cell_coord(pos[3 * i + 1], g.y0, g.inv_h, g.ny);
  const int iz = cell_coord(pos[3 * i + 2], g.z0, g.inv_h, g.nz);
  const int k = (i / g.nper) * g.cells + (ix * g.ny + iy) * g.nz + iz;
  key[i] = k;
  atomicAdd(cnt + k, 1);
}

// exclusive scan of cnt[0..T) into start[0..T] (start[T] = total), one CTA
__global__ void __launch_bounds__(kScanThreads)
knn_scan_kernel(const int *__restrict__ cnt, int T, int *__restrict__ start) {
  __shared__ int part[kScanThreads];
  const int per = (T + kScanThreads - 1) / kScanThreads;
  const int b = threadIdx.x * per, e = min(T, b + per);
  int sum = 0;
  for (int k = b; k < e; k++) sum += cnt[k];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {  // inclusive Hillis-Steele scan
    const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = part[threadIdx.x] - sum;
  for (int k = b; k < e; k++) {
    start[k] = run;
    run += cnt[k];
  }
  if (threadIdx.x == kScanThreads - 1) start[T] = part[kScanThreads - 1];
}

__global__ void knn_scatter_kernel(const float *__restrict__ pos, int N, const int *key,
                                   const int *start, int *fill, int *sidx, float4 *spos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int k = key[i];
  const int slot = start[k] + atomicAdd(fill + k, 1);
  sidx[slot] = i;
  spos[slot] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.f);
}

// Particles are taken in cell order (thread t -> sidx[t]), so the lanes of a
// warp search the same cells: their loops stay in step and share cached reads.
// Each thread's sorted list of the KB nearest lives in shared memory
// (entry q of thread t at [q][t]: the lanes of a warp use distinct banks);
// a candidate is placed by binary search and only the tail moves.
constexpr int kSearchThreads = 64;

template <int KB>
__global__ void __launch_bounds__(kSearchThreads)
knn_search_kernel(int N, KnnGridShape g, const int *__restrict__ start,
                  const int *__restrict__ sidx, const float4 *__restrict__ spos,
                  int *__restrict__ nb) {
  __shared__ float ld[KB][kSearchThreads];
  __shared__ int lj[KB][kSearchThreads];
  const int tl = threadIdx.x;
  const int t0 = blockIdx.x * kSearchThreads + tl;
  if (t0 >= N) return;
  const int i = sidx[t0];
  const float4 pi = spos[t0];
  const float xi = pi.x, yi = pi.y, zi = pi.z;
  const int ix = cell_coord(xi, g.x0, g.inv_h, g.nx);
  const int iy = cell_coord(yi, g.y0, g.inv_h, g.ny);
  const int iz = cell_coord(zi, g.z0, g.inv_h, g.nz);
  const int base = (i / g.nper) * g.cells;
  int len = 0;
  float worst = FLT_MAX;  // ld[KB-1] once the list is full
  auto scan_cell = [&](int cx, int cy, int cz) {
    const int k = base + (cx * g.ny + cy) * g.nz + cz;
    const int e = start[k + 1];
    for (int t = start[k]; t < e; t++) {
      const float4 p = spos[t];
      const float dx = p.x - xi, dy = p.y - yi, dz = p.z - zi;
      float cd = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      if (cd < worst) {
        const int j = sidx[t];
        if (j == i) cd = -1.0f;  // the particle itself goes first
        int lo = 0, hi = len;    // first entry greater than cd
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (ld[mid][tl] > cd) hi = mid; else lo = mid + 1;
        }
        const int last = len < KB ? len : KB - 1;
        for (int q = last; q > lo; q--) {
          ld[q][tl] = ld[q - 1][tl];
          lj[q][tl] = lj[q - 1][tl];
        }
        ld[lo][tl] = cd;
        lj[lo][tl] = j;
        if (len < KB) len++;
        if (len == KB) worst = ld[KB - 1][tl];
      }
    }
  };
  const int smax = max(g.nx, max(g.ny, g.nz));
  for (int s = 0; s <= smax; s++) {
    // the cells at Chebyshev distance exactly s
    for (int dx = -s; dx <= s; dx++) {
      const int cx = ix + dx;
      if (cx < 0 || cx >= g.nx) continue;
      for (int dy = -s; dy <= s; dy++) {
        const int cy = iy + dy;
        if (cy < 0 || cy >= g.ny) continue;
        const bool face = (dx == -s || dx == s || dy == -s || dy == s);
        for (int dz = -s; dz <= s; dz += face ? 1 : (s > 0 ? 2 * s : 1)) {
          const int cz = iz + dz;
          if (cz >= 0 && cz < g.nz) scan_cell(cx, cy, cz);
        }
      }
    }
    const float r = s * g.h;
    if (len == KB && worst <= r * r) break;
  }
  for (int q = 0; q < KB; q++) nb[(size_t)q * N + i] = q < len ? lj[q][tl] : i;
}

cudaError_t knn_launch(int K, const float *pos, int N, int nper, int *nb, cudaStream_t stream,
                       KnnScratch *scratch) {
  if (K != 16 && K != 32 && K != 48 && K != 64) return cudaErrorInvalidValue;
  if (N <= 0) return cudaSuccess;
  KnnScratch local;
  KnnScratch &w = scratch ? *scratch : local;
  if (nper <= 0 || nper > N) nper = N;
  const int nbat = (N + nper - 1) / nper;
  // bounding box (one small copy back to the host)
  unsigned *box = w.box.ensure(6);
  cudaError_t e = cudaMemsetAsync(box, 0xff, 3 * sizeof(unsigned), stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(box + 3, 0, 3 * sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  count_launch();
  knn_box_kernel<<<std::min((N + 255) / 256, 1024), 256, 0, stream>>>(pos, N, box);
  unsigned *hb = w.hbox.ensure(6);
  e = cudaMemcpyAsync(hb, box, 6 * sizeof(unsigned), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return e;
  float lo[3], ext[3];
  for (int c = 0; c < 3; c++) {
    lo[c] = ord_float(hb[c]);
    ext[c] = std::max(ord_float(hb[3 + c]) - lo[c], 1e-3f);
  }
  if (!std::isfinite(ext[0] + ext[1] + ext[2])) return cudaErrorInvalidValue;
  // cell side half the expected distance r_K of the K-th neighbour at the
  // mean density (then about 2 shells reach r_K and ~ (5 r_K / 2)^3 n
  // candidates are examined); at most 2^24 cells in all
  const double per_batch = (double)N / nbat;
  const double density = per_batch / ((double)ext[0] * ext[1] * ext[2]);
  const double rK = std::cbrt(3.0 * (K + 1) / (4.0 * M_PI * density));
  double h = 0.5 * rK;
  const double cap = std::min(8.0 * per_batch + 64.0, (double)(1 << 24) / nbat);
  int dims[3];
  for (int it = 0; it < 64; it++) {
    double cells = 1;
    for (int c = 0; c < 3; c++) {
      dims[c] = std::max(1, std::min(1 << 20, (int)std::ceil(ext[c] / h)));
      cells *= dims[c];
    }
    if (cells <= cap) break;
    h *= 1.25;
  }
  KnnGridShape g;
  g.x0 = lo[0];
  g.y0 = lo[1];
  g.z0 = lo[2];
  g.h = (float)h;
  g.inv_h = (float)(1.0 / h);
  g.nx = dims[0];
  g.ny = dims[1];
  g.nz = dims[2];
  g.cells = dims[0] * dims[1] * dims[2];
  g.nper = nper;
  const int T = nbat * g.cells;
  int *key = w.key.ensure(N);
  int *cnt = w.cnt.ensure((size_t)T + 1);
  int *start = w.start.ensure((size_t)T + 1);
  int *sidx = w.sidx.ensure(N);
  float4 *spos = w.spos.ensure(N);
  e = cudaMemsetAsync(cnt, 0, ((size_t)T + 1) * sizeof(int), stream);
  if (e != cudaSuccess) return e;
  const int grid = (N + 255) / 256;
  count_launch();
  knn_key_kernel<<<grid, 256, 0, stream>>>(pos, N, g, key, cnt);
  count_launch();
  knn_scan_kernel<<<1, kScanThreads, 0, stream>>>(cnt, T, start);
  e = cudaMemsetAsync(cnt, 0, ((size_t)T + 1) * sizeof(int), stream);  // reused as fill counts
  if (e != cudaSuccess) return e;
  count_launch();
  knn_scatter_kernel<<<grid, 256, 0, stream>>>(pos, N, key, start, cnt, sidx, spos);
  const int sg = (N + kSearchThreads - 1) / kSearchThreads;
  count_launch();
  if (K == 16) knn_search_kernel<17><<<sg, kSearchThreads, 0, stream>>>(N, g, start, sidx, spos, nb);
  if (K == 32) knn_search_kernel<33><<<sg, kSearchThreads, 0, stream>>>(N, g, start, sidx, spos, nb);
  if (K == 48) knn_search_kernel<49><<<sg, kSearchThreads, 0, stream>>>(N, g, start, sidx, spos, nb);
  if (K == 64) knn_search_kernel<65><<<sg, kSearchThreads, 0, stream>>>(N, g, start, sidx, spos, nb);
  e = cudaGetLastError();
  if (e == cudaSuccess && !scratch) e = cudaStreamSynchronize(stream);  // before `local` goes
  return e;
}

// ---------------------------------------------------------------------------
// P rows: canonical frame and features (one thread per particle), the MLP as
// three GEMMs over all particles (gemm_launch below, bias and tanh fused),
// then the blocks rotated back to the lab frame (one thread per block).
// ---------------------------------------------------------------------------
constexpr int kBuildThreads = 128;

template <int K, bool WALL>
__global__ void __launch_bounds__(kBuildThreads)
precond_features_kernel(const float *__restrict__ pos, const int *__restrict__ nb, int N,
                        const float *__restrict__ xmean, const float *__restrict__ xstd,
                        float inv_a, float *__restrict__ X, int ldx, float *__restrict__ E) {
  constexpr int In = 3 * K + (WALL ? 1 : 0);
  const int i = blockIdx.x * kBuildThreads + threadIdx.x;
  if (i >= N) return;
  const int *nbi = nb + i;  // nb[n][i]
  const float xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
  float rel[K][3];
#pragma unroll
  for (int n = 0; n < K; n++) {
    const int j = nbi[(size_t)(n + 1) * N];
    rel[n][0] = (pos[3 * j] - xi) * inv_a;
    rel[n][1] = (pos[3 * j + 1] - yi) * inv_a;
    rel[n][2] = (pos[3 * j + 2] - zi) * inv_a;
  }
  // canonical frame: x to the nearest neighbour, y to the first neighbour
  // that is not collinear with it, z = x cross y; with a wall, z is the wall
  // normal and x the horizontal direction to the nearest neighbour that is
  // not straight above or below
  float e[3][3];
  if (WALL) {
    float c = 1.f, s = 0.f;
    bool found = false;
#pragma unroll
    for (int n = 0; n < K; n++) {
      const float hh = rel[n][0] * rel[n][0] + rel[n][1] * rel[n][1];
      if (!found && hh > 1e-12f) {
        const float li = rsqrtf(hh);
        c = rel[n][0] * li;
        s = rel[n][1] * li;
        found = true;
      }
    }
    e[0][0] = c;   e[0][1] = s;   e[0][2] = 0.f;
    e[1][0] = -s;  e[1][1] = c;   e[1][2] = 0.f;
    e[2][0] = 0.f; e[2][1] = 0.f; e[2][2] = 1.f;
  } else {
    const float l = rsqrtf(fmaxf(rel[0][0] * rel[0][0] + rel[0][1] * rel[0][1] +
                                 rel[0][2] * rel[0][2], 1e-30f));
    e[0][0] = rel[0][0] * l;
    e[0][1] = rel[0][1] * l;
    e[0][2] = rel[0][2] * l;
    float y0 = 0.f, y1 = 1.f, y2 = 0.f;
    bool found = false;
#pragma unroll
    for (int n = 1; n < K; n++) {
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
  float *x = X + (size_t)i * ldx;
#pragma unroll
  for (int n = 0; n < K; n++) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float v = rel[n][0] * e[c][0] + rel[n][1] * e[c][1] + rel[n][2] * e[c][2];
      x[3 * n + c] = (v - xmean[3 * n + c]) / xstd[3 * n + c];
    }
  }
  if (WALL) {  // height above the wall, clamped at one radius as the physics does
    const float h = fmaxf(zi * inv_a, 1.f);
    x[3 * K] = (h - xmean[3 * K]) / xstd[3 * K];
  }
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) E[9 * (size_t)i + 3 * r + c] = e[r][c];
}

// One thread per (particle, block n): de-normalised outputs -> block in the
// canonical frame (n = 0: symmetric self block from 6 units 00 01 02 11 12
// 22; n > 0: 9 units) -> lab frame E^T b E, times scale.
template <int K, class T>
__global__ void precond_assemble_kernel(const float *__restrict__ Y,
                                        const float *__restrict__ E, int N,
                                        const float *__restrict__ ymean,
                                        const float *__restrict__ ystd, float scale,
                                        T *__restrict__ blocks) {
  constexpr int Out = 6 + 9 * K;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)N * (K + 1)) return;
  const int n = (int)(t / N), i = (int)(t % N);  // consecutive threads: consecutive i
  const float *y = Y + (size_t)i * Out;
  auto unit = [&](int o) { return y[o] * ystd[o] + ymean[o]; };
  float b[3][3];
  if (n == 0) {
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
  float e[3][3];
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) e[r][c] = E[9 * (size_t)i + 3 * r + c];
  T *out = blocks + (size_t)n * 9 * N + i;  // blocks[n][e][i]
#pragma unroll
  for (int r = 0; r < 3; r++) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float acc = 0.f;
#pragma unroll
      for (int p = 0; p < 3; p++) {
        const float tt = b[p][0] * e[0][c] + b[p][1] * e[1][c] + b[p][2] * e[2][c];
        acc = fmaf(e[p][r], tt, acc);
      }
      stf(out + (size_t)(3 * r + c) * N, acc * scale);
    }
  }
}

cudaError_t gemm_launch(int ta, int tb, int M, int N, int K, const float *A, int lda,
                        const float *B, int ldb, float *C, int ldc, const float *bias, int act,
                        float beta, cudaStream_t s);

// out[c][r] = in[r][c] (in: rows x cols, row-major; out rows ldo apart)
__global__ void transpose_kernel(const float *__restrict__ in, int rows, int cols,
                                 float *__restrict__ out, int ldo) {
  __shared__ float t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[k][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (c < cols && r < rows) out[(size_t)c * ldo + r] = t[threadIdx.x][k];
  }
}

cudaError_t transpose_launch(const float *in, int rows, int cols, float *out, int ldo,
                             cudaStream_t s) {
  count_launch();
  transpose_kernel<<<dim3((cols + 31) / 32, (rows + 31) / 32), dim3(32, 8), 0, s>>>(in, rows, cols,
                                                                                    out, ldo);
  return cudaGetLastError();
}

cudaError_t precond_build_launch(const PrecLayout &L, const float *pos, const int *nb, int N,
                                 const float *params, float inv_a, float scale, void *blocks,
                                 bool half, PrecWork *work, cudaStream_t stream) {
  if (L.K != 16 && L.K != 32 && L.K != 48 && L.K != 64) return cudaErrorInvalidValue;
  if (N <= 0) return cudaSuccess;
  PrecWork local;
  PrecWork &w = work ? *work : local;
  // the tensor-core GEMM takes rows of a multiple of 4 floats (16 bytes)
  const bool tc = g_precond_tc.load() != 0 && tc_gemm_available();
  const int ldx = tc ? (L.In + 3) & ~3 : L.In;
  float *X = w.X.ensure((size_t)N * ldx);
  float *E = w.E.ensure((size_t)N * 9);
  float *H1 = w.H1.ensure((size_t)N * L.H);
  float *H2 = w.H2.ensure((size_t)N * L.H);
  float *Y = w.Y.ensure((size_t)N * L.Out);
  const int g = (N + kBuildThreads - 1) / kBuildThreads;
  const float *xm = params + L.Xm, *xs = params + L.Xs;
  count_launch();
#define LMG_FEATURES(KK)                                                                   \
  if (L.K == KK) {                                                                         \
    if (L.wall)                                                                            \
      precond_features_kernel<KK, true><<<g, kBuildThreads, 0, stream>>>(pos, nb, N, xm, xs, \
                                                                         inv_a, X, ldx, E); \
    else                                                                                   \
      precond_features_kernel<KK, false><<<g, kBuildThreads, 0, stream>>>(               \
          pos, nb, N, xm, xs, inv_a, X, ldx, E);                                           \
  }
  LMG_FEATURES(16)
  LMG_FEATURES(32)
  LMG_FEATURES(48)
  LMG_FEATURES(64)
#undef LMG_FEATURES
  cudaError_t e = cudaGetLastError();
  if (tc) {
    // tcgen05 (TF32) layers: the weights transposed to K-major rows first
    const int ld1 = (L.In + 3) & ~3;
    float *WT = w.WT.ensure((size_t)L.H * ld1 + (size_t)L.H * L.H + (size_t)L.Out * L.H);
    float *WT1 = WT, *WT2 = WT1 + (size_t)L.H * ld1, *WT3 = WT2 + (size_t)L.H * L.H;
    if (e == cudaSuccess) e = transpose_launch(params + L.W1, L.In, L.H, WT1, ld1, stream);
    if (e == cudaSuccess) e = transpose_launch(params + L.W2, L.H, L.H, WT2, L.H, stream);
    if (e == cudaSuccess) e = transpose_launch(params + L.W3, L.H, L.Out, WT3, L.H, stream);
    if (e == cudaSuccess)
      e = tc_gemm_launch(N, L.H, L.In, X, ldx, WT1, ld1, H1, L.H, params + L.B1, 1, stream);
    if (e == cudaSuccess)
      e = tc_gemm_launch(N, L.H, L.H, H1, L.H, WT2, L.H, H2, L.H, params + L.B2, 1, stream);
    if (e == cudaSuccess)
      e = tc_gemm_launch(N, L.Out, L.H, H2, L.H, WT3, L.H, Y, L.Out, params + L.B3, 0, stream);
  } else {
    if (e == cudaSuccess)
      e = gemm_launch(0, 0, N, L.H, L.In, X, L.In, params + L.W1, L.H, H1, L.H, params + L.B1,
                      1, 0.f, stream);
    if (e == cudaSuccess)
      e = gemm_launch(0, 0, N, L.H, L.H, H1, L.H, params + L.W2, L.H, H2, L.H, params + L.B2,
                      1, 0.f, stream);
    if (e == cudaSuccess)
      e = gemm_launch(0, 0, N, L.Out, L.H, H2, L.H, params + L.W3, L.Out, Y, L.Out,
                      params + L.B3, 0, 0.f, stream);
  }
  if (e != cudaSuccess) return e;
  const long nblk = (long)N * (L.K + 1);
  const int ga = (int)((nblk + 255) / 256);
  const float *ym = params + L.Ym, *ys = params + L.Ys;
  count_launch();
  float *bf = static_cast<float *>(blocks);
  __half *bh = static_cast<__half *>(blocks);
  if (L.K == 16 && half) precond_assemble_kernel<16><<<ga, 256, 0, stream>>>(Y, E, N, ym, ys, scale, bh);
  if (L.K == 32 && half) precond_assemble_kernel<32><<<ga, 256, 0, stream>>>(Y, E, N, ym, ys, scale, bh);
  if (L.K == 48 && half) precond_assemble_kernel<48><<<ga, 256, 0, stream>>>(Y, E, N, ym, ys, scale, bh);
  if (L.K == 64 && half) precond_assemble_kernel<64><<<ga, 256, 0, stream>>>(Y, E, N, ym, ys, scale, bh);
  if (L.K == 16 && !half) precond_assemble_kernel<16><<<ga, 256, 0, stream>>>(Y, E, N, ym, ys, scale, bf);
  if (L.K == 32 && !half) precond_assemble_kernel<32><<<ga, 256, 0, stream>>>(Y, E, N, ym, ys, scale, bf);
  if (L.K == 48 && !half) precond_assemble_kernel<48><<<ga, 256, 0, stream>>>(Y, E, N, ym, ys, scale, bf);
  if (L.K == 64 && !half) precond_assemble_kernel<64><<<ga, 256, 0, stream>>>(Y, E, N, ym, ys, scale, bf);
  e = cudaGetLastError();
  if (e == cudaSuccess && !work) e = cudaStreamSynchronize(stream);  // before `local` goes
  return e;
}

// ---------------------------------------------------------------------------
// Sparse products with P (rows of K+1 3x3 blocks)
// ---------------------------------------------------------------------------
// Each row is shared by kRowSplit threads (threadIdx.y), each taking every
// kRowSplit-th block, so there are enough threads in flight to cover the
// memory latency; threadIdx.x runs along the rows, so every load of blocks
// and neighbour lists is coalesced.
constexpr int kRowX = 64, kRowSplit = 4;

template <int KB, class T>
__global__ void __launch_bounds__(kRowX * kRowSplit, 8)
precond_apply_kernel(const T *__restrict__ B, const int *__restrict__ nb, int N,
                     const float *__restrict__ x, float *__restrict__ out, float scale) {
  __shared__ float part[kRowSplit][3][kRowX];
  const int i = blockIdx.x * kRowX + threadIdx.x;
  const int q = threadIdx.y;
  const size_t sN = (size_t)N;
  float o0 = 0.f, o1 = 0.f, o2 = 0.f;
  if (i < N) {
#pragma unroll 2
    for (int n = q; n < KB; n += kRowSplit) {
      const int j = nb[n * sN + i];
      const T *b = B + (size_t)n * 9 * sN + i;  // b[e * N]: element e of block n
      const float v0 = x[3 * j], v1 = x[3 * j + 1], v2 = x[3 * j + 2];
      o0 = fmaf(ldf(b), v0, fmaf(ldf(b + sN), v1, fmaf(ldf(b + 2 * sN), v2, o0)));
      o1 = fmaf(ldf(b + 3 * sN), v0, fmaf(ldf(b + 4 * sN), v1, fmaf(ldf(b + 5 * sN), v2, o1)));
      o2 = fmaf(ldf(b + 6 * sN), v0, fmaf(ldf(b + 7 * sN), v1, fmaf(ldf(b + 8 * sN), v2, o2)));
    }
  }
  part[q][0][threadIdx.x] = o0;
  part[q][1][threadIdx.x] = o1;
  part[q][2][threadIdx.x] = o2;
  __syncthreads();
  if (q < 3 && i < N) {  // thread row q writes component q, summing the groups in order
    float t = 0.f;
#pragma unroll
    for (int g = 0; g < kRowSplit; g++) t += part[g][q][threadIdx.x];
    out[3 * i + q] = t * scale;
  }
}

// P^T x: one thread per row scatters its K+1 products with one 16-byte
// vector atomic each into a float4-padded copy of the output (a third of
// the L2 atomic operations of three scalar ones, which saturated L2), then
// a second pass packs the padded copy into the 3-component output.
template <int KB, class T>
__global__ void __launch_bounds__(256, 4)
precond_apply_t_kernel(const T *__restrict__ B, const int *__restrict__ nb, int N,
                       const float *__restrict__ x, float4 *pad, float scale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const size_t sN = (size_t)N;
  const float v0 = scale * x[3 * i], v1 = scale * x[3 * i + 1], v2 = scale * x[3 * i + 2];
#pragma unroll 4
  for (int n = 0; n < KB; n++) {
    const int j = nb[n * sN + i];
    const T *b = B + (size_t)n * 9 * sN + i;
    atomicAdd(pad + j,
              make_float4(ldf(b) * v0 + ldf(b + 3 * sN) * v1 + ldf(b + 6 * sN) * v2,
                          ldf(b + sN) * v0 + ldf(b + 4 * sN) * v1 + ldf(b + 7 * sN) * v2,
                          ldf(b + 2 * sN) * v0 + ldf(b + 5 * sN) * v1 + ldf(b + 8 * sN) * v2,
                          0.f));
  }
}

__global__ void __launch_bounds__(256) unpad3_kernel(const float4 *pad, int N, float *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const float4 p = pad[i];
  out[3 * i] = p.x;
  out[3 * i + 1] = p.y;
  out[3 * i + 2] = p.z;
}

template <int KB, class T>
void apply_dispatch(bool transpose, const T *B, const int *nb, int N, const float *x, float *out,
                    float4 *pad, float scale, cudaStream_t stream) {
  if (transpose)
    precond_apply_t_kernel<KB, T><<<(N + 255) / 256, 256, 0, stream>>>(B, nb, N, x, pad, scale);
  else
    precond_apply_kernel<KB, T><<<(N + kRowX - 1) / kRowX, dim3(kRowX, kRowSplit), 0, stream>>>(
        B, nb, N, x, out, scale);
}

template <class T>
cudaError_t apply_k(int K, bool transpose, const void *blocks, const int *nb, int N,
                    const float *x, float *out, float4 *pad, float scale, cudaStream_t stream) {
  const T *B = static_cast<const T *>(blocks);
  if (K != 16 && K != 32 && K != 48 && K != 64) return cudaErrorInvalidValue;
  if (N <= 0) return cudaSuccess;
  if (transpose) {
    if (!pad) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(pad, 0, (size_t)N * sizeof(float4), stream);
    if (e != cudaSuccess) return e;
  }
  count_launch();
  if (K == 16) apply_dispatch<17, T>(transpose, B, nb, N, x, out, pad, scale, stream);
  if (K == 32) apply_dispatch<33, T>(transpose, B, nb, N, x, out, pad, scale, stream);
  if (K == 48) apply_dispatch<49, T>(transpose, B, nb, N, x, out, pad, scale, stream);
  if (K == 64) apply_dispatch<65, T>(transpose, B, nb, N, x, out, pad, scale, stream);
  if (transpose) {
    count_launch();
    unpad3_kernel<<<(N + 255) / 256, 256, 0, stream>>>(pad, N, out);
  }
  return cudaGetLastError();
}

cudaError_t precond_apply_launch(int K, const void *blocks, bool half, float scale,
                                 const int *nb, int N, const float *x, float *out,
                                 cudaStream_t stream) {
  return half ? apply_k<__half>(K, false, blocks, nb, N, x, out, nullptr, scale, stream)
              : apply_k<float>(K, false, blocks, nb, N, x, out, nullptr, scale, stream);
}

cudaError_t precond_apply_t_launch(int K, const void *blocks, bool half, float scale,
                                   const int *nb, int N, const float *x, float *out,
                                   float4 *pad, cudaStream_t stream) {
  return half ? apply_k<__half>(K, true, blocks, nb, N, x, out, pad, scale, stream)
              : apply_k<float>(K, true, blocks, nb, N, x, out, pad, scale, stream);
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

// Register-blocked form for large products: 128 x 128 tile per CTA, 16-deep
// slabs of A and B in shared memory, 8 x 8 outputs per thread in two 4-wide
// groups per dimension (rows 4 ty + r and 64 + 4 ty + r, columns likewise
// with tx), so the inner loop reads shared memory as float4 without bank
// conflicts and does 64 FMAs per 4 vector loads.  Tile loads put consecutive
// threads on consecutive addresses for every transposition.
constexpr int kGT2 = 128, kGK2 = 16;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
gemm_kernel2(int M, int N, int K, const float *__restrict__ A, int lda,
             const float *__restrict__ B, int ldb, float *__restrict__ C, int ldc,
             const float *__restrict__ bias, int act, float beta) {
  __shared__ __align__(16) float sa[kGK2][kGT2 + 4];
  __shared__ __align__(16) float sb[kGK2][kGT2 + 4];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int row0 = blockIdx.y * kGT2, col0 = blockIdx.x * kGT2;
  float acc[8][8] = {};
  for (int k0 = 0; k0 < K; k0 += kGK2) {
#pragma unroll
    for (int q = 0; q < (kGK2 * kGT2) / 256; q++) {
      const int t = tid + 256 * q;
      // A tile: element (mm, kk) = op(A)[row0 + mm][k0 + kk]
      const int amm = TA ? t % kGT2 : t / kGK2, akk = TA ? t / kGT2 : t % kGK2;
      const int gi = row0 + amm, gk = k0 + akk;
      float va = 0.f;
      if (gi < M && gk < K) va = TA ? A[(size_t)gk * lda + gi] : A[(size_t)gi * lda + gk];
      sa[akk][amm] = va;
      // B tile: element (kk, nn) = op(B)[k0 + kk][col0 + nn]
      const int bnn = TB ? t / kGK2 : t % kGT2, bkk = TB ? t % kGK2 : t / kGT2;
      const int gj = col0 + bnn, gk2 = k0 + bkk;
      float vb = 0.f;
      if (gj < N && gk2 < K) vb = TB ? B[(size_t)gj * ldb + gk2] : B[(size_t)gk2 * ldb + gj];
      sb[bkk][bnn] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK2; kk++) {
      const float4 a0 = *reinterpret_cast<const float4 *>(&sa[kk][4 * ty]);
      const float4 a1 = *reinterpret_cast<const float4 *>(&sa[kk][64 + 4 * ty]);
      const float4 b0 = *reinterpret_cast<const float4 *>(&sb[kk][4 * tx]);
      const float4 b1 = *reinterpret_cast<const float4 *>(&sb[kk][64 + 4 * tx]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 8; c++) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int gi = row0 + (r < 4 ? 4 * ty + r : 64 + 4 * ty + r - 4);
    if (gi >= M) continue;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int gj = col0 + (c < 4 ? 4 * tx + c : 64 + 4 * tx + c - 4);
      if (gj >= N) continue;
      float v = acc[r][c];
      if (bias) v += bias[gj];
      if (beta != 0.f) v += beta * C[(size_t)gi * ldc + gj];
      if (act == 1) v = tanhf(v);
      C[(size_t)gi * ldc + gj] = v;
    }
  }
}

cudaError_t gemm_launch(int ta, int tb, int M, int N, int K, const float *A, int lda,
                        const float *B, int ldb, float *C, int ldc, const float *bias, int act,
                        float beta, cudaStream_t s) {
  if ((long)M * N >= 64L * 128 * 128) {  // enough output tiles for the large form
    dim3 grid2((N + kGT2 - 1) / kGT2, (M + kGT2 - 1) / kGT2);
    count_launch();
    if (!ta && !tb) gemm_kernel2<false, false><<<grid2, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
    else if (ta && !tb) gemm_kernel2<true, false><<<grid2, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
    else if (!ta && tb) gemm_kernel2<false, true><<<grid2, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
    else gemm_kernel2<true, true><<<grid2, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
    return cudaGetLastError();
  }
  dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT);
  count_launch();
  if (!ta && !tb) gemm_kernel<false, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
  else if (ta && !tb) gemm_kernel<true, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
  else if (!ta && tb) gemm_kernel<false, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
  else gemm_kernel<true, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta);
  return cudaGetLastError();
}

}  // namespace lmg

using namespace lmg;

extern "C" {

// Internal entry points used by the training driver (libmobility_gb300/
// precond.py) and the tests; all pointers are device memory.
int lmg_internal_gemm(int ta, int tb, int M, int N, int K, const float *A, int lda,
                      const float *B, int ldb, float *C, int ldc, const float *bias, int act,
                      float beta, void *stream) {
  return (int)lmg::gemm_launch(ta, tb, M, N, K, A, lda, B, ldb, C, ldc, bias, act, beta,
                               (cudaStream_t)stream);
}

// C = act(A Bt^T + bias) on the tensor cores (tcgen05, TF32); see tc_gemm.cuh.
int lmg_internal_tc_gemm(int M, int N, int K, const float *A, int lda, const float *Bt, int ldbt,
                         float *C, int ldc, const float *bias, int act, void *stream) {
  return (int)lmg::tc_gemm_launch(M, N, K, A, lda, Bt, ldbt, C, ldc, bias, act,
                                  (cudaStream_t)stream);
}

// Status word of the tensor-core GEMM (non-zero: a bounded wait ran out);
// reset != 0 clears it.  -1 if it cannot be read.
int lmg_internal_tc_status(int reset) { return lmg::tc_gemm_status(reset != 0); }

// 1: the preconditioner build runs its network on the tensor cores where the
// GPU has them; 0: on the CUDA cores.  Returns 1 for a bad value.
int lmg_internal_precond_tc(int on) {
  if (on != 0 && on != 1) return 1;
  lmg::g_precond_tc.store(on);
  return 0;
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
  try {
    return (int)knn_launch(K, pos, N, nper, nb, (cudaStream_t)stream, nullptr);
  } catch (const std::exception &) {
    return (int)cudaErrorMemoryAllocation;
  }
}

int lmg_internal_precond_build_kh(int K, int H, const float *pos, const int *nb, int N,
                                  const float *params, float inv_a, float scale, float *blocks,
                                  void *stream) {
  try {
    return (int)precond_build_launch(prec_layout(K, H), pos, nb, N, params, inv_a, scale,
                                     blocks, false, nullptr, (cudaStream_t)stream);
  } catch (const std::exception &) {
    return (int)cudaErrorMemoryAllocation;
  }
}


// The same for a wall network (frame about the wall normal, height input).
int lmg_internal_precond_build_wall(int K, int H, const float *pos, const int *nb, int N,
                                    const float *params, float inv_a, float scale, float *blocks,
                                    void *stream) {
  try {
    return (int)precond_build_launch(prec_layout(K, H, true), pos, nb, N, params, inv_a, scale,
                                     blocks, false, nullptr, (cudaStream_t)stream);
  } catch (const std::exception &) {
    return (int)cudaErrorMemoryAllocation;
  }
}

// Either product with float (half = 0) or half blocks (half = 1, applied
// with scale 1).  The transposed product needs a float4 work array of N
// entries: `pad`, or one allocated and freed here (the call then waits).
int lmg_internal_precond_apply_kh(int K, const void *blocks, int half, const int *nb, int N,
                                  const float *x, float *out, int transpose, float *pad,
                                  void *stream) {
  const cudaStream_t st = (cudaStream_t)stream;
  if (!transpose)
    return (int)precond_apply_launch(K, blocks, half != 0, 1.0f, nb, N, x, out, st);
  float4 *p = reinterpret_cast<float4 *>(pad);
  if (p) return (int)precond_apply_t_launch(K, blocks, half != 0, 1.0f, nb, N, x, out, p, st);
  cudaError_t e = cudaMalloc(&p, (size_t)std::max(N, 1) * sizeof(float4));
  if (e != cudaSuccess) return (int)e;
  e = precond_apply_t_launch(K, blocks, half != 0, 1.0f, nb, N, x, out, p, st);
  const cudaError_t e2 = cudaStreamSynchronize(st);
  cudaFree(p);
  return (int)(e != cudaSuccess ? e : e2);
}

int lmg_internal_precond_apply_k(int K, const float *blocks, const int *nb, int N,
                                 const float *x, float *out, int transpose, void *stream) {
  return lmg_internal_precond_apply_kh(K, blocks, 0, nb, N, x, out, transpose, nullptr, stream);
}

// K = 16 forms
int lmg_internal_knn(const float *pos, int N, int nper, int *nb, void *stream) {
  return lmg_internal_knn_k(16, pos, N, nper, nb, stream);
}

int lmg_internal_precond_build(const float *pos, const int *nb, int N, const float *params,
                               float inv_a, float scale, float *blocks, void *stream) {
  return lmg_internal_precond_build_kh(16, 64, pos, nb, N, params, inv_a, scale, blocks, stream);
}

int lmg_internal_precond_apply(const float *blocks, const int *nb, int N, const float *x,
                               float *out, int transpose, void *stream) {
  return lmg_internal_precond_apply_k(16, blocks, nb, N, x, out, transpose, stream);
}

}  // extern "C"
