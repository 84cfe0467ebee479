// Tensor-core GEMM for the preconditioner network: tcgen05.mma of kind::tf32
// with the accumulator in tensor memory, operand tiles brought to shared
// memory by TMA (cp.async.bulk.tensor, 128-byte swizzle) through a 4-stage
// mbarrier pipeline.
//
// One CTA of 4 warps computes a 128 x 256 tile of C:
//   * thread 0 issues the TMA loads (A rows m0.., Bt rows n0.., 32 K a stage,
//     128 bytes per row: one 128-byte swizzle row) and, as each stage lands,
//     four tcgen05.mma (M = 128, N = 256, K = 8) into the 256 tensor-memory
//     columns the CTA allocated; tcgen05.commit frees the stage for its next
//     load, and a last commit signals the end of the products;
//   * all four warps then read their 32 tensor-memory lanes (rows) with
//     tcgen05.ld, add the bias, apply tanh, stage the rows in the idle stage
//     buffers and write them to C with consecutive lanes on consecutive
//     columns.
// Every wait on an mbarrier is bounded (~0.4 s); one that runs out sets a
// status word, the CTA waits (bounded) for its products and copies in flight,
// frees its tensor memory and returns without writing C.
// Operands out of range (rows past M or N, K past K) are zero-filled by TMA.
#include <cstdint>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include "launch_count.hpp"
#include "tc_gemm.cuh"

namespace lmg {
namespace {

constexpr int kBM = 128;  // rows of C per CTA = tensor-memory lanes
constexpr int kBN = 256;  // columns of C per CTA = tensor-memory columns (FP32)
constexpr int kBK = 32;   // K per stage: 32 FP32 = 128 bytes, one swizzle row
constexpr int kUK = 8;    // K of one tcgen05.mma of kind::tf32
constexpr int kStages = 4;
constexpr int kThreads = 128;
constexpr uint32_t kABytes = kBM * kBK * 4;
constexpr uint32_t kBBytes = kBN * kBK * 4;
constexpr uint32_t kStageBytes = kABytes + kBBytes;
constexpr size_t kSmem = (size_t)kStages * kStageBytes + 1024;  // + alignment slack
constexpr int kPitch = kBN + 4;  // floats per row of the output staging tile
static_assert((size_t)kBM * kPitch * 4 <= (size_t)kStages * kStageBytes,
              "the output staging tile reuses the stage buffers");
constexpr long kSpins = 1L << 22;

__device__ int g_tc_status;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for the phase of the given parity; false if it never came
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long it = 0; it < kSpins; it++) {
    if (mbar_test(bar, parity)) return true;
    if (it > 64) __nanosleep(100);
  }
  return false;
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, uint32_t bar,
                                           int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}
// shared-memory matrix descriptor of a K-major operand tile with 128-byte
// swizzle: rows of 128 bytes, 8-row groups 1024 bytes apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address, 16-byte units
  d |= (uint64_t)1 << 16;                            // leading offset (unused here)
  d |= (uint64_t)(1024 >> 4) << 32;                  // stride offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                            // descriptor version
  d |= (uint64_t)2 << 61;                            // 128-byte swizzle
  return d;
}
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               int M, int N, int K, float *__restrict__ C, int ldc,
               const float *__restrict__ bias, int act) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t s_bar[2 * kStages + 2];  // full, empty, done, drain
  __shared__ uint32_t s_tmem;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;  // swizzle atoms: 1024-aligned
  const uint32_t bar0 = smem_u32(s_bar);
  const uint32_t done = bar0 + 8u * (2 * kStages);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  const int nk = (K + kBK - 1) / kBK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < 2 * kStages + 2; s++) mbar_init(bar0 + 8u * s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&s_tmem)),
                 "r"(kBN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;

  if (threadIdx.x == 0) {
    // D = F32, A = B = TF32, both K-major, N = 256, M = 128
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                           ((uint32_t)(kBM >> 4) << 24);
    int loaded = 0, consumed = 0, fail = 0;
    auto load = [&](int c) {
      const int s = c % kStages;
      const uint32_t sa = base + (uint32_t)s * kStageBytes;
      mbar_expect_tx(bar0 + 8u * s, kStageBytes);
      tma_load_2d(sa, &tmA, bar0 + 8u * s, c * kBK, m0);
      tma_load_2d(sa + kABytes, &tmB, bar0 + 8u * s, c * kBK, n0);
      loaded = c + 1;
    };
    for (int c = 0; c < nk && c < kStages; c++) load(c);
    for (int c = 0; c < nk; c++) {
      const int s = c % kStages;
      if (!mbar_wait(bar0 + 8u * s, (uint32_t)(c / kStages) & 1u)) {
        fail = 1;
        break;
      }
      consumed = c + 1;
      const uint32_t sa = base + (uint32_t)s * kStageBytes;
#pragma unroll
      for (int k = 0; k < kBK / kUK; k++)
        mma_tf32(tmem, sw128_desc(sa + 4u * kUK * k), sw128_desc(sa + kABytes + 4u * kUK * k),
                 idesc, (c | k) != 0 ? 1u : 0u);
      mma_commit(bar0 + 8u * (kStages + s));
      // refill the stage of the previous chunk once its products are done
      if (c >= 1 && c - 1 + kStages < nk) {
        const int sp = (c - 1) % kStages;
        if (!mbar_wait(bar0 + 8u * (kStages + sp), (uint32_t)((c - 1) / kStages) & 1u)) {
          fail = 2;
          break;
        }
        load(c - 1 + kStages);
      }
    }
    if (!fail) {
      mma_commit(done);
    } else {
      // no result: the products issued and the copies in flight end before
      // the CTA leaves ("done" never completes, so no warp writes C)
      mma_commit(done + 8u);
      (void)mbar_wait(done + 8u, 0);
      for (int c = consumed; c < loaded; c++)
        (void)mbar_wait(bar0 + 8u * (c % kStages), (uint32_t)(c / kStages) & 1u);
      atomicExch(&g_tc_status, fail);
    }
  }
  __syncwarp();
  const bool ok = mbar_wait(done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    // tensor memory -> bias, activation -> a row-major staging tile in the
    // (now idle) stage buffers -> coalesced rows of C
    float *stage = reinterpret_cast<float *>(smem_raw + (base - smem_u32(smem_raw)));
    const int r = 32 * warp + lane;  // this thread's row of the tile
    const uint32_t lane_base = tmem + ((uint32_t)(32 * warp) << 16);
    const int ncols = min(kBN, N - n0);
    for (int j = 0; j < ncols; j += 16) {
      uint32_t v[16];
      tmem_ld16(lane_base + (uint32_t)j, v);
      float x[16];
#pragma unroll
      for (int q = 0; q < 16; q++) {
        x[q] = __uint_as_float(v[q]);
        const int col = n0 + j + q;
        if (bias && col < N) x[q] += __ldg(bias + col);
        if (act == 1) x[q] = tanhf(x[q]);
      }
      float4 *dst = reinterpret_cast<float4 *>(stage + (size_t)r * kPitch + j);
#pragma unroll
      for (int q = 0; q < 4; q++) dst[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
    }
    __syncwarp();
    // each warp writes its own 32 rows, a row at a time, lanes on consecutive columns
    for (int rr = 0; rr < 32; rr++) {
      const int row = m0 + 32 * warp + rr;
      if (row >= M) break;
      const float *src = stage + (size_t)(32 * warp + rr) * kPitch;
      float *out = C + (size_t)row * ldc + n0;
      for (int c = lane; c < ncols; c += 32) out[c] = src[c];
    }
  } else if (threadIdx.x == 0) {
    atomicExch(&g_tc_status, 3);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kBN)
                 : "memory");
}

using EncodeTiled = PFN_cuTensorMapEncodeTiled_v12000;

EncodeTiled encoder() {
  static const EncodeTiled fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      (void)cudaGetLastError();
      return (EncodeTiled) nullptr;
    }
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

// 2-D map of a row-major FP32 matrix (rows x cols, ld floats per row) with
// boxes of 32 columns x box_rows rows and the 128-byte swizzle
bool make_map(CUtensorMap *m, const float *base, int rows, int cols, int ld, int box_rows) {
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return encoder()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims,
                   strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool tc_gemm_available() {
  int dev = 0, major = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return major == 10 && encoder() != nullptr;
}

int tc_gemm_status(bool reset) {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_status, sizeof(int)) != cudaSuccess) return -1;
  if (reset) {
    const int zero = 0;
    if (cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(int)) != cudaSuccess) return -1;
  }
  return v;
}

cudaError_t tc_gemm_launch(int M, int N, int K, const float *A, int lda, const float *Bt,
                           int ldbt, float *C, int ldc, const float *bias, int act,
                           cudaStream_t stream) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  if (K < 1 || lda < K || ldbt < K || lda % 4 || ldbt % 4 ||
      (reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(Bt) & 15) ||
      ldc < N || (act != 0 && act != 1))
    return cudaErrorInvalidValue;
  if (!tc_gemm_available()) return cudaErrorNotSupported;
  static const cudaError_t attr = cudaFuncSetAttribute(
      tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  if (attr != cudaSuccess) return attr;
  CUtensorMap ma, mb;
  if (!make_map(&ma, A, M, K, lda, kBM) || !make_map(&mb, Bt, N, K, ldbt, kBN))
    return cudaErrorInvalidValue;
  const dim3 grid((M + kBM - 1) / kBM, (N + kBN - 1) / kBN);
  if (grid.y > 65535) return cudaErrorInvalidValue;
  count_launch();
  tc_gemm_kernel<<<grid, kThreads, kSmem, stream>>>(ma, mb, M, N, K, C, ldc, bias, act);
  return cudaGetLastError();
}

}  // namespace lmg
