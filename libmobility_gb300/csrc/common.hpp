// Shared host-side definitions: status-carrying exception and CUDA checks.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstring>
#include <stdexcept>
#include <string>

#include "libmobility_gb300.h"

namespace lmg {

// Every failure inside the library is an Error; the C ABI turns it into an
// lmg_status and keeps the message for lmg_last_error.
struct Error : std::runtime_error {
  lmg_status code;
  Error(lmg_status c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void throw_cuda(cudaError_t e, const char *what) {
  cudaGetLastError();  // clear a sticky-free error so the handle stays usable
  lmg_status st = (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                      ? LMG_ERR_NO_DEVICE : LMG_ERR_CUDA;
  throw Error(st, std::string("[libmobility_gb300] CUDA error in ") + what + ": " +
                      cudaGetErrorString(e));
}

#define LMG_CUDA(call)                                  \
  do {                                                  \
    cudaError_t lmg_e_ = (call);                        \
    if (lmg_e_ != cudaSuccess) ::lmg::throw_cuda(lmg_e_, #call); \
  } while (0)

// Where a caller's buffer lives, from its pointer attributes: 0 host memory,
// 1 memory the current GPU's kernels may use directly (its own device memory,
// or managed memory), -1 device memory of another GPU (kernels would read it
// through peer access or fault, so it is refused).
inline int classify_pointer(int type, int ptr_device, int current_device) {
  if (type == cudaMemoryTypeManaged) return 1;
  if (type != cudaMemoryTypeDevice) return 0;
  return ptr_device == current_device ? 1 : -1;
}

// True for a device buffer of the current GPU, false for host memory; throws
// for device memory of another GPU.
inline bool device_pointer(const void *p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const int kind = classify_pointer(at.type, at.device, dev);
  if (kind < 0)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] a buffer lives on GPU " + std::to_string(at.device) +
                    ", not on the current GPU " + std::to_string(dev));
  return kind == 1;
}

// Named range on the profiler timeline (NVTX) for the lifetime of the object:
// the entry points and the phases of a solve (a no-op without a profiler).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// Owning device allocation that only grows.
template <class T> struct DeviceBuffer {
  T *ptr = nullptr;
  size_t count = 0;
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  ~DeviceBuffer() { release(); }
  T *ensure(size_t n) {
    if (n > count) {
      release();
      LMG_CUDA(cudaMalloc((void **)&ptr, (n ? n : 1) * sizeof(T)));
      count = n;
    }
    return ptr;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    count = 0;
  }
};

// Page-locked host staging allocation that only grows.
template <class T> struct PinnedBuffer {
  T *ptr = nullptr;
  size_t count = 0;
  PinnedBuffer() = default;
  PinnedBuffer(const PinnedBuffer &) = delete;
  PinnedBuffer &operator=(const PinnedBuffer &) = delete;
  ~PinnedBuffer() { release(); }
  T *ensure(size_t n) {
    if (n > count) {
      release();
      LMG_CUDA(cudaMallocHost((void **)&ptr, (n ? n : 1) * sizeof(T)));
      count = n;
    }
    return ptr;
  }
  void release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    count = 0;
  }
};

// Page-locked host allocation mapped into the device address space: small
// results written by kernels (Lanczos scalars) are read by the host after an
// event, without a copy operation.
template <class T> struct MappedBuffer {
  T *ptr = nullptr;
  T *dptr = nullptr;
  size_t count = 0;
  MappedBuffer() = default;
  MappedBuffer(const MappedBuffer &) = delete;
  MappedBuffer &operator=(const MappedBuffer &) = delete;
  ~MappedBuffer() { release(); }
  T *ensure(size_t n) {
    if (n > count) {
      release();
      LMG_CUDA(cudaHostAlloc((void **)&ptr, n * sizeof(T), cudaHostAllocMapped));
      LMG_CUDA(cudaHostGetDevicePointer((void **)&dptr, ptr, 0));
      std::memset(ptr, 0, n * sizeof(T));
      count = n;
    }
    return ptr;
  }
  T *device_ptr() const { return dptr; }
  void release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = dptr = nullptr;
    count = 0;
  }
};

}  // namespace lmg
