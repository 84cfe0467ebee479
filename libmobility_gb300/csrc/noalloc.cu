// M.[F;T] for callers that cannot allocate device memory.
//
// Who needs this: a host program that owns every byte of device memory through
// its own pool and forbids other allocations (a framework with a fixed memory
// budget, a multi-tenant service with hard quotas), or a latency-critical loop
// that must not pay the device-wide synchronisation that cudaMalloc and
// cudaFree imply.  Such callers cannot use the handle API, which allocates its
// position copy, staging buffers and scratch on first use.
//
// This entry point allocates nothing.  The caller passes device buffers for
// every input and output.  The only scratch the pair kernel needs -- the
// per-split partial sums and the per-tile tickets of mdot_kernel's split-source
// reduction -- lives in the file-scope arrays below, which every GPU that loads
// the library holds until the process exits.  Their size caps how finely the
// sources of a target tile are split (a performance limit only); the particle
// count itself is limited to kMaxParticles.
//
// Set-up: every call, with its device current, looks up the device addresses
// of the arrays (cudaGetSymbolAddress: cheap, allocates nothing), so a device
// reset or another context on the device never leaves a stale address; the
// first call on a device also loads the library's device code there, so make
// that first call before any stream capture.  Every call shares the arrays and
// they keep the last call's contents: the tickets, which must start at zero,
// are cleared by each call on its stream; two calls whose work overlaps on the
// GPU (different streams, no ordering) race on the arrays and give wrong
// results.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.hpp"
#include "libmobility_gb300.h"
#include "mdot_launch.cuh"
#include "rpy_pair.cuh"

namespace {

constexpr size_t kScratchBytes = LMG_MDOT_NOALLOC_SCRATCH_BYTES;
constexpr size_t kScratchFloats = kScratchBytes / sizeof(float);
constexpr int kMaxTiles = 65536;
constexpr long long kMaxParticles = LMG_MDOT_NOALLOC_MAX_PARTICLES;

static __device__ __align__(256) float g_noalloc_partials[kScratchFloats];
static __device__ __align__(256) unsigned g_noalloc_tickets[kMaxTiles];

struct DeviceScratch {
  float *partials = nullptr;
  unsigned *tickets = nullptr;
  int sms = 0;
  bool ready = false;
};
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
DeviceScratch g_devices[kMaxDevices];

lmg_status fail(char *err, size_t len, lmg_status st, const char *msg) {
  if (err && len) {
    std::strncpy(err, msg, len - 1);
    err[len - 1] = 0;
  }
  return st;
}

lmg_status fail_cuda(char *err, size_t len, const char *what, cudaError_t e) {
  cudaGetLastError();
  char buf[256];
  std::snprintf(buf, sizeof(buf), "[libmobility_gb300] %s failed: %s", what,
                cudaGetErrorString(e));
  return fail(err, len, e == cudaErrorNoDevice ? LMG_ERR_NO_DEVICE : LMG_ERR_CUDA, buf);
}

// Once per device, with that device current: device addresses of the arrays.
lmg_status setup(DeviceScratch *&out, char *err, size_t len) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_cuda(err, len, "cudaGetDevice", e);
  if (dev < 0 || dev >= kMaxDevices)
    return fail(err, len, LMG_ERR_INVALID_ARGUMENT, "[libmobility_gb300] device ordinal too large");
  std::lock_guard<std::mutex> lock(g_mutex);
  DeviceScratch &d = g_devices[dev];
  e = cudaGetSymbolAddress((void **)&d.partials, g_noalloc_partials);
  if (e != cudaSuccess) return fail_cuda(err, len, "cudaGetSymbolAddress(partials)", e);
  e = cudaGetSymbolAddress((void **)&d.tickets, g_noalloc_tickets);
  if (e != cudaSuccess) return fail_cuda(err, len, "cudaGetSymbolAddress(tickets)", e);
  if (!d.ready) {
    e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail_cuda(err, len, "cudaDeviceGetAttribute", e);
    d.ready = true;
  }
  out = &d;
  return LMG_OK;
}

// 1: device memory of the current GPU (or managed), 0: host memory, -1:
// device memory of another GPU.
int on_device(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return lmg::classify_pointer(at.type, at.device, dev);
}

}  // namespace

extern "C" lmg_status lmg_mdot_noalloc_f32(const float *pos, const float *F, const float *T,
                                           float *U, float *W, int64_t numberParticles,
                                           int64_t NperBatch, int single_wall, double viscosity,
                                           double hydrodynamicRadius, int includeAngular,
                                           void *cuda_stream, char *err, size_t err_len) {
  if (err && err_len) err[0] = 0;
  const long long N = numberParticles;
  if (N < 1 || N > kMaxParticles) {
    char buf[200];
    std::snprintf(buf, sizeof(buf),
                  "[libmobility_gb300] lmg_mdot_noalloc_f32: numberParticles must be in [1, %lld]",
                  kMaxParticles);
    return fail(err, err_len, LMG_ERR_INVALID_ARGUMENT, buf);
  }
  const long long nper = NperBatch <= 0 ? N : NperBatch;
  if (N % nper != 0)
    return fail(err, err_len, LMG_ERR_INVALID_ARGUMENT,
                "[Mobility] Invalid batch parameters for NBody. If in doubt, use the defaults.");
  if (!(viscosity > 0) || !(hydrodynamicRadius > 0))
    return fail(err, err_len, LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] viscosity and hydrodynamicRadius must be positive");
  if (!pos || !U || (!F && !T))
    return fail(err, err_len, LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] lmg_mdot_noalloc_f32 needs pos, U and F and/or T");
  if (T && !includeAngular)
    return fail(err, err_len, LMG_ERR_INVALID_ARGUMENT,
                "The solver was configured without including angular velocities. Set "
                "includeAngular to true when initializing if you want to use torques");
  if (includeAngular && !W)
    return fail(err, err_len, LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] lmg_mdot_noalloc_f32 needs W when includeAngular is set");
  const void *bufs[5] = {pos, F, T, U, W};
  for (const void *b : bufs) {
    if (!b) continue;
    const int kind = on_device(b);
    if (kind < 0)
      return fail(err, err_len, LMG_ERR_INVALID_ARGUMENT,
                  "[libmobility_gb300] lmg_mdot_noalloc_f32: a buffer lives on another GPU "
                  "than the current one");
    if (kind == 0)
      return fail(err, err_len, LMG_ERR_INVALID_ARGUMENT,
                  "[libmobility_gb300] lmg_mdot_noalloc_f32 takes device buffers only (it "
                  "cannot stage host memory without allocating)");
  }

  DeviceScratch *d = nullptr;
  lmg_status st = setup(d, err, err_len);
  if (st != LMG_OK) return st;

  lmg::MdotShape s;
  s.geom = single_wall ? lmg::kWall : lmg::kOpen;
  s.ang = includeAngular != 0;
  s.has_f = F != nullptr;
  s.has_t = T != nullptr && s.ang;
  // launch plan of the handle API, with the source splitting capped so the
  // partial sums fit the static array
  lmg::MdotPlan plan;
  cudaError_t e = lmg::mdot_plan<float>(s, (int)N, (int)N, d->sms, 0, 0, plan);
  if (e != cudaSuccess) return fail_cuda(err, err_len, "mdot_plan", e);
  const int span = lmg::mdot_max_span((int)N, (int)nper, nullptr, 0, plan.threads * plan.tpt);
  e = lmg::mdot_plan<float>(s, (int)N, span, d->sms, plan.tpt, 0, plan);
  if (e != cudaSuccess) return fail_cuda(err, err_len, "mdot_plan", e);
  if (plan.nsplit > 1 && (plan.part_elems > kScratchFloats || plan.tiles > kMaxTiles)) {
    const int nc = s.ang ? 6 : 3;
    const size_t per_split = (size_t)plan.tiles * 2 * nc * plan.threads * plan.tpt;
    int fit = plan.tiles > kMaxTiles ? 1 : (int)(kScratchFloats / per_split);
    if (fit < 1) fit = 1;
    e = lmg::mdot_plan<float>(s, (int)N, span, d->sms, plan.tpt, fit, plan);
    if (e != cudaSuccess) return fail_cuda(err, err_len, "mdot_plan", e);
  }
  cudaStream_t stream = (cudaStream_t)cuda_stream;
  if (plan.nsplit > 1) {
    // the tickets must start at zero; a previous call may have been cut short
    e = cudaMemsetAsync(d->tickets, 0, plan.tiles * sizeof(unsigned), stream);
    if (e != cudaSuccess) return fail_cuda(err, err_len, "cudaMemsetAsync", e);
  }
  const double a = hydrodynamicRadius;
  lmg::MdotArgs<float> args{};
  args.pos = pos;
  args.F = F;
  args.T = s.has_t ? T : nullptr;
  args.U = U;
  args.W = s.ang ? W : nullptr;
  args.N = (int)N;
  args.nper = (int)nper;
  args.inv_a = (float)(1.0 / a);
  const double t0 = 1.0 / (6.0 * M_PI * viscosity * a);
  const double r0 = 1.0 / (8.0 * M_PI * viscosity * a * a * a);
  const double rt0 = 1.0 / (8.0 * M_PI * viscosity * a * a);
  args.k = lmg::make_pair_const<float>(t0, r0, rt0);
  args.kw = lmg::make_wall_const(t0, r0, rt0);
  args.part = plan.nsplit > 1 ? d->partials : nullptr;
  args.ticket = plan.nsplit > 1 ? d->tickets : nullptr;
  e = lmg::mdot_launch<float>(s, args, plan, stream);
  if (e != cudaSuccess) return fail_cuda(err, err_len, "mdot kernel launch", e);
  return LMG_OK;
}
