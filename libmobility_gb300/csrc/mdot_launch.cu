// Template instantiation and dispatch of the all-pairs kernel.  Compiled once
// per precision (LMG_REAL = float | double) so the two halves build in
// parallel.
#include "launch_count.hpp"
#include "mdot_launch.cuh"

#ifndef LMG_REAL
#define LMG_REAL float
#endif

namespace lmg {

namespace {
constexpr int kThreads = 128;

template <class R, int GEOM, bool HF, bool HT, bool ANG, int TPT>
void *kernel_ptr() {
  return (void *)mdot_kernel<R, GEOM, HF, HT, ANG, TPT, kThreads>;
}

// kernel pointer for a shape; TPT in {1, 2}
template <class R>
void *select_kernel(const MdotShape &s, int tpt) {
#define LMG_SEL(G, HF, HT, A)                                              \
  if (s.geom == G && s.has_f == HF && s.has_t == HT && s.ang == A)         \
    return tpt == 2 ? kernel_ptr<R, G, HF, HT, A, 2>() : kernel_ptr<R, G, HF, HT, A, 1>();
  LMG_SEL(kOpen, true, false, false)
  LMG_SEL(kOpen, true, false, true)
  LMG_SEL(kOpen, false, true, true)
  LMG_SEL(kOpen, true, true, true)
  LMG_SEL(kWall, true, false, false)
  LMG_SEL(kWall, true, false, true)
  LMG_SEL(kWall, false, true, true)
  LMG_SEL(kWall, true, true, true)
#undef LMG_SEL
  return nullptr;
}
}  // namespace

template <class R>
cudaError_t mdot_plan(const MdotShape &s, int N, int max_src_span, int num_sms, int force_tpt,
                      int force_split, MdotPlan &plan) {
  plan = MdotPlan{};
  plan.threads = kThreads;
  // FP32: two targets per thread once there are enough targets to keep every
  // SM busy; FP64 stays at one (register pressure, the FP64 pipe is the limit)
  int tpt = 1;
  if (sizeof(R) == 4 && N >= 2 * kThreads * num_sms) tpt = 2;
  if (force_tpt == 1 || force_tpt == 2) tpt = force_tpt;
  plan.tpt = tpt;
  const int bt = kThreads * tpt;
  plan.tiles = (N + bt - 1) / bt;
  void *k = select_kernel<R>(s, tpt);
  if (!k) return cudaErrorInvalidValue;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, 0);
  if (e != cudaSuccess) return e;
  per_sm = std::max(per_sm, 1);
  // two waves of CTAs, and at least 32 CTAs per SM: kernels with few
  // resident CTAs (the wall kernel holds 5 per SM) otherwise lose a large
  // share of the last wave; measured on wall N = 16384 / 65536, 32 splits
  // beat 12 by 7 % and 3 by 10 %
  const long want = std::max(2L * num_sms * per_sm, 32L * num_sms);
  int nsplit = (int)std::max(1L, (want + plan.tiles - 1) / plan.tiles);
  // at least one full source tile per split
  const int max_split = std::max(1, max_src_span / kThreads);
  nsplit = std::min(nsplit, max_split);
  if (force_split > 0) nsplit = force_split;
  nsplit = std::min(nsplit, 65535);
  int chunk = (max_src_span + nsplit - 1) / nsplit;
  chunk = (chunk + kThreads - 1) / kThreads * kThreads;
  if (chunk <= 0) chunk = kThreads;
  nsplit = (max_src_span + chunk - 1) / chunk;
  if (nsplit < 1) nsplit = 1;
  plan.nsplit = nsplit;
  plan.chunk = chunk;
  const int nc = s.ang ? 6 : 3;
  plan.part_elems = nsplit > 1 ? (size_t)plan.tiles * nsplit * 2 * nc * bt : 0;
  plan.tickets = nsplit > 1 ? (size_t)plan.tiles : 0;
  return cudaSuccess;
}

template <class R>
cudaError_t mdot_launch(const MdotShape &s, const MdotArgs<R> &args, const MdotPlan &plan,
                        cudaStream_t stream) {
  void *k = select_kernel<R>(s, plan.tpt);
  if (!k) return cudaErrorInvalidValue;
  MdotArgs<R> a = args;
  a.chunk = plan.chunk;
  a.part_cap = plan.part_elems;
  a.ticket_cap = plan.tickets;
  dim3 grid(plan.tiles, plan.nsplit);
  void *params[] = {(void *)&a};
  count_launch();
  return cudaLaunchKernel(k, grid, dim3(plan.threads), params, 0, stream);
}

// this translation unit's bounds status (the checked build; 0 otherwise)
#define LMG_STATUS_FN(tag) bounds_status_mdot_##tag
#define LMG_STATUS_NAME(tag) LMG_STATUS_FN(tag)
unsigned long long LMG_STATUS_NAME(LMG_REAL)(bool reset) { return bounds_status_here(reset); }

template cudaError_t mdot_plan<LMG_REAL>(const MdotShape &, int, int, int, int, int, MdotPlan &);
template cudaError_t mdot_launch<LMG_REAL>(const MdotShape &, const MdotArgs<LMG_REAL> &,
                                           const MdotPlan &, cudaStream_t);

}  // namespace lmg
