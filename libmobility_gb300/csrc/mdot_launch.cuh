// Launch planning and template dispatch for the all-pairs mobility kernel.
#pragma once
#include <algorithm>
#include <cstddef>
#include <vector>

#include "mdot.cuh"

namespace lmg {

struct MdotShape {
  int geom = kOpen;
  bool has_f = false;
  bool has_t = false;  // torques present AND includeAngular
  bool ang = false;    // includeAngular
};

// Occupancy-based plan: enough CTAs to cover every SM a few times, splitting
// the sources of each target tile when there are too few target tiles.
// `max_src_span` is the longest source range any target tile needs.
template <class R>
cudaError_t mdot_plan(const MdotShape &s, int N, int max_src_span, int num_sms, int force_tpt,
                      int force_split, MdotPlan &plan);

template <class R>
cudaError_t mdot_launch(const MdotShape &s, const MdotArgs<R> &args, const MdotPlan &plan,
                        cudaStream_t stream);

// Longest source range needed by a tile of `bt` consecutive targets (batches
// of nper, or the explicit batch table `sys_begin` of nsys batches), tiles
// starting at target t_lo and ending before t_hi (0: N).
inline int mdot_max_span(int N, int nper, const int *sys_begin_host, int nsys, int bt,
                         int t_lo = 0, int t_hi = 0) {
  if (t_hi <= 0) t_hi = N;
  auto sys_of = [&](int i) {
    if (!sys_begin_host) return i / nper;
    int lo = 0, hi = nsys;
    while (hi - lo > 1) {
      int mid = (lo + hi) / 2;
      if (sys_begin_host[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
  };
  auto start = [&](int s) { return sys_begin_host ? sys_begin_host[s] : s * nper; };
  auto end = [&](int s) {
    int e = sys_begin_host ? sys_begin_host[s + 1] : (s + 1) * nper;
    return e < N ? e : N;
  };
  if (!sys_begin_host && nper >= N) return N;
  int span = 0;
  for (int t0 = t_lo; t0 < t_hi; t0 += bt) {
    int last = std::min(t_hi, t0 + bt) - 1;
    span = std::max(span, end(sys_of(last)) - start(sys_of(t0)));
  }
  return span;
}

}  // namespace lmg
