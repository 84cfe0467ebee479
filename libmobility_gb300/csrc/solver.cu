// Numeric half of the solver, templated on the precision `real`.
//
//   setPositions   solvers/NBody/mobility.h:116-162
//   Mdot           mobility.h:166-182 -> NbodyRPY.cu:254-287
//   sqrtMdotW      MobilityInterface.h:132-188 + lanczos.h:43-58 +
//                  LanczosAlgorithm.cu:173-232
//   divM           mobility.h:184-236 + random_finite_differences.h:30-63
//   clean          MobilityInterface.h:220-223
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <tuple>
#include <type_traits>
#include <vector>

#include "krylov.cuh"
#include "launch_count.hpp"
#include "mdot_launch.cuh"
#include "mdot_sym.cuh"
#include "precond.cuh"
#include "solver.hpp"

namespace lmg {

namespace {

bool is_device_ptr(const void *p) { return device_pointer(p); }

template <class R>
__global__ void shift_min_kernel(R *pos, int N, R height, double *partials, unsigned *ticket,
                                 double *out_min) {
  double v = 1e300;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    R z = pos[3 * i + 2];
    if (height != R(0)) {
      z = z - height;
      pos[3 * i + 2] = z;
    }
    v = fmin(v, (double)z);
  }
  // min reduction through the shared grid machinery: negate and take max as sum? use block min
  __shared__ double red[kRedThreads / 32];
  __shared__ bool last;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int w = 1; w < (int)(blockDim.x / 32); w++) m = fmin(m, red[w]);
    __stcg(partials + blockIdx.x, m);
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double m = 1e300;
    for (int b = 0; b < (int)gridDim.x; b++) m = fmin(m, __ldcg(partials + b));
    *out_min = m;
    *ticket = 0u;
  }
}

// pos_delta = pos + s * noise  (random finite differences)
template <class R>
__global__ void displace_kernel(const R *pos, const R *noise, R *out, size_t n, R s) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    out[e] = pos[e] + s * noise[e];
}

// out += c * (a - b)
template <class R>
__global__ void add_scaled_diff_kernel(R *out, const R *a, const R *b, size_t n, R c) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    out[e] += c * (a[e] - b[e]);
}

}  // namespace

template <class R> class Solver final : public SolverBase {
 public:
  Solver(Periodicity x, Periodicity y, Periodicity z) : SolverBase(x, y, z) {}
  ~Solver() override {
    release_all();
    for (auto &e : ev_iter_)
      if (e) cudaEventDestroy(e);
    for (auto &e : ev_prod_)
      if (e) cudaEventDestroy(e);
    for (auto &e : ev_check_)
      if (e) cudaEventDestroy(e);
    if (ev_side_) cudaEventDestroy(ev_side_);
    for (auto &e : ev_phase_)
      if (e) cudaEventDestroy(e);
    for (auto &e : ev_pre_)
      if (e) cudaEventDestroy(e);
    if (side_) cudaStreamDestroy(side_);
  }

  const char *precision() const override { return sizeof(R) == 4 ? "float" : "double"; }

  void set_positions(const void *pos, size_t n) override;
  void mdot(const void *F, size_t nF, const void *T, size_t nT, void *U, size_t nU, void *W,
            size_t nW) override;
  void mdot_rows(int64_t row_begin, int64_t row_end, const void *F, size_t nF, const void *T,
                 size_t nT, void *U, size_t nU, void *W, size_t nW) override;
  void sqrt_mdot_w(void *U, size_t nU, void *W, size_t nW, double prefactor, const void *dW,
                   size_t ndW, int *iterations, double *residual) override;
  void div_m(void *U, size_t nU, void *W, size_t nW, double prefactor) override;
  void clean() override;
  void set_preconditioner(const std::string &kind, const float *params, size_t n) override;

 private:
  // device state
  DeviceBuffer<R> pos_, pos_tmp_;
  DeviceBuffer<R> in_stage_, out_stage_;  // host<->device staging of user arrays
  PinnedBuffer<R> pin_;                   // pinned bounce buffer
  DeviceBuffer<R> part_;                  // Mdot split partials
  DeviceBuffer<unsigned> tickets_;        // Mdot split tickets (self-resetting)
  DeviceBuffer<double> red_part_;         // reduction partials
  DeviceBuffer<unsigned> red_ticket_;     // reduction ticket (self-resetting)
  DeviceBuffer<double> dmin_;
  // Lanczos
  DeviceBuffer<R> V_, w_, y_, ybuf_, z_;
  DeviceBuffer<KrylovScalars> sc_;
  DeviceBuffer<double> cvec_;
  MappedBuffer<double> mirror_;       // (alpha_i, beta_i) pairs + err, device-written
  MappedBuffer<double> hc_;           // host T^{1/2} e1, read by the check kernel (2 slots)
  DeviceBuffer<double> quad_g_;       // node sums of the device square root
  std::vector<double> ql_work_;       // host QL work arrays
  std::vector<double2> rot_cs_;       // host QL rotation log
  std::vector<int> rot_idx_;
  PinnedBuffer<double> h_dbl_;
  cudaStream_t side_ = nullptr;       // high-priority stream for per-check work
  // iteration j completes ev_iter_[j % kIterEvents] (a ring: up to kMaxLookahead
  // iterations run ahead of the check being evaluated)
  static constexpr int kMaxLookahead = 4, kIterEvents = kMaxLookahead + 2;
  // ev_prod_ likewise the end of iteration j's matrix-vector product;
  // ev_check_[i & 1]: the check of iteration i done (two checks in flight)
  cudaEvent_t ev_iter_[kIterEvents] = {}, ev_prod_[kIterEvents] = {}, ev_check_[2] = {},
              ev_side_ = nullptr;
  // phase timing: per iteration j, [5j, 5j+1] bracket the operator, [5j+1,
  // 5j+2] the vector updates and [5j+3, 5j+4] the check; ev_pre_ the
  // preconditioner build and P solve (created on the first timed solve)
  std::vector<cudaEvent_t> ev_phase_;
  cudaEvent_t ev_pre_[4] = {nullptr, nullptr, nullptr, nullptr};
  void ensure_phase_events();
  // RFD
  DeviceBuffer<R> rfd_noise_, rfd_pos_, rfd_mp_, rfd_mm_;
  // learned preconditioner
  bool prec_on_ = false;
  bool prec_dirty_ = true;
  int prec_k_ = 16;  // neighbours per row of P, from the network's parameter count
  PrecLayout prec_layout_;
  // trained with t0 = 1: M^{-1/2} scales as t0^{-1/2}
  float prec_scale() const { return (float)(1.0 / std::sqrt(t0_)); }
  PrecWork prec_work_;
  DeviceBuffer<float> prec_params_;
  DeviceBuffer<uint16_t> prec_blocks_;  // P blocks in half precision, unit scale
  DeviceBuffer<int> prec_nb_;
  KnnScratch knn_scratch_;
  DeviceBuffer<R> pt_, pu_, bx_, br_, brh_, bp_, bv_, bs_, bt_;  // operator and BiCGSTAB vectors
  DeviceBuffer<float> ppad_;  // float4-padded work array of the P^T product
  int num_sms_ = 0;
  int step_per_sm_ = 0;  // resident krylov_step_kernel blocks per SM
  int step_ctas_ = -1;   // CTAs of the cluster of krylov_step_cluster_kernel (0: none fits)
  bool tickets_zeroed_ = false;
  std::map<long, MdotPlan> plans_;
  // symmetric open-space product (FP32): plans with their device tables,
  // partial sums and barrier counts, and the flag a barrier that timed out
  // raises
  struct SymState {
    SymPlan plan;
    DeviceBuffer<int4> pairs, warps;
    DeviceBuffer<int> pseg;
    // arrival count of the kernel's grid barrier: one per plan, so every
    // launch that uses it has the same block count
    DeviceBuffer<unsigned long long> count;
    DeviceBuffer<float> part;  // partial sums (slots nobody writes stay zero)
  };
  std::map<std::tuple<int, int, int, int>, std::unique_ptr<SymState>> sym_plans_;
  MappedBuffer<int> sym_err_;
  bool mdot_sym(const R *pos, const R *F, R *U);

  void release_all();
  int sms();
  int vec_blocks(size_t n) {
    size_t b = (n + kRedThreads - 1) / kRedThreads;
    size_t cap = (size_t)sms() * 4;
    return (int)std::max<size_t>(1, std::min(b, cap));
  }
  void ensure_reduction(int blocks);
  size_t red_half() const { return red_part_.count / 2; }
  void ensure_side();
  const R *device_input(const void *p, size_t n, R *stage);
  // M . [F;T] on device buffers: the Lanczos matvec and the RFD probes; with
  // row_end > 0 only targets [row_begin, row_end), written from row 0 of U, W
  void mdot_device(const R *pos, const R *F, const R *T, R *U, R *W, int row_begin = 0,
                   int row_end = 0);
  void mdot_rows_device(const R *pos, const R *F, const R *T, R *U, R *W, int row_begin,
                        int row_end);
  std::map<std::tuple<int, int, int, int, int>, MdotPlan> row_plans_;
  int lanczos(const R *z, R *y, size_t n, double tol, double *residual);
  bool prec_active() const;
  void prec_build();
  void apply_operator(const R *v, R *out);  // M v, or P M P^T v with the preconditioner
  int solve_p(const R *b, R *x);             // P x = b (BiCGSTAB), returns iterations
};

template <class R> int Solver<R>::sms() {
  if (!num_sms_) {
    int dev = 0;
    LMG_CUDA(cudaGetDevice(&dev));
    LMG_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
  }
  return num_sms_;
}

template <class R> void Solver<R>::release_all() {
  pos_.release(); pos_tmp_.release(); in_stage_.release(); out_stage_.release(); pin_.release();
  part_.release(); tickets_.release(); red_part_.release(); red_ticket_.release(); dmin_.release();
  V_.release(); w_.release(); y_.release(); ybuf_.release(); z_.release(); sc_.release();
  cvec_.release(); mirror_.release(); hc_.release(); quad_g_.release(); ql_work_ = {}; rot_cs_ = {}; rot_idx_ = {};
  h_dbl_.release(); rfd_noise_.release(); rfd_pos_.release(); rfd_mp_.release(); rfd_mm_.release();
  plans_.clear();
  row_plans_.clear();
  sym_plans_.clear();
  sym_err_.release();
  tickets_zeroed_ = false;
}

template <class R> void Solver<R>::ensure_reduction(int blocks) {
  // two halves: the solver stream and the side stream reduce independently
  red_part_.ensure((size_t)8 * std::max(blocks, 1024));
  if (!red_ticket_.ptr) {
    // [0] solver-stream ticket, [1] side-stream ticket, [3] min ticket,
    // [4..5] grid barrier of the fused Lanczos step
    red_ticket_.ensure(8);
    LMG_CUDA(cudaMemsetAsync(red_ticket_.ptr, 0, 8 * sizeof(unsigned), stream()));
  }
}

template <class R> void Solver<R>::set_positions(const void *pos, size_t n) {
  NvtxRange nvtx_range_("lmg setPositions");
  if (n % 3 != 0)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libMobility] The input arrays for positions, forces, and torques must each "
                "have total size 3*N.");
  const int64_t N = (int64_t)(n / 3);
  if (N > (int64_t)(1 << 30))
    throw Error(LMG_ERR_INVALID_ARGUMENT, "[libmobility_gb300] too many particles");
  const int64_t nb = nbatch_ < 0 ? 1 : nbatch_;
  const int64_t np = nper_ < 0 ? N : nper_;
  if (nb * np != N)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[Mobility] Invalid batch parameters for NBody. If in doubt, use the defaults.");
  const char *below =
      "[Mobility] The center of a particle has fallen below the wall. Check your "
      "configuration and forces to ensure particle centers stay above the wall.";
  if (N == 0) {
    N_ = 0;
    return;
  }
  const bool dev = is_device_ptr(pos);
  if (!dev) {
    // host input: shift and check on the host (no GPU needed to reject it)
    const R *p = static_cast<const R *>(pos);
    std::vector<R> tmp(p, p + n);
    if (wall_) {
      R zmin = std::numeric_limits<R>::max();
      for (int64_t i = 0; i < N; i++) {
        if (wall_height_ != 0) tmp[3 * i + 2] = tmp[3 * i + 2] - (R)wall_height_;
        zmin = std::min(zmin, tmp[3 * i + 2]);
      }
      if (zmin < 0) throw Error(LMG_ERR_BELOW_WALL, below);
    }
    R *d = pos_tmp_.ensure(n);
    R *h = pin_.ensure(n);
    std::memcpy(h, tmp.data(), n * sizeof(R));
    LMG_CUDA(cudaMemcpyAsync(d, h, n * sizeof(R), cudaMemcpyHostToDevice, stream()));
    LMG_CUDA(cudaStreamSynchronize(stream()));
  } else {
    R *d = pos_tmp_.ensure(n);
    LMG_CUDA(cudaMemcpyAsync(d, pos, n * sizeof(R), cudaMemcpyDeviceToDevice, stream()));
    if (wall_) {
      const int blocks = std::min<int>((int)((N + kRedThreads - 1) / kRedThreads), sms() * 4);
      ensure_reduction(blocks);
      dmin_.ensure(1);
      shift_min_kernel<R><<<blocks, kRedThreads, 0, stream()>>>(
          d, (int)N, (R)wall_height_, red_part_.ptr, red_ticket_.ptr + 3, dmin_.ptr);
      count_launch();
      LMG_CUDA(cudaGetLastError());
      double *hm = h_dbl_.ensure(1);
      LMG_CUDA(cudaMemcpyAsync(hm, dmin_.ptr, sizeof(double), cudaMemcpyDeviceToHost, stream()));
      LMG_CUDA(cudaStreamSynchronize(stream()));
      if (*hm < 0) throw Error(LMG_ERR_BELOW_WALL, below);
    }
  }
  std::swap(pos_.ptr, pos_tmp_.ptr);
  std::swap(pos_.count, pos_tmp_.count);
  N_ = N;
  prec_dirty_ = true;
}

// Device pointer for a user array: used in place when it is device memory,
// otherwise copied through the pinned bounce buffer into `stage`.
template <class R> const R *Solver<R>::device_input(const void *p, size_t n, R *stage) {
  if (!p || n == 0) return nullptr;
  if (is_device_ptr(p)) return static_cast<const R *>(p);
  R *h = pin_.ensure(n);
  std::memcpy(h, p, n * sizeof(R));
  LMG_CUDA(cudaMemcpyAsync(stage, h, n * sizeof(R), cudaMemcpyHostToDevice, stream()));
  // the bounce buffer is reused by the next staging: wait for this copy
  LMG_CUDA(cudaStreamSynchronize(stream()));
  return stage;
}

template <class R>
void Solver<R>::mdot_device(const R *pos, const R *F, const R *T, R *U, R *W, int row_begin,
                            int row_end) {
  const bool rows = row_end > 0 && !(row_begin == 0 && row_end == (int)N_);
  if (rows) {
    mdot_rows_device(pos, F, T, U, W, row_begin, row_end);
    return;
  }
  MdotShape s;
  s.geom = wall_ ? kWall : kOpen;
  s.ang = ang_;
  s.has_f = F != nullptr;
  s.has_t = T != nullptr && ang_;
  const int N = (int)N_;
  const int nper = batch_size();
  if (!s.has_f && !s.has_t) {
    if (U) LMG_CUDA(cudaMemsetAsync(U, 0, 3 * (size_t)N * sizeof(R), stream()));
    if (W) LMG_CUDA(cudaMemsetAsync(W, 0, 3 * (size_t)N * sizeof(R), stream()));
    return;
  }
  if (s.geom == kOpen && s.has_f && !s.has_t && !s.ang && mdot_sym(pos, F, U)) return;
  const int ftpt = g_force_tpt.load(), fsplit = g_force_split.load();
  const long key = ((long)N << 30) | ((long)fsplit << 10) | (ftpt << 8) | (s.geom << 3) |
                   (s.has_f << 2) | (s.has_t << 1) | s.ang;
  auto it = plans_.find(key);
  if (it == plans_.end() || it->second.tiles == 0) {
    MdotPlan plan;
    // span depends on the tile width, which the plan picks: plan twice
    LMG_CUDA(mdot_plan<R>(s, N, N, sms(), ftpt, fsplit, plan));
    const int span = mdot_max_span(N, nper, nullptr, 0, plan.threads * plan.tpt);
    LMG_CUDA(mdot_plan<R>(s, N, span, sms(), plan.tpt, fsplit, plan));
    it = plans_.insert_or_assign(key, plan).first;
  }
  const MdotPlan &plan = it->second;
  if (plan.nsplit > 1) {
    part_.ensure(plan.part_elems);
    if (tickets_.count < plan.tickets || !tickets_zeroed_) {
      tickets_.ensure(std::max(plan.tickets, tickets_.count));
      LMG_CUDA(cudaMemsetAsync(tickets_.ptr, 0, tickets_.count * sizeof(unsigned), stream()));
      tickets_zeroed_ = true;
    }
  }
  MdotArgs<R> a{};
  a.pos = pos;
  a.F = F;
  a.T = s.has_t ? T : nullptr;
  a.U = U;
  a.W = ang_ ? W : nullptr;
  a.sys_begin = nullptr;
  a.nsys = 0;
  a.N = N;
  a.nper = nper;
  a.inv_a = (R)(1.0 / a_);
  a.k = make_pair_const<R>(t0_, r0_, rt0_);
  a.kw = make_wall_const(t0_, r0_, rt0_);
  a.part = part_.ptr;
  a.ticket = tickets_.ptr;
  LMG_CUDA(mdot_launch<R>(s, a, plan, stream()));
}

// Targets [row_begin, row_end) only, with the tiled kernel: every source of
// a target's batch counts, results from row 0 of U and W.
template <class R>
void Solver<R>::mdot_rows_device(const R *pos, const R *F, const R *T, R *U, R *W,
                                 int row_begin, int row_end) {
  MdotShape s;
  s.geom = wall_ ? kWall : kOpen;
  s.ang = ang_;
  s.has_f = F != nullptr;
  s.has_t = T != nullptr && ang_;
  const int N = (int)N_, rows = row_end - row_begin;
  if (!s.has_f && !s.has_t) {
    if (U) LMG_CUDA(cudaMemsetAsync(U, 0, 3 * (size_t)rows * sizeof(R), stream()));
    if (W) LMG_CUDA(cudaMemsetAsync(W, 0, 3 * (size_t)rows * sizeof(R), stream()));
    return;
  }
  const int shape = (s.geom << 3) | (s.has_f << 2) | (s.has_t << 1) | (int)s.ang;
  const auto key = std::make_tuple(N, row_begin, row_end, batch_size(), shape);
  auto it = row_plans_.find(key);
  if (it == row_plans_.end()) {
    MdotPlan plan;
    LMG_CUDA(mdot_plan<R>(s, rows, N, sms(), 0, 0, plan));
    const int span = mdot_max_span(N, batch_size(), nullptr, 0, plan.threads * plan.tpt,
                                   row_begin, row_end);
    LMG_CUDA(mdot_plan<R>(s, rows, span, sms(), plan.tpt, 0, plan));
    it = row_plans_.insert_or_assign(key, plan).first;
  }
  const MdotPlan &plan = it->second;
  if (plan.nsplit > 1) {
    part_.ensure(plan.part_elems);
    if (tickets_.count < plan.tickets || !tickets_zeroed_) {
      tickets_.ensure(std::max(plan.tickets, tickets_.count));
      LMG_CUDA(cudaMemsetAsync(tickets_.ptr, 0, tickets_.count * sizeof(unsigned), stream()));
      tickets_zeroed_ = true;
    }
  }
  MdotArgs<R> a{};
  a.pos = pos;
  a.F = F;
  a.T = s.has_t ? T : nullptr;
  a.U = U;
  a.W = ang_ ? W : nullptr;
  a.N = N;
  a.nper = batch_size();
  a.tgt_begin = row_begin;
  a.tgt_end = row_end;
  a.inv_a = (R)(1.0 / a_);
  a.k = make_pair_const<R>(t0_, r0_, rt0_);
  a.kw = make_wall_const(t0_, r0_, rt0_);
  a.part = part_.ptr;
  a.ticket = tickets_.ptr;
  LMG_CUDA(mdot_launch<R>(s, a, plan, stream()));
}

template <class R>
void Solver<R>::mdot_rows(int64_t row_begin, int64_t row_end, const void *F, size_t nF,
                          const void *T, size_t nT, void *U, size_t nU, void *W, size_t nW) {
  NvtxRange nvtx_range_("lmg Mdot rows");
  if (!F) nF = 0;
  if (!T) nT = 0;
  if (!U) nU = 0;
  if (!W) nW = 0;
  check_positions_set("Mdot");
  if (row_begin < 0 || row_end <= row_begin || row_end > N_)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] rows must satisfy 0 <= row_begin < row_end <= N");
  check_mdot_args(nF, nT, 0, 0);
  const size_t n3 = 3 * (size_t)N_, r3 = 3 * (size_t)(row_end - row_begin);
  if ((nU && nU != r3) || (nW && nW != r3))
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] row outputs must have 3 * (row_end - row_begin) values");
  R *stage = in_stage_.ensure(2 * n3);
  out_stage_.ensure(2 * n3);
  pin_.ensure(2 * n3);
  const R *Fd = device_input(F, nF, stage);
  const R *Td = device_input(T, nT, stage + n3);
  const bool u_dev = nU && is_device_ptr(U);
  const bool w_dev = nW && is_device_ptr(W);
  R *Ud = nU ? (u_dev ? static_cast<R *>(U) : out_stage_.ensure(2 * n3)) : nullptr;
  R *Wd = nW ? (w_dev ? static_cast<R *>(W) : out_stage_.ensure(2 * n3) + n3) : nullptr;
  mdot_rows_device(pos_.ptr, Fd, Td, Ud, Wd, (int)row_begin, (int)row_end);
  LMG_CUDA(cudaGetLastError());
  if ((nU && !u_dev) || (nW && !w_dev)) {
    R *h = pin_.ensure(2 * n3);
    if (nU && !u_dev)
      LMG_CUDA(cudaMemcpyAsync(h, Ud, r3 * sizeof(R), cudaMemcpyDeviceToHost, stream()));
    if (nW && !w_dev)
      LMG_CUDA(cudaMemcpyAsync(h + n3, Wd, r3 * sizeof(R), cudaMemcpyDeviceToHost, stream()));
    LMG_CUDA(cudaStreamSynchronize(stream()));
    if (nU && !u_dev) std::memcpy(U, h, r3 * sizeof(R));
    if (nW && !w_dev) std::memcpy(W, h + n3, r3 * sizeof(R));
  }
}

// U = M F with the symmetric open-space kernel (FP32, forces only, no
// angular part): returns false where that kernel does not apply.
template <class R> bool Solver<R>::mdot_sym(const R *pos, const R *F, R *U) {
  if constexpr (!std::is_same_v<R, float>) {
    return false;
  } else {
    if (g_sym_mode.load() != 0 || U == nullptr) return false;
    if ((reinterpret_cast<uintptr_t>(F) | reinterpret_cast<uintptr_t>(pos)) & 15) return false;
    const int N = (int)N_;
    const int warps = g_sym_warps.load();
    const auto key = std::make_tuple(N, batch_size(), warps, g_sym_variant.load());
    auto it = sym_plans_.find(key);
    if (it == sym_plans_.end()) {
      auto st = std::make_unique<SymState>();
      const cudaError_t e = mdot_sym_plan(N, batch_size(), sms(), warps, st->plan);
      if (e != cudaSuccess && e != cudaErrorNotSupported) LMG_CUDA(e);
      if (e != cudaSuccess) {
        st->plan.grid = 0;
      } else {
        const SymPlan &p = st->plan;
        auto up = [&](auto &buf, const auto &v) {
          buf.ensure(v.size());
          LMG_CUDA(cudaMemcpyAsync(buf.ptr, v.data(), v.size() * sizeof(v[0]),
                                   cudaMemcpyHostToDevice, stream()));
        };
        up(st->pairs, p.pairs);
        up(st->pseg, p.pseg);
        up(st->warps, p.warps);
        st->count.ensure(1);
        LMG_CUDA(cudaMemsetAsync(st->count.ptr, 0, sizeof(unsigned long long), stream()));
        st->part.ensure(p.part_elems);
        LMG_CUDA(cudaMemsetAsync(st->part.ptr, 0, p.part_elems * sizeof(float), stream()));
        // the host tables must outlive the copies
        LMG_CUDA(cudaStreamSynchronize(stream()));
      }
      it = sym_plans_.insert_or_assign(key, std::move(st)).first;
    }
    const SymState &st = *it->second;
    const SymPlan &p = st.plan;
    if (p.grid <= 0) return false;
    if (!sym_err_.ptr) sym_err_.ensure(1);
    if (*(volatile int *)sym_err_.ptr) {
      // a barrier wait ran out in an earlier launch: arrival counts are
      // inconsistent, start them afresh
      LMG_CUDA(cudaStreamSynchronize(stream()));
      for (auto &kv : sym_plans_)
        if (kv.second->count.ptr)
          LMG_CUDA(cudaMemsetAsync(kv.second->count.ptr, 0, sizeof(unsigned long long),
                                   stream()));
      *(volatile int *)sym_err_.ptr = 0;
      throw Error(LMG_ERR_TIMEOUT,
                  "[libmobility_gb300] Mdot: grid barrier of the symmetric kernel timed out");
    }
    const PairConst<float> k = make_pair_const<float>(t0_, r0_, rt0_);
    SymTables tab;
    tab.pairs = st.pairs.ptr;
    tab.pseg = st.pseg.ptr;
    tab.warps = st.warps.ptr;
    LMG_CUDA(mdot_sym_launch(p, tab, pos, F, U, (float)(1.0 / a_), k, st.part.ptr, st.count.ptr,
                             sym_err_.device_ptr(), stream()));
    return true;
  }
}

template <class R>
void Solver<R>::mdot(const void *F, size_t nF, const void *T, size_t nT, void *U, size_t nU,
                     void *W, size_t nW) {
  NvtxRange nvtx_range_("lmg Mdot");
  if (!F) nF = 0;
  if (!T) nT = 0;
  if (!U) nU = 0;
  if (!W) nW = 0;
  check_mdot_args(nF, nT, nU, nW);
  const size_t n3 = 3 * (size_t)N_;
  R *stage = in_stage_.ensure(2 * n3);
  out_stage_.ensure(2 * n3);
  pin_.ensure(2 * n3);
  const R *Fd = device_input(F, nF, stage);
  const R *Td = device_input(T, nT, stage + n3);
  const bool u_dev = nU && is_device_ptr(U);
  const bool w_dev = nW && is_device_ptr(W);
  R *Ud = nU ? (u_dev ? static_cast<R *>(U) : out_stage_.ensure(2 * n3)) : nullptr;
  R *Wd = nW ? (w_dev ? static_cast<R *>(W) : out_stage_.ensure(2 * n3) + n3) : nullptr;
  mdot_device(pos_.ptr, Fd, Td, Ud, Wd);
  LMG_CUDA(cudaGetLastError());
  if ((nU && !u_dev) || (nW && !w_dev)) {
    R *h = pin_.ensure(2 * n3);
    if (nU && !u_dev)
      LMG_CUDA(cudaMemcpyAsync(h, Ud, n3 * sizeof(R), cudaMemcpyDeviceToHost, stream()));
    if (nW && !w_dev)
      LMG_CUDA(cudaMemcpyAsync(h + n3, Wd, n3 * sizeof(R), cudaMemcpyDeviceToHost, stream()));
    LMG_CUDA(cudaStreamSynchronize(stream()));
    if (nU && !u_dev) std::memcpy(U, h, n3 * sizeof(R));
    if (nW && !w_dev) std::memcpy(W, h + n3, n3 * sizeof(R));
  }
}

template <class R> void Solver<R>::ensure_side() {
  if (!side_) {
    int lo = 0, hi = 0;
    LMG_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    LMG_CUDA(cudaStreamCreateWithPriority(&side_, cudaStreamNonBlocking, hi));
    for (auto &e : ev_iter_) LMG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto &e : ev_prod_) LMG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto &e : ev_check_) LMG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    LMG_CUDA(cudaEventCreateWithFlags(&ev_side_, cudaEventDisableTiming));
  }
}

namespace {
// vectors up to this length take the check kernel with four threads per element
constexpr size_t kCheckShortN = 65536;

template <class R> const void *step_cluster_fn(int ept) {
  switch (ept) {
    case 1: return (const void *)krylov_step_cluster_kernel<R, 1>;
    case 2: return (const void *)krylov_step_cluster_kernel<R, 2>;
    case 4: return (const void *)krylov_step_cluster_kernel<R, 4>;
    case 8: return (const void *)krylov_step_cluster_kernel<R, 8>;
    default: return (const void *)krylov_step_cluster_kernel<R, 0>;
  }
}

cudaLaunchConfig_t cluster_config(int ctas, int threads, cudaStream_t st,
                                  cudaLaunchAttribute *at) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ctas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cfg;
}

// The largest cluster (16, 8, 4, 2 CTAs of kClusterThreads) of the Krylov
// step that fits on the current GPU; 0 if none does.
template <class R> int step_cluster_ctas() {
  const int epts[] = {0, 1, 2, 4, 8};
  for (int e : epts)
    LMG_CUDA(cudaFuncSetAttribute(step_cluster_fn<R>(e),
                                  cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  for (int c : {16, 8, 4, 2}) {
    cudaLaunchAttribute at[1];
    const cudaLaunchConfig_t cfg = cluster_config(c, kClusterThreads, nullptr, at);
    int clusters = 0;
    bool ok = true;
    for (int e : epts) {
      if (cudaOccupancyMaxActiveClusters(&clusters, step_cluster_fn<R>(e), &cfg) != cudaSuccess ||
          clusters < 1) {
        ok = false;
        (void)cudaGetLastError();
        break;
      }
    }
    if (ok) return c;
  }
  return 0;
}

// One Krylov step as one cluster: elements a thread keeps in registers from
// the vector length (up to 8 in FP32, 4 in FP64; beyond that streamed).
template <class R>
cudaError_t launch_step_cluster(int ctas, int cta_threads, R *w, const R *vi, const R *vprev,
                                R *vnext, size_t n, int i, KrylovScalars *sc, double *host_ab,
                                cudaStream_t st) {
  const size_t threads = (size_t)ctas * cta_threads;
  const size_t per = (n + threads - 1) / threads;
  const int max_ept = sizeof(R) == 4 ? 8 : 4;
  int ept = 0;
  for (int e : {1, 2, 4, 8})
    if (ept == 0 && e <= max_ept && per <= (size_t)e) ept = e;
  cudaLaunchAttribute at[1];
  const cudaLaunchConfig_t cfg = cluster_config(ctas, cta_threads, st, at);
  void *args[] = {&w, (void *)&vi, (void *)&vprev, &vnext, &n, &i, &sc, &host_ab};
  count_launch();
  return cudaLaunchKernelExC(&cfg, step_cluster_fn<R>(ept), args);
}
}  // namespace

// Lanczos to tolerance (LanczosAlgorithm.cu:173-200); returns the iteration
// index at convergence and leaves y = sqrt(M) z in *y_out.
//
// Schedule per iteration i on the solver stream S: matvec, alpha, beta (which
// also writes alpha_i, beta_i to mapped host memory), next -> event I_i.  The
// GPU is kept ahead of the host: iterations up to i+3 (batches of up to 8192
// particles, else i+1) are issued before the host handles the convergence
// check of iteration i.  A check (every i >= k, the adaptive start of
// LanczosAlgorithm.cu:179-184, or every i with a callback) waits for I_i,
// takes the FP64 T^{1/2} e1 on the host while the GPU runs ahead, then on
// the high-priority side stream P computes y_i = |z| V c_i and
// |y_i - y_{i-1}| / |y_{i-1}| into mapped host memory.  That error is read
// one check late (after check i+1 is launched), so the host never waits on
// the check it has just launched; iterations issued past the stopping step
// are discarded.  At the first check of a solve there is no y_{i-1}; its
// error counts as infinite (the reference compares against a zero or stale
// buffer there).
template <class R> void Solver<R>::ensure_phase_events() {
  if (ev_phase_.empty()) {
    ev_phase_.assign(5 * (kMaxLanczosIterations + 1), nullptr);
    for (auto &e : ev_phase_) LMG_CUDA(cudaEventCreate(&e));
  }
  for (auto &e : ev_pre_)
    if (!e) LMG_CUDA(cudaEventCreate(&e));
}

template <class R>
int Solver<R>::lanczos(const R *z, R *y_out, size_t n, double tol, double *residual) {
  NvtxRange nvtx_range_("lmg Lanczos");
  const int limit = hard_limit_;
  const int blocks = vec_blocks(n);
  ensure_reduction(blocks);
  ensure_side();
  R *V = V_.ensure((size_t)(limit + 1) * n);
  R *w = w_.ensure(n);
  R *yb = ybuf_.ensure(2 * n);
  KrylovScalars *sc = sc_.ensure(1);
  double *cdev = cvec_.ensure(2 * kMaxLanczosIterations);
  // [2i] alpha_i, [2i+1] beta_i, [512] err, [516] barrier timeout, [520]
  // device square root fell back
  double *mir = mirror_.ensure(2 * 256 + 16);
  double *mir_dev = mirror_.device_ptr();
  double *hc = hc_.ensure(2 * kMaxLanczosIterations);
  double *quad_g = quad_g_.ensure((size_t)kQuadThreads * 2 * kQuadThreads);
  const int rot_cap = 24 * limit * limit + 1024;
  if ((int)rot_cs_.size() < rot_cap) {
    rot_cs_.resize(rot_cap);
    rot_idx_.resize(rot_cap);
  }
  ql_work_.resize(3 * 256 + 18 * 256);  // QL arrays, then the quadrature's work
  RotLog log{rot_cs_.data(), rot_idx_.data(), rot_cap};
  cudaStream_t st = stream();
  cudaStream_t sd = side_;
  unsigned *tk = red_ticket_.ptr, *tk_side = red_ticket_.ptr + 1, *bar = red_ticket_.ptr + 4;
  double *rp = red_part_.ptr, *rp_side = red_part_.ptr + red_half();
  // the fused vector step is a cooperative launch: every block resident
  if (!step_per_sm_) {
    LMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&step_per_sm_, krylov_step_kernel<R>,
                                                           kRedThreads, 0));
    if (step_per_sm_ < 1)
      throw Error(LMG_ERR_INTERNAL, "[libmobility_gb300] Lanczos step kernel cannot be resident");
  }
  const int step_blocks = std::min(blocks, step_per_sm_ * sms());
  if (step_ctas_ < 0) step_ctas_ = step_cluster_ctas<R>();
  const bool step_cluster = g_lanczos_step_mode.load() == 0 && step_ctas_ > 0;
  // 256-thread CTAs while every thread keeps its elements in registers with
  // them (measured at n = 12288: 11 us against 17 us with 1024), else 1024
  // (n = 98304: 20 against 28 us)
  const int shape = g_lanczos_step_shape.load();
  const int cl_ctas = shape ? std::min(shape >> 16, step_ctas_) : step_ctas_;
  const size_t small_n = (size_t)std::max(step_ctas_, 1) * 256 * (sizeof(R) == 4 ? 8 : 4);
  const int cl_threads = shape ? (shape & 0xffff) : (n <= small_n ? 256 : kClusterThreads);
  double *err_flag = mir_dev + 516;
  mir[516] = 0.0;
  // the tickets and barrier words return to zero after every reduction and
  // barrier; a barrier that timed out leaves them inconsistent, so every
  // solve starts from zero (the side stream's last work precedes this point)
  LMG_CUDA(cudaMemsetAsync(red_ticket_.ptr, 0, 6 * sizeof(unsigned), st));

  LMG_CUDA(cudaMemsetAsync(sc, 0, sizeof(KrylovScalars), st));
  krylov_norm_kernel<R><<<blocks, kRedThreads, 0, st>>>(z, n, rp, tk, sc);
  count_launch();
  krylov_scale_first_kernel<R><<<blocks, kRedThreads, 0, st>>>(z, V, n, sc);
  count_launch();

  if (timing_) ensure_phase_events();
  int issued = 0;
  std::vector<int> checked;
  auto nper_lookahead = [&]() {
    const int forced = g_lanczos_lookahead.load();
    if (forced > 0) return std::min(forced, (int)kMaxLookahead);
    // one matrix-vector product of a batch of up to 8192 particles takes
    // tens of microseconds, less than a check
    return batch_size() <= 8192 ? 3 : 1;
  };
  auto issue = [&](int j) {
    R *vj = V + (size_t)j * n;
    if (timing_) LMG_CUDA(cudaEventRecord(ev_phase_[5 * j], st));
    apply_operator(vj, w);
    LMG_CUDA(cudaEventRecord(ev_prod_[j % kIterEvents], st));
    if (timing_) LMG_CUDA(cudaEventRecord(ev_phase_[5 * j + 1], st));
    const R *vprev = j > 0 ? vj - n : vj;
    R *vnext = vj + n;
    size_t nn = n;
    int jj = j;
    if (step_cluster) {
      LMG_CUDA(launch_step_cluster<R>(cl_ctas, cl_threads, w, vj, vprev, vnext, nn, jj, sc,
                                      mir_dev, st));
    } else {
      void *args[] = {&w, (void *)&vj, (void *)&vprev, &vnext, &nn, &jj, &rp, &tk, &bar,
                      &sc, &mir_dev, &err_flag};
      LMG_CUDA(cudaLaunchCooperativeKernel((const void *)krylov_step_kernel<R>,
                                           dim3(step_blocks), dim3(kRedThreads), args, 0, st));
      count_launch();
    }
    if (timing_) LMG_CUDA(cudaEventRecord(ev_phase_[5 * j + 2], st));
    LMG_CUDA(cudaEventRecord(ev_iter_[j % kIterEvents], st));
    issued = j + 1;
  };

  const int k = std::min(check_steps_, limit - 2);
  std::vector<double> al(limit), be(limit);
  issue(0);
  bool have_prev = false;
  int done = -1;
  double err = 0;
  // iterations issued ahead of the check of iteration i: the check (a host or
  // device square root of T, the estimate and its error) waits for the
  // host, so with cheap matrix-vector products several iterations keep the
  // GPU busy meanwhile; past convergence they are discarded
  int ahead = nper_lookahead();
  // A check is read one check late: the check of iteration i is launched,
  // then the error of the previous check (whose kernel has finished by then)
  // decides, so the host never waits on a check it just launched while the
  // GPU drains its queue.  The stopping step and result are the same as
  // deciding at once (the later launches are discarded); the error slots,
  // estimate buffers and host c slots alternate by iteration parity, and a
  // slot is reused only after the check that used it was read.
  int pend_i = -1;
  bool pend_tested = false;
  // a solve that ends in an error may leave the next check running on the
  // side stream; the next solve resets the tickets that check uses from the
  // main stream, so the side stream is drained before the error is raised
  auto fail = [&](lmg_status code, const char *msg) {
    cudaStreamSynchronize(sd);
    throw Error(code, msg);
  };
  auto resolve = [&](int pi, bool tested) {
    LMG_CUDA(cudaEventSynchronize(ev_check_[pi & 1]));
    if (mir[516] != 0.0)
      fail(LMG_ERR_TIMEOUT, "[libmobility_gb300] Lanczos step: grid barrier timed out");
    err = tested ? mir[512 + (pi & 1)] : HUGE_VAL;
    if (tested) {  // the reference never tests the first estimate (i > 0 there)
      if (residual) *residual = err;
      if (std::isnan(err)) fail(LMG_ERR_NAN, "[Lanczos] Unknown error (found NaN in result guess)");
    }
    if (cb_ && pi > 0) cb_(pi, err, cb_user_);
    if (tested && err <= tol) {
      lanczos_register(pi);
      done = pi;
    }
  };
  for (int i = 0; i < limit; i++) {
    while (issued <= i + ahead && issued < limit) issue(issued);
    if (!(i >= k || cb_ != nullptr)) continue;
    const int m = i + 1;
    double *cd = cdev + (i & 1) * kMaxLanczosIterations;
    R *yi = yb + (size_t)(i & 1) * n;
    // estimate y = |z| V c and its error against the previous estimate, one
    // launch on the side stream (c in device memory or mapped host memory)
    auto estimate_and_error = [&](const double *c_dev) {
      const R *yprev = have_prev ? yb + (size_t)((i + 1) & 1) * n : nullptr;
      double *e_out = mir_dev + 512 + (i & 1);
      if (n <= kCheckShortN)
        krylov_check_kernel<R, 4><<<vec_blocks(4 * n), kRedThreads, 0, sd>>>(
            V, n, m, c_dev, sc, yi, yprev, n, rp_side, tk_side, e_out);
      else
        krylov_check_kernel<R, 1><<<blocks, kRedThreads, 0, sd>>>(
            V, n, m, c_dev, sc, yi, yprev, n, rp_side, tk_side, e_out);
      count_launch();
      if (timing_) LMG_CUDA(cudaEventRecord(ev_phase_[5 * i + 4], sd));
      LMG_CUDA(cudaEventRecord(ev_check_[i & 1], sd));
      LMG_CUDA(cudaGetLastError());
    };
    NvtxRange nvtx_check("lmg Lanczos check");
    const int sqrt_mode = g_lanczos_device_sqrt.load();
    bool on_host = sqrt_mode != 1;
    if (!on_host) {
      // c = T^{1/2} e1 by quadrature on the device, right after iteration i
      LMG_CUDA(cudaStreamWaitEvent(sd, ev_iter_[i % kIterEvents], 0));
      if (timing_) LMG_CUDA(cudaEventRecord(ev_phase_[5 * i + 3], sd));
      tridiag_sqrt_quad_kernel<<<1, kQuadThreads, 0, sd>>>(sc, m, cd, quad_g, mir_dev + 520);
      count_launch();
      estimate_and_error(cd);
      LMG_CUDA(cudaEventSynchronize(ev_check_[i & 1]));  // for the fallback flag
      if (mir[516] != 0.0)
        fail(LMG_ERR_TIMEOUT, "[libmobility_gb300] Lanczos step: grid barrier timed out");
      on_host = mir[520] != 0.0;  // not positive definite or too ill-conditioned
    }
    if (on_host) {
      // T^{1/2} e1 on the host (quadrature, or the exact implicit QL; FP64)
      LMG_CUDA(cudaEventSynchronize(ev_iter_[i % kIterEvents]));
      if (mir[516] != 0.0)
        fail(LMG_ERR_TIMEOUT, "[libmobility_gb300] Lanczos step: grid barrier timed out");
      for (int q = 0; q < m; q++) {
        al[q] = mir[2 * q];
        be[q] = mir[2 * q + 1];
      }
      double *c = hc + (i & 1) * kMaxLanczosIterations;
      int rc = 1;
      if (sqrt_mode == 2)
        rc = tridiag_sqrt_e1_quad(al.data(), be.data(), m, ql_work_.data() + 768, c);
      if (rc != 0)
        rc = tridiag_sqrt_e1(al.data(), be.data(), m, ql_work_.data(), ql_work_.data() + 256,
                             ql_work_.data() + 512, log, c);
      if (rc != 0)
        for (int q = 0; q < m; q++) c[q] = std::nan("");
      // c is read by the kernel from mapped host memory: this slot is written
      // again two checks later, after this check was read.  The kernel reads
      // rows 0..i of V and the previous estimate, which the next product
      // and vector step leave alone, so it may also start after the next
      // product (check_wait 1)
      const bool after_next = g_lanczos_check_wait.load() == 1 && issued > i + 1;
      LMG_CUDA(cudaStreamWaitEvent(
          sd, after_next ? ev_prod_[(i + 1) % kIterEvents] : ev_iter_[i % kIterEvents], 0));
      if (timing_) LMG_CUDA(cudaEventRecord(ev_phase_[5 * i + 3], sd));
      estimate_and_error(hc_.device_ptr() + (i & 1) * kMaxLanczosIterations);
    }
    if (timing_) checked.push_back(i);
    if (pend_i >= 0) {
      resolve(pend_i, pend_tested);
      if (done >= 0) break;
    }
    pend_i = i;
    pend_tested = have_prev;
    have_prev = true;
  }
  if (done < 0 && pend_i >= 0) resolve(pend_i, pend_tested);
  if (done < 0) {
    LMG_CUDA(cudaStreamSynchronize(st));
    throw Error(LMG_ERR_NO_CONVERGENCE, "[Lanczos] Could not converge");
  }
  // the caller's stream sees the result after the side stream's last work
  LMG_CUDA(cudaMemcpyAsync(y_out, yb + (size_t)(done & 1) * n, n * sizeof(R),
                           cudaMemcpyDeviceToDevice, sd));
  LMG_CUDA(cudaEventRecord(ev_side_, sd));
  LMG_CUDA(cudaStreamWaitEvent(st, ev_side_, 0));
  if (timing_) {
    // algorithmic bytes: per iteration w, v_i, v_{i-1} read and v_{i+1}
    // written (4n); per check the m basis vectors read and y written, then
    // y and the previous y read for the error (2n, from the second check on)
    LMG_CUDA(cudaStreamSynchronize(st));
    const double vb = (double)n * sizeof(R);
    for (int j = 0; j < issued; j++) {
      float op = 0, ms = 0;
      LMG_CUDA(cudaEventElapsedTime(&op, ev_phase_[5 * j], ev_phase_[5 * j + 1]));
      LMG_CUDA(cudaEventElapsedTime(&ms, ev_phase_[5 * j + 1], ev_phase_[5 * j + 2]));
      phase_.operator_ms += op;
      phase_.vector_ms += ms;
      phase_.vector_bytes += 4 * vb;
    }
    for (size_t q = 0; q < checked.size(); q++) {
      const int i = checked[q];
      float ms = 0;
      LMG_CUDA(cudaEventElapsedTime(&ms, ev_phase_[5 * i + 3], ev_phase_[5 * i + 4]));
      phase_.check_ms += ms;
      phase_.check_bytes += (i + 2) * vb + (q > 0 ? 2 * vb : 0);
    }
    phase_.iterations += issued;
    phase_.checks += (long)checked.size();
    phase_.solves += 1;
  }
  return done;
}

template <class R>
void Solver<R>::sqrt_mdot_w(void *U, size_t nU, void *W, size_t nW, double prefactor,
                            const void *dW, size_t ndW, int *iterations, double *residual) {
  NvtxRange nvtx_range_("lmg sqrtMdotW");
  if (prefactor == 0) return;
  if (!initialized_)
    throw Error(LMG_ERR_NOT_INITIALIZED,
                "[libMobility] You must initialize the base class in order to use the default "
                "stochastic displacement computation");
  if (N_ <= 0)
    throw Error(LMG_ERR_NO_POSITIONS,
                "[libMobility] The number of particles is not set. Did you forget to call "
                "setPositions?");
  if (!U) nU = 0;
  if (!W) nW = 0;
  if (nU == 0)
    throw Error(LMG_ERR_INVALID_ARGUMENT, "[libMobility] This solver requires linear velocities");
  if (nU / 3 != (size_t)N_)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libMobility] The number of linear velocities does not match the number of "
                "particles");
  const size_t n3 = 3 * (size_t)N_;
  if (nW && nW != n3)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libMobility] The number of angular velocities does not match the number of "
                "particles");
  const size_t n = ang_ ? 2 * n3 : n3;
  if (dW && ndW != n)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] dW must hold 3N values (6N with includeAngular)");
  ensure_lanczos();
  R *z = z_.ensure(n);
  pin_.ensure(2 * n3);
  out_stage_.ensure(2 * n3);
  if (dW) {
    if (is_device_ptr(dW)) {
      LMG_CUDA(cudaMemcpyAsync(z, dW, n * sizeof(R), cudaMemcpyDeviceToDevice, stream()));
    } else {
      R *h = pin_.ensure(n);
      std::memcpy(h, dW, n * sizeof(R));
      LMG_CUDA(cudaMemcpyAsync(z, h, n * sizeof(R), cudaMemcpyHostToDevice, stream()));
    }
  } else {
    uint32_t s1, s2;
    draw_noise_seeds(s1, s2);
    gauss_fill_kernel<R><<<vec_blocks(n / 4 + 1), kRedThreads, 0, stream()>>>(z, n, s1, s2);
    count_launch();
    LMG_CUDA(cudaGetLastError());
  }
  R *y = y_.ensure(n);
  double res = 0;
  const bool prec = prec_active();
  const bool tp = timing_ && prec;
  if (tp) {
    ensure_phase_events();
    LMG_CUDA(cudaEventRecord(ev_pre_[0], stream()));
  }
  if (prec) prec_build();
  if (tp) LMG_CUDA(cudaEventRecord(ev_pre_[1], stream()));
  const int it = lanczos(z, y, n, tol_, &res);
  if (prec) {
    // y currently holds S^{1/2} z with S = P M P^T; the sample is P^{-1} of it
    // (translational part by BiCGSTAB, angular part by the scalar factor)
    R *x = bx_.ensure(n);
    if (tp) LMG_CUDA(cudaEventRecord(ev_pre_[2], stream()));
    last_inner_iters_ = solve_p(y, x);
    if (tp) {
      LMG_CUDA(cudaEventRecord(ev_pre_[3], stream()));
      LMG_CUDA(cudaEventSynchronize(ev_pre_[3]));
      float b = 0, q = 0;
      LMG_CUDA(cudaEventElapsedTime(&b, ev_pre_[0], ev_pre_[1]));
      LMG_CUDA(cudaEventElapsedTime(&q, ev_pre_[2], ev_pre_[3]));
      phase_.build_ms += b;
      phase_.psolve_ms += q;
    }
    if (ang_) {
      const R sc = (R)std::sqrt(r0_);
      scale_kernel<R><<<vec_blocks(n3), kRedThreads, 0, stream()>>>(x + n3, y + n3, n3, sc);
      count_launch();
    }
    LMG_CUDA(cudaMemcpyAsync(y, x, n * sizeof(R), cudaMemcpyDeviceToDevice, stream()));
  }
  if (iterations) *iterations = it;
  if (residual) *residual = res;
  // out += prefactor * y   (MobilityInterface.h:179-187)
  const bool u_dev = is_device_ptr(U);
  const bool w_dev = nW && is_device_ptr(W);
  R *Ud = u_dev ? static_cast<R *>(U) : out_stage_.ensure(2 * n3);
  R *Wd = nW ? (w_dev ? static_cast<R *>(W) : out_stage_.ensure(2 * n3) + n3) : nullptr;
  R *h = nullptr;
  if (!u_dev || (nW && !w_dev)) {
    h = pin_.ensure(2 * n3);
    if (!u_dev) std::memcpy(h, U, n3 * sizeof(R));
    if (nW && !w_dev) std::memcpy(h + n3, W, n3 * sizeof(R));
    if (!u_dev) LMG_CUDA(cudaMemcpyAsync(Ud, h, n3 * sizeof(R), cudaMemcpyHostToDevice, stream()));
    if (nW && !w_dev)
      LMG_CUDA(cudaMemcpyAsync(Wd, h + n3, n3 * sizeof(R), cudaMemcpyHostToDevice, stream()));
  }
  const int vb = vec_blocks(n3);
  axpy_kernel<R><<<vb, kRedThreads, 0, stream()>>>(Ud, y, n3, (R)prefactor);
  count_launch();
  if (ang_ && nW) {
    axpy_kernel<R><<<vb, kRedThreads, 0, stream()>>>(Wd, y + n3, n3, (R)prefactor);
    count_launch();
  }
  LMG_CUDA(cudaGetLastError());
  if (h) {
    if (!u_dev) LMG_CUDA(cudaMemcpyAsync(h, Ud, n3 * sizeof(R), cudaMemcpyDeviceToHost, stream()));
    if (nW && !w_dev)
      LMG_CUDA(cudaMemcpyAsync(h + n3, Wd, n3 * sizeof(R), cudaMemcpyDeviceToHost, stream()));
    LMG_CUDA(cudaStreamSynchronize(stream()));
    if (!u_dev) std::memcpy(U, h, n3 * sizeof(R));
    if (nW && !w_dev) std::memcpy(W, h + n3, n3 * sizeof(R));
  } else {
    LMG_CUDA(cudaStreamSynchronize(stream()));
  }
}

// Thermal drift by random finite differences.  Positions are displaced in the
// wall frame in which they are stored, so the solver's positions are left
// exactly as they were.
template <class R>
void Solver<R>::div_m(void *U, size_t nU, void *W, size_t nW, double prefactor) {
  NvtxRange nvtx_range_("lmg divM");
  if (prefactor == 0) return;
  if (!wall_) return;  // no wall, no thermal drift (mobility.h:189-190)
  if (!U) nU = 0;
  if (!W) nW = 0;
  const size_t n3 = 3 * (size_t)N_;
  if (nU != n3)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libMobility] The number of forces does not match the number of particles");
  if (ang_ && nW != n3)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libMobility] The number of torques does not match the number of particles");
  if (!ang_ && nW != 0)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libMobility] Received torques but the solver was initialized with "
                "includeAngular=False");
  check_positions_set("divM");
  const uint32_t seed = nbody_rng_();
  R *noise = rfd_noise_.ensure(n3);
  R *pd = rfd_pos_.ensure(n3);
  R *mp = rfd_mp_.ensure(2 * n3);
  R *mm = rfd_mm_.ensure(2 * n3);
  pin_.ensure(2 * n3);
  out_stage_.ensure(2 * n3);
  cudaStream_t st = stream();
  const int vb = vec_blocks(n3);
  gauss_fill_kernel<R><<<vec_blocks(n3 / 4 + 1), kRedThreads, 0, st>>>(noise, n3, seed,
                                                                       0x52464431u);
  count_launch();
  const R delta = (R)(delta_ * a_);
  displace_kernel<R><<<vb, kRedThreads, 0, st>>>(pos_.ptr, noise, pd, n3, delta * R(0.5));
  count_launch();
  mdot_device(pd, noise, nullptr, mp, ang_ ? mp + n3 : nullptr);
  displace_kernel<R><<<vb, kRedThreads, 0, st>>>(pos_.ptr, noise, pd, n3, -delta * R(0.5));
  count_launch();
  mdot_device(pd, noise, nullptr, mm, ang_ ? mm + n3 : nullptr);
  LMG_CUDA(cudaGetLastError());
  const R c = (R)(prefactor / (delta_ * a_));
  const bool u_dev = is_device_ptr(U);
  const bool w_dev = nW && is_device_ptr(W);
  R *Ud = u_dev ? static_cast<R *>(U) : out_stage_.ensure(2 * n3);
  R *Wd = nW ? (w_dev ? static_cast<R *>(W) : out_stage_.ensure(2 * n3) + n3) : nullptr;
  R *h = nullptr;
  if (!u_dev || (nW && !w_dev)) {
    h = pin_.ensure(2 * n3);
    if (!u_dev) std::memcpy(h, U, n3 * sizeof(R));
    if (nW && !w_dev) std::memcpy(h + n3, W, n3 * sizeof(R));
    if (!u_dev) LMG_CUDA(cudaMemcpyAsync(Ud, h, n3 * sizeof(R), cudaMemcpyHostToDevice, st));
    if (nW && !w_dev)
      LMG_CUDA(cudaMemcpyAsync(Wd, h + n3, n3 * sizeof(R), cudaMemcpyHostToDevice, st));
  }
  add_scaled_diff_kernel<R><<<vb, kRedThreads, 0, st>>>(Ud, mp, mm, n3, c);
  count_launch();
  if (ang_ && nW) {
    add_scaled_diff_kernel<R><<<vb, kRedThreads, 0, st>>>(Wd, mp + n3, mm + n3, n3, c);
    count_launch();
  }
  LMG_CUDA(cudaGetLastError());
  if (h) {
    if (!u_dev) LMG_CUDA(cudaMemcpyAsync(h, Ud, n3 * sizeof(R), cudaMemcpyDeviceToHost, st));
    if (nW && !w_dev)
      LMG_CUDA(cudaMemcpyAsync(h + n3, Wd, n3 * sizeof(R), cudaMemcpyDeviceToHost, st));
    LMG_CUDA(cudaStreamSynchronize(st));
    if (!u_dev) std::memcpy(U, h, n3 * sizeof(R));
    if (nW && !w_dev) std::memcpy(W, h + n3, n3 * sizeof(R));
  }
}

template <class R> void Solver<R>::clean() {
  // Mobility::clean drops the Lanczos object (its engine and check schedule)
  // and its storage; positions and parameters stay.
  if (have_stream_) cudaStreamSynchronize(stream_);
  if (side_) cudaStreamSynchronize(side_);
  lanczos_alive_ = false;
  check_steps_ = 3;
  V_.release(); w_.release(); y_.release(); ybuf_.release(); z_.release();
  rot_cs_ = {}; rot_idx_ = {};
  part_.release(); tickets_.release(); tickets_zeroed_ = false; plans_.clear();
  rfd_noise_.release(); rfd_pos_.release(); rfd_mp_.release(); rfd_mm_.release();
}

template <class R>
void Solver<R>::set_preconditioner(const std::string &kind, const float *params, size_t n) {
  if (kind == "none") {
    prec_on_ = false;
    return;
  }
  if (kind != "mlp")
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] preconditioner must be \"none\" or \"mlp\"");
  if (!std::is_same<R, float>::value)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] the learned preconditioner needs precision float");
  const PrecLayout L = params ? prec_layout_for_params(n) : PrecLayout{};
  if (L.K == 0)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] preconditioner parameters: " + std::to_string(n) +
                    " floats is not the size of a network over K = 16, 32, 48 or 64 neighbours "
                    "with 64, 128, 256, 512 or 1024 hidden units");
  if (L.wall && !wall_)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] this preconditioner network was trained above a wall; "
                "the solver has an open boundary");
  float *d = prec_params_.ensure(n);
  LMG_CUDA(cudaMemcpy(d, params, n * sizeof(float), cudaMemcpyHostToDevice));
  prec_layout_ = L;
  prec_k_ = L.K;
  prec_on_ = true;
  prec_dirty_ = true;
}

// The preconditioner needs at least K + 1 particles per batch; smaller
// systems fall back to plain Lanczos.
template <class R> bool Solver<R>::prec_active() const {
  return prec_on_ && std::is_same<R, float>::value && batch_size() >= prec_k_ + 1;
}

template <class R> void Solver<R>::prec_build() {
  NvtxRange nvtx_range_("lmg preconditioner build");
  if constexpr (std::is_same<R, float>::value) {
    if (!prec_dirty_) return;
    const int N = (int)N_;
    const int kb = prec_k_ + 1;
    int *nb = prec_nb_.ensure((size_t)N * kb);
    uint16_t *blocks = prec_blocks_.ensure((size_t)N * kb * 9);
    LMG_CUDA(knn_launch(prec_k_, pos_.ptr, N, batch_size(), nb, stream(), &knn_scratch_));
    // blocks at unit scale (the network's t0 = 1), in half precision; the
    // products apply t0^{-1/2} (prec_scale)
    LMG_CUDA(precond_build_launch(prec_layout_, pos_.ptr, nb, N, prec_params_.ptr, (float)(1.0 / a_),
                                  1.0f, blocks, true, &prec_work_, stream()));
    prec_dirty_ = false;
  }
}

template <class R> void Solver<R>::apply_operator(const R *v, R *out) {
  const size_t n3 = 3 * (size_t)N_;
  if (!prec_active()) {
    mdot_device(pos_.ptr, v, ang_ ? v + n3 : nullptr, out, ang_ ? out + n3 : nullptr);
    return;
  }
  if constexpr (std::is_same<R, float>::value) {
    const int N = (int)N_;
    const size_t n = ang_ ? 2 * n3 : n3;
    R *t = pt_.ensure(n);
    R *u = pu_.ensure(n);
    const R s = (R)(1.0 / std::sqrt(r0_));  // angular part: scalar r0^{-1/2}
    float4 *pad = reinterpret_cast<float4 *>(ppad_.ensure(4 * (size_t)N));
    LMG_CUDA(precond_apply_t_launch(prec_k_, prec_blocks_.ptr, true, prec_scale(), prec_nb_.ptr, N,
                                    v, t, pad, stream()));
    if (ang_) {
      scale_kernel<R><<<vec_blocks(n3), kRedThreads, 0, stream()>>>(t + n3, v + n3, n3, s);
      count_launch();
    }
    mdot_device(pos_.ptr, t, ang_ ? t + n3 : nullptr, u, ang_ ? u + n3 : nullptr);
    LMG_CUDA(precond_apply_launch(prec_k_, prec_blocks_.ptr, true, prec_scale(), prec_nb_.ptr, N, u, out, stream()));
    if (ang_) {
      scale_kernel<R><<<vec_blocks(n3), kRedThreads, 0, stream()>>>(out + n3, u + n3, n3, s);
      count_launch();
    }
  }
}

// BiCGSTAB (van der Vorst 1992) for P x = b on the translational part,
// relative residual 1e-7 (the Lanczos tolerance is at least 1e-6 on single
// precision vectors).  Scalars in FP64 on the host; each reduction is read
// back through mapped memory.
template <class R> int Solver<R>::solve_p(const R *b, R *x) {
  NvtxRange nvtx_range_("lmg preconditioner solve");
  if constexpr (!std::is_same<R, float>::value) {
    (void)b; (void)x;
    return 0;
  } else {
    const int N = (int)N_;
    const size_t n = 3 * (size_t)N;
    cudaStream_t st = stream();
    const int blocks = vec_blocks(n);
    ensure_reduction(blocks);
    unsigned *tk = red_ticket_.ptr;
    double *rp = red_part_.ptr;
    double *mir = mirror_.ensure(2 * 256 + 8);
    double *out = mirror_.device_ptr() + 514;
    double *hout = mir + 514;
    R *r = br_.ensure(n), *rh = brh_.ensure(n), *p = bp_.ensure(n), *v = bv_.ensure(n);
    R *s = bs_.ensure(n), *t = bt_.ensure(n);
    auto sync = [&]() { LMG_CUDA(cudaStreamSynchronize(st)); };
    LMG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(R), st));
    LMG_CUDA(cudaMemsetAsync(p, 0, n * sizeof(R), st));
    LMG_CUDA(cudaMemsetAsync(v, 0, n * sizeof(R), st));
    LMG_CUDA(cudaMemcpyAsync(r, b, n * sizeof(R), cudaMemcpyDeviceToDevice, st));
    LMG_CUDA(cudaMemcpyAsync(rh, b, n * sizeof(R), cudaMemcpyDeviceToDevice, st));
    dot2_kernel<R><<<blocks, kRedThreads, 0, st>>>(b, b, b, b, n, rp, tk, out);
    count_launch();
    sync();
    const double bnorm2 = hout[0];
    if (!(bnorm2 > 0)) return 0;
    const double tol2 = 1e-14 * bnorm2;
    double rho = 1, alpha = 1, omega = 1, rho1 = bnorm2;
    const int max_it = 500;
    for (int it = 1; it <= max_it; it++) {
      const double beta = (rho1 / rho) * (alpha / omega);
      bicg_p_kernel<R><<<blocks, kRedThreads, 0, st>>>(p, r, v, it == 1 ? 0.0 : beta,
                                                       omega, n);
      count_launch();
      LMG_CUDA(precond_apply_launch(prec_k_, prec_blocks_.ptr, true, prec_scale(), prec_nb_.ptr, N, p, v, st));
      dot2_kernel<R><<<blocks, kRedThreads, 0, st>>>(rh, v, rh, v, n, rp, tk, out);
      count_launch();
      sync();
      const double rv = hout[0];
      if (rv == 0 || std::isnan(rv))
        throw Error(LMG_ERR_NAN, "[libmobility_gb300] preconditioner solve broke down");
      alpha = rho1 / rv;
      bicg_s_kernel<R><<<blocks, kRedThreads, 0, st>>>(s, r, v, alpha, n, rp, tk, out);
      count_launch();
      sync();
      if (hout[0] <= tol2) {  // x += alpha p
        bicg_xr_kernel<R><<<blocks, kRedThreads, 0, st>>>(x, p, s, s, r, rh, alpha, 0.0, n,
                                                          rp, tk, out);
        count_launch();
        sync();
        return it;
      }
      LMG_CUDA(precond_apply_launch(prec_k_, prec_blocks_.ptr, true, prec_scale(), prec_nb_.ptr, N, s, t, st));
      dot2_kernel<R><<<blocks, kRedThreads, 0, st>>>(t, s, t, t, n, rp, tk, out);
      count_launch();
      sync();
      omega = hout[0] / hout[1];
      bicg_xr_kernel<R><<<blocks, kRedThreads, 0, st>>>(x, p, s, t, r, rh, alpha, omega, n, rp,
                                                        tk, out);
      count_launch();
      sync();
      rho = rho1;
      rho1 = hout[1];
      if (hout[0] <= tol2) return it;
      if (std::isnan(hout[0]))
        throw Error(LMG_ERR_NAN, "[libmobility_gb300] preconditioner solve broke down");
    }
    throw Error(LMG_ERR_NO_CONVERGENCE,
                "[libmobility_gb300] preconditioner solve did not converge");
  }
}

SolverBase *make_solver(Periodicity x, Periodicity y, Periodicity z, int precision) {
  if (precision == LMG_PRECISION_DOUBLE) return new Solver<double>(x, y, z);
  if (precision == LMG_PRECISION_FLOAT) return new Solver<float>(x, y, z);
  throw Error(LMG_ERR_INVALID_ARGUMENT, "[libmobility_gb300] precision must be 0 (float) or 1 (double)");
}

int tridiag_sqrt_e1_quad_host(const double *alpha, const double *beta, int m, double *out) {
  if (m < 1 || m > 256) return 3;
  std::vector<double> work(18 * (size_t)m);
  return tridiag_sqrt_e1_quad(alpha, beta, m, work.data(), out);
}

int tridiag_sqrt_e1_host(const double *alpha, const double *beta, int m, double *out) {
  if (m < 1 || m > 256) return 3;
  std::vector<double> d(m), e(m), q(m);
  const int cap = 64 * m * m + 64;
  std::vector<double2> cs(cap);
  std::vector<int> idx(cap);
  RotLog log{cs.data(), idx.data(), cap};
  return tridiag_sqrt_e1(alpha, beta, m, d.data(), e.data(), q.data(), log, out);
}

}  // namespace lmg
