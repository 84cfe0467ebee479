// Ensembles: many independent NBody systems of uneven size, open and
// bottom-wall geometries mixed, run together.
//
// Every system behaves as its own NBody solver (solvers/NBody/mobility.h):
// same constants, same wall shift and below-the-wall check, same pair
// formulas, and for sqrtMdotW the same Lanczos recurrence, breakdown rule,
// successive-iterate error, adaptive check schedule and iteration limit
// (LanczosAlgorithm.cu:110-232), each system stopping at its own
// convergence.  What is shared is the work:
//
//   * layout: systems are stored in an internal order, sorted by geometry
//     and by size bucket (powers of two), each padded to a multiple of 128
//     particles with dummy particles of zero strength placed far away
//     (1e5 radii off, 4 radii apart), so that every tile of 128 targets of
//     the all-pairs kernel lies inside one system and takes the full-tile
//     path; dummies add exactly zero to real particles and their own
//     outputs are never read;
//   * matrix-vector product: one all-pairs launch per group (geometry x size
//     bucket) with the group's batch table; each group has its own launch
//     plan (source splits), picked by timing the candidates on first use
//     (autotune) or by the occupancy planner; systems already converged are
//     skipped tile by tile through a per-system flag;
//   * Lanczos: one launch per iteration updates every active system's
//     vectors (one CTA per system: alpha, beta with the breakdown rule, the
//     next basis vector), the per-iteration launches are captured once in a
//     CUDA graph and replayed, and result estimates with their errors are one
//     more launch per check; the FP64 tridiagonal square roots of the
//     systems due for a check run on a pool of host threads while the GPU
//     already works on the next iteration.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <random>
#include <sstream>
#include <thread>
#include <vector>

#include "ensemble.hpp"
#include "krylov.cuh"
#include "launch_count.hpp"
#include "mdot_launch.cuh"
#include "solver.hpp"

namespace lmg {

namespace {

constexpr int kPad = 128;            // systems padded to a multiple of this
constexpr int kEnsThreads = 256;     // threads of the per-system vector kernels
constexpr int kEnsLimit = 200;       // lanczos::Solver::iterationHardLimit
constexpr size_t kEnsBranches = 8;   // streams the groups' products run on side by side
constexpr int kEstChunk = 4 * kEnsThreads;  // elements of one system per estimate CTA
constexpr double kDummyFar = 1e5;    // dummy particles: radii away from everything

bool ens_is_device_ptr(const void *p) { return device_pointer(p); }

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Block-wide FP64 sums of NV values (kEnsThreads threads); every thread gets
// the totals, summed in a fixed order.
template <int NV> __device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double red[NV][kEnsThreads / 32];
#pragma unroll
  for (int q = 0; q < NV; q++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; q++) {
    double t = 0.0;
    for (int w = 0; w < kEnsThreads / 32; w++) t += red[q][w];
    v[q] = t;
  }
  __syncthreads();
}

// Internal positions: gathered from the caller's order, wall systems shifted
// by their wall height (mobility.h:124-148) and checked; dummies placed far.
template <class R>
__global__ void ens_gather_pos(const R *pos_user, const int *imap, const int *psys,
                               const int *sgeom, const double *sheight, R *pos_int, int npad,
                               R far, R a, int *below) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npad) return;
  const int u = imap[i];
  if (u < 0) {
    pos_int[3 * i] = far + R(4) * a * (R)(i % 262144);
    pos_int[3 * i + 1] = R(4) * a * (R)(i / 262144);
    pos_int[3 * i + 2] = far;
    return;
  }
  const int s = psys[i];
  R x = pos_user[3 * u], y = pos_user[3 * u + 1], z = pos_user[3 * u + 2];
  if (sgeom[s]) {
    z = z - (R)sheight[s];
    if (z < R(0)) atomicOr(below, 1);
  }
  pos_int[3 * i] = x;
  pos_int[3 * i + 1] = y;
  pos_int[3 * i + 2] = z;
}

// dst (internal) = src (caller's order); dummies get 0
template <class R>
__global__ void ens_gather_vec(const R *src, const int *imap, R *dst, int npad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npad) return;
  const int u = imap[i];
#pragma unroll
  for (int c = 0; c < 3; c++) dst[3 * i + c] = u >= 0 ? src[3 * u + c] : R(0);
}

// dst (caller's order) = pf * src (internal), or += with accumulate; src is
// taken from buffer parity[psys[i]] of `src` when parity is given
template <class R>
__global__ void ens_scatter(const R *src, size_t ld, const int *parity, const int *imap,
                            const int *psys, R *dst, int npad, R pf, int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npad) return;
  const int u = imap[i];
  if (u < 0) return;
  const R *s = parity ? src + (size_t)parity[psys[i]] * ld : src;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const R v = pf * s[3 * i + c];
    dst[3 * u + c] = accumulate ? dst[3 * u + c] + v : v;
  }
}

// |z_s| and v0 = z_s / |z_s| per system (one CTA per system)
template <class R>
__global__ void ens_first(const R *z, R *V0, R *vcur, const int *off3, const int *nn,
                          double *normz) {
  const int s = blockIdx.x;
  const int o = off3[s], n = nn[s];
  double v[1] = {0.0};
  for (int e = threadIdx.x; e < n; e += kEnsThreads) {
    const double x = (double)z[o + e];
    v[0] += x * x;
  }
  block_sum<1>(v);
  const double nz = sqrt(v[0]);
  if (threadIdx.x == 0) normz[s] = nz;
  const R inv = (R)(1.0 / nz);
  for (int e = threadIdx.x; e < n; e += kEnsThreads) {
    const R x = z[o + e] * inv;
    V0[o + e] = x;
    vcur[o + e] = x;
  }
}

// One Lanczos iteration i = *iter for every active system, after w = M v_i
// (KrylovSubspace, LanczosAlgorithm.cu:131-152), split over CTAs (s, c), c a
// chunk of kEstChunk elements of system s, in three launches (one CTA per
// system took a fifth of an iteration for the largest systems).  Each
// reduction goes through per-system chunk partials, summed in chunk order by
// the last CTA of the system to finish (ticket), which publishes the scalar.
template <class R>
__device__ __forceinline__ bool ens_chunk_sum(double v, double *part, unsigned *ticket, int s,
                                              int c, int nch, double &total) {
  __shared__ bool s_last;
  double a[1] = {v};
  block_sum<1>(a);
  if (threadIdx.x == 0) {
    __stcg(part + (size_t)s * gridDim.y + c, a[0]);
    __threadfence();
    s_last = atomicAdd(ticket + s, 1u) == (unsigned)(nch - 1);
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return false;
  __threadfence();
  double t = 0.0;
  for (int q = 0; q < nch; q++) t += __ldcg(part + (size_t)s * gridDim.y + q);
  total = t;
  ticket[s] = 0u;
  return true;
}

// w -= beta_{i-1} v_{i-1};  alpha_i = w . v_i
template <class R>
__global__ void ens_step_alpha(R *w, const R *V, size_t ldv, const int *iter, const int *off3,
                               const int *nn, const int *active, const double *beta,
                               double *alpha, int lim, double *part, unsigned *ticket) {
  const int s = blockIdx.x;
  if (!active[s]) return;
  const int n = nn[s], nch = (n + kEstChunk - 1) / kEstChunk, c = blockIdx.y;
  if (c >= nch) return;
  const int i = *iter, o = off3[s];
  R *ws = w + o;
  const R *vi = V + (size_t)i * ldv + o;
  const R *vp = i > 0 ? vi - ldv : vi;
  const R bprev = i > 0 ? (R)beta[s * lim + i - 1] : R(0);
  double acc = 0.0;
  for (int e = c * kEstChunk + threadIdx.x; e < min(n, (c + 1) * kEstChunk); e += kEnsThreads) {
    R x = ws[e];
    if (i > 0) x -= bprev * vp[e];
    ws[e] = x;
    acc += (double)x * (double)vi[e];
  }
  double tot;
  if (ens_chunk_sum<R>(acc, part, ticket, s, c, nch, tot)) alpha[s * lim + i] = tot;
}

// w -= alpha_i v_i;  beta_i = |w| (0 below 1e-3 alpha_i/|z|); both to the
// device arrays and to mapped host memory
template <class R>
__global__ void ens_step_beta(R *w, const R *V, size_t ldv, const int *iter, const int *off3,
                              const int *nn, const int *active, const double *normz,
                              const double *alpha, double *beta, int lim, double *host_ab,
                              double *part, unsigned *ticket) {
  const int s = blockIdx.x;
  if (!active[s]) return;
  const int n = nn[s], nch = (n + kEstChunk - 1) / kEstChunk, c = blockIdx.y;
  if (c >= nch) return;
  const int i = *iter, o = off3[s];
  R *ws = w + o;
  const R *vi = V + (size_t)i * ldv + o;
  const double al = alpha[s * lim + i];
  const R alr = (R)al;
  double acc = 0.0;
  for (int e = c * kEstChunk + threadIdx.x; e < min(n, (c + 1) * kEstChunk); e += kEnsThreads) {
    const R x = ws[e] - alr * vi[e];
    ws[e] = x;
    acc += (double)x * (double)x;
  }
  double tot;
  if (ens_chunk_sum<R>(acc, part, ticket, s, c, nch, tot)) {
    double b = sqrt(tot);
    if (b < 1e-3 * al / normz[s]) b = 0.0;
    beta[s * lim + i] = b;
    host_ab[2 * (s * lim + i)] = al;
    host_ab[2 * (s * lim + i) + 1] = b;
  }
}

// v_{i+1} = w / beta_i, or e1 after a breakdown
template <class R>
__global__ void ens_step_next(const R *w, R *V, R *vcur, size_t ldv, const int *iter,
                              const int *off3, const int *nn, const int *active,
                              const double *beta, int lim) {
  const int s = blockIdx.x;
  if (!active[s]) return;
  const int n = nn[s], nch = (n + kEstChunk - 1) / kEstChunk, c = blockIdx.y;
  if (c >= nch) return;
  const int i = *iter, o = off3[s];
  const double b = beta[s * lim + i];
  const R inv = b > 0.0 ? (R)(1.0 / b) : R(0);
  R *vn = V + (size_t)(i + 1) * ldv + o;
  for (int e = c * kEstChunk + threadIdx.x; e < min(n, (c + 1) * kEstChunk); e += kEnsThreads) {
    const R x = b > 0.0 ? w[o + e] * inv : (e == 0 ? R(1) : R(0));
    vn[e] = x;
    vcur[o + e] = x;
  }
}

__global__ void ens_iter_inc(int *iter) { *iter += 1; }

// Result estimate y_s = |z_s| V_s c_s (m basis vectors) for the systems due
// for a check, written to ynew, and err_s = |y_s - yold_s| / |yold_s|
// (LanczosAlgorithm.cu:202-222).  CTA (s, c) takes elements [c, c+1) x
// kEstChunk of system s (one CTA per system left a 4000-particle system's
// estimate to a single SM, slower than an iteration's products); the last
// CTA of a system to finish sums the chunks' partial norms in chunk order.
template <class R>
__global__ void ens_estimate(const R *V, size_t ldv, int m, const double *coef, int lim,
                             const int *due, const double *normz, const int *off3,
                             const int *nn, R *ynew, const R *yold, double *part,
                             unsigned *ticket, double *err) {
  const int s = blockIdx.x;
  if (!due[s]) return;
  const int n = nn[s];
  const int nch = (n + kEstChunk - 1) / kEstChunk, c = blockIdx.y;
  if (c >= nch) return;
  __shared__ R cs[kEnsLimit + 1];
  __shared__ bool s_last;
  const double nz = normz[s];
  for (int k = threadIdx.x; k < m; k += kEnsThreads) cs[k] = (R)(nz * coef[s * lim + k]);
  __syncthreads();
  const int o = off3[s];
  const int e_end = min(n, (c + 1) * kEstChunk);
  double v[2] = {0.0, 0.0};
  for (int e = c * kEstChunk + threadIdx.x; e < e_end; e += kEnsThreads) {
    // eight independent partial sums: eight basis-vector loads in flight
    R part[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const R *col = V + o + e;
    int k = 0;
    for (; k + 8 <= m; k += 8) {
#pragma unroll
      for (int u = 0; u < 8; u++) part[u] += cs[k + u] * col[(size_t)(k + u) * ldv];
    }
    for (; k < m; k++) part[k & 7] += cs[k] * col[(size_t)k * ldv];
    const R acc = ((part[0] + part[1]) + (part[2] + part[3])) +
                  ((part[4] + part[5]) + (part[6] + part[7]));
    ynew[o + e] = acc;
    const double a = (double)yold[o + e], d = (double)acc - a;
    v[0] += a * a;
    v[1] += d * d;
  }
  block_sum<2>(v);
  double *mine = part + ((size_t)s * gridDim.y + c) * 2;
  if (threadIdx.x == 0) {
    __stcg(mine, v[0]);
    __stcg(mine + 1, v[1]);
    __threadfence();
    s_last = atomicAdd(ticket + s, 1u) == (unsigned)(nch - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    const double *ps = part + (size_t)s * gridDim.y * 2;
    double a = 0.0, d = 0.0;
    for (int q = 0; q < nch; q++) {
      a += __ldcg(ps + 2 * q);
      d += __ldcg(ps + 2 * q + 1);
    }
    err[s] = fabs(sqrt(d) / sqrt(a));
    ticket[s] = 0u;
  }
}

// ---------------------------------------------------------------------------
// Host thread pool for the per-system eigen-solves
// ---------------------------------------------------------------------------
class WorkerPool {
 public:
  explicit WorkerPool(int n) {
    for (int t = 0; t < n; t++) threads_.emplace_back([this] { loop(); });
  }
  ~WorkerPool() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto &t : threads_) t.join();
  }
  // runs f(0) ... f(jobs-1) on the workers and the calling thread
  void run(int jobs, const std::function<void(int)> &f) {
    if (jobs <= 0) return;
    {
      std::lock_guard<std::mutex> lk(m_);
      job_.store(&f);
      jobs_.store(jobs);
      next_.store(0);
      left_ = jobs;
      gen_++;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(m_);
    done_.wait(lk, [this] { return left_ == 0; });
    job_.store(nullptr);
  }

 private:
  void work() {
    for (;;) {
      const int k = next_.fetch_add(1);
      if (k >= jobs_.load()) return;
      (*job_.load())(k);
      std::lock_guard<std::mutex> lk(m_);
      if (--left_ == 0) done_.notify_all();
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return stop_ || (gen_ != seen && job_.load() != nullptr); });
        if (stop_) return;
        seen = gen_;
      }
      work();
    }
  }
  std::vector<std::thread> threads_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  std::atomic<const std::function<void(int)> *> job_{nullptr};
  std::atomic<int> jobs_{0};
  std::atomic<int> next_{0};
  int left_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

int pool_threads() {
  const unsigned hc = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(hc ? hc : 4u, 16u)) - 1;
}

// ---------------------------------------------------------------------------
// The ensemble
// ---------------------------------------------------------------------------
template <class R> class Ensemble final : public EnsembleBase {
 public:
  Ensemble() : pool_(pool_threads()) {}
  ~Ensemble() override {
    drop_graph();
    release_branches();
    if (ev_ready_) {
      cudaEventDestroy(ev_iter_[0]);
      cudaEventDestroy(ev_iter_[1]);
      cudaEventDestroy(ev_check_);
      cudaEventDestroy(ev_side_);
      cudaEventDestroy(ev_t0_);
      cudaEventDestroy(ev_t1_);
    }
    if (side_) cudaStreamDestroy(side_);
    if (cap_) cudaStreamDestroy(cap_);
    if (own_) cudaStreamDestroy(own_);
  }

  void set_stream(cudaStream_t s) override {
    stream_ = s;
    have_stream_ = true;
  }
  void use_own_stream() override { have_stream_ = false; }

  void set_systems(int nsys, const int *sizes, const int *geometry,
                   const double *wall_heights) override;
  void initialize(double eta, double a, double tol, uint64_t seed, bool autotune) override;
  void set_positions(const void *pos, size_t n) override;
  void mdot(const void *F, size_t nF, void *U, size_t nU) override;
  void sqrt_mdot_w(const void *dW, size_t ndW, void *U, size_t nU, double pf, int *its,
                   double *errs, double *ms) override;
  std::string describe() const override;

 private:
  struct Group {
    int geom = 0, bucket = 0;
    int s0 = 0, s1 = 0;  // internal systems [s0, s1)
    int p0 = 0, p1 = 0;  // internal (padded) particles [p0, p1)
    int span = 0;        // largest padded system
    DeviceBuffer<int> sys_begin;
    MdotPlan plan;
    bool tuned = false;
    std::vector<std::pair<int, double>> trials;  // (1000 tpt + nsplit, ms)
    // this group's share of the split scratch, so groups can run at once
    size_t part_off = 0, ticket_off = 0;
    double work = 0;  // pair flops of one product (padded sizes)
    int branch = 0;   // stream it runs on beside the others
  };

  cudaStream_t stream() {
    if (!have_stream_) {
      if (!own_) LMG_CUDA(cudaStreamCreateWithFlags(&own_, cudaStreamNonBlocking));
      stream_ = own_;
      have_stream_ = true;
    }
    return stream_;
  }
  void ensure_events() {
    if (ev_ready_) return;
    LMG_CUDA(cudaEventCreateWithFlags(&ev_iter_[0], cudaEventDisableTiming));
    LMG_CUDA(cudaEventCreateWithFlags(&ev_iter_[1], cudaEventDisableTiming));
    LMG_CUDA(cudaEventCreateWithFlags(&ev_check_, cudaEventDisableTiming));
    LMG_CUDA(cudaEventCreateWithFlags(&ev_side_, cudaEventDisableTiming));
    LMG_CUDA(cudaEventCreate(&ev_t0_));
    LMG_CUDA(cudaEventCreate(&ev_t1_));
    LMG_CUDA(cudaStreamCreateWithPriority(&side_, cudaStreamNonBlocking, -1));
    LMG_CUDA(cudaStreamCreateWithFlags(&cap_, cudaStreamNonBlocking));
    ev_ready_ = true;
  }
  void drop_graph() {
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
    graph_key_.clear();
  }
  int sms() {
    if (sms_ == 0) {
      int dev = 0;
      LMG_CUDA(cudaGetDevice(&dev));
      LMG_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
    }
    return sms_;
  }
  MdotShape shape(const Group &g) const {
    MdotShape s;
    s.geom = g.geom ? kWall : kOpen;
    s.has_f = true;
    s.has_t = false;
    s.ang = false;
    return s;
  }
  void require_ready() const {
    if (nsys_ == 0)
      throw Error(LMG_ERR_INVALID_ARGUMENT, "[libmobility_gb300] the ensemble has no systems");
    if (!init_)
      throw Error(LMG_ERR_NOT_INITIALIZED,
                  "[libMobility] You must initialize the base class in order to use the default "
                  "stochastic displacement computation");
    if (!have_pos_)
      throw Error(LMG_ERR_NO_POSITIONS,
                  "[libMobility] The number of particles is not set. Did you forget to call "
                  "setPositions?");
  }
  const R *to_device_user(const void *p, size_t n, DeviceBuffer<R> &stage) {
    if (ens_is_device_ptr(p)) return static_cast<const R *>(p);
    R *h = pin_.ensure(n);
    std::memcpy(h, p, n * sizeof(R));
    R *d = stage.ensure(n);
    LMG_CUDA(cudaMemcpyAsync(d, h, n * sizeof(R), cudaMemcpyHostToDevice, stream()));
    return d;
  }
  static int grid(int n) { return (n + 255) / 256; }
  MdotArgs<R> args(const Group &g, const R *x, R *y, const int *active) {
    MdotArgs<R> a{};
    a.pos = pos_.ptr + 3 * (size_t)g.p0;
    a.F = x + 3 * (size_t)g.p0;
    a.T = nullptr;
    a.U = y + 3 * (size_t)g.p0;
    a.W = nullptr;
    a.sys_begin = g.sys_begin.ptr;
    a.nsys = g.s1 - g.s0;
    a.N = g.p1 - g.p0;
    a.nper = a.N;
    a.inv_a = (R)(1.0 / a_);
    a.k = make_pair_const<R>(t0_, r0_, rt0_);
    a.kw = make_wall_const(t0_, r0_, rt0_);
    a.part = part_.ptr + g.part_off;
    a.ticket = tickets_.ptr + g.ticket_off;
    a.sys_active = active ? active + g.s0 : nullptr;
    return a;
  }
  void ensure_scratch(const MdotPlan &p) {
    part_.ensure(std::max<size_t>(p.part_elems, 1));
    if (tickets_.count < std::max<size_t>(p.tickets, 1)) {
      tickets_.ensure(std::max<size_t>(p.tickets, 1));
      LMG_CUDA(cudaMemsetAsync(tickets_.ptr, 0, tickets_.count * sizeof(unsigned), stream()));
    }
  }
  void launch_group(Group &g, const R *x, R *y, const int *active, cudaStream_t st) {
    LMG_CUDA(mdot_launch<R>(shape(g), args(g, x, y, active), g.plan, st));
  }
  // every group's product, the groups side by side on streams forked from
  // st and joined back into it (their outputs, scratch and tickets are
  // disjoint), so one group's last wave overlaps the others' work
  void launch_groups(const R *x, R *y, const int *active, cudaStream_t st) {
    if (groups_.size() <= 1) {
      for (auto &g : groups_) launch_group(*g, x, y, active, st);
      return;
    }
    ensure_branches();
    LMG_CUDA(cudaEventRecord(ev_fork_, st));
    for (size_t q = 0; q < branch_.size(); q++) LMG_CUDA(cudaStreamWaitEvent(branch_[q], ev_fork_, 0));
    // the largest products are issued first on their streams
    std::vector<int> ord(groups_.size());
    for (size_t q = 0; q < ord.size(); q++) ord[q] = (int)q;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int a, int b) { return groups_[a]->work > groups_[b]->work; });
    for (int q : ord)
      launch_group(*groups_[q], x, y, active, branch_[groups_[q]->branch % branch_.size()]);
    for (size_t q = 0; q < branch_.size() && q < groups_.size(); q++) {
      LMG_CUDA(cudaEventRecord(ev_join_[q], branch_[q]));
      LMG_CUDA(cudaStreamWaitEvent(st, ev_join_[q], 0));
    }
  }
  void ensure_branches() {
    if (!branch_.empty()) return;
    const size_t nb = std::min<size_t>(groups_.size(), kEnsBranches);
    branch_.resize(nb);
    ev_join_.resize(nb);
    for (size_t q = 0; q < nb; q++) {
      LMG_CUDA(cudaStreamCreateWithFlags(&branch_[q], cudaStreamNonBlocking));
      LMG_CUDA(cudaEventCreateWithFlags(&ev_join_[q], cudaEventDisableTiming));
    }
    LMG_CUDA(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
  }
  void release_branches() {
    for (auto b : branch_) cudaStreamDestroy(b);
    for (auto e : ev_join_) cudaEventDestroy(e);
    if (ev_fork_) cudaEventDestroy(ev_fork_);
    branch_.clear();
    ev_join_.clear();
    ev_fork_ = nullptr;
  }
  void matvec(const R *x, R *y, const int *active) { launch_groups(x, y, active, stream()); }
  void ensure_plans();
  void build_graph(R *V, size_t ldv);

  // systems, in the caller's order (u) and in the internal order (q)
  int nsys_ = 0, ntot_ = 0, npad_ = 0;
  std::vector<int> size_u_, geom_u_, uoff_, order_, ioff_, pad_;
  std::vector<double> height_u_;
  std::vector<std::unique_ptr<Group>> groups_;
  DeviceBuffer<int> imap_, psys_, sgeom_, off3_, nn_, active_, parity_, iter_, below_;
  DeviceBuffer<double> sheight_, normz_, alpha_, beta_;
  DeviceBuffer<R> pos_, in_, out_, ustage_, ustage2_, V_, w_, vcur_, z_, yb_, part_;
  DeviceBuffer<unsigned> tickets_;
  // estimate partial norms [system][chunk][2] and per-system tickets
  // (self-resetting, zeroed when allocated)
  int est_chunks_ = 1;
  DeviceBuffer<double> est_part_, step_part_;
  DeviceBuffer<unsigned> est_ticket_, step_ticket_;
  PinnedBuffer<R> pin_;
  PinnedBuffer<int> hflags_;
  MappedBuffer<double> hab_, coef_, err_;
  MappedBuffer<int> due_;
  // parameters
  bool init_ = false, have_pos_ = false, autotune_ = true;
  double eta_ = 0, a_ = 0, tol_ = 1e-4, t0_ = 0, r0_ = 0, rt0_ = 0;
  std::mt19937 eng_;
  std::vector<int> check_steps_;  // per internal system (registerRequiredStepsForConverge)
  // execution
  // cap_ only records the per-iteration graph (the caller's stream may be
  // the legacy default stream, which cannot be captured); the graph is then
  // launched on the working stream
  cudaStream_t stream_ = nullptr, own_ = nullptr, side_ = nullptr, cap_ = nullptr;
  // streams the groups' products run on side by side, and their fork / join
  std::vector<cudaStream_t> branch_;
  std::vector<cudaEvent_t> ev_join_;
  cudaEvent_t ev_fork_ = nullptr;
  bool have_stream_ = false, ev_ready_ = false;
  cudaEvent_t ev_iter_[2] = {nullptr, nullptr}, ev_check_ = nullptr, ev_side_ = nullptr;
  cudaEvent_t ev_t0_ = nullptr, ev_t1_ = nullptr;
  cudaGraphExec_t graph_ = nullptr;
  std::vector<const void *> graph_key_;
  int sms_ = 0;
  WorkerPool pool_;
};

template <class R>
void Ensemble<R>::set_systems(int nsys, const int *sizes, const int *geometry,
                              const double *wall_heights) {
  if (nsys < 1 || !sizes || !geometry)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] an ensemble needs nsys >= 1, sizes and geometries");
  long tot = 0, totpad = 0;
  for (int s = 0; s < nsys; s++) {
    if (sizes[s] < 1)
      throw Error(LMG_ERR_INVALID_ARGUMENT,
                  "[libmobility_gb300] every system needs at least one particle");
    if (geometry[s] != 0 && geometry[s] != 1)
      throw Error(LMG_ERR_INVALID_ARGUMENT,
                  "[libmobility_gb300] geometry must be 0 (open) or 1 (bottom wall)");
    tot += sizes[s];
    totpad += (sizes[s] + kPad - 1) / kPad * kPad;
  }
  if (totpad > (1L << 27))
    throw Error(LMG_ERR_INVALID_ARGUMENT, "[libmobility_gb300] ensemble too large");
  drop_graph();
  nsys_ = nsys;
  ntot_ = (int)tot;
  npad_ = (int)totpad;
  size_u_.assign(sizes, sizes + nsys);
  geom_u_.assign(geometry, geometry + nsys);
  height_u_.assign(nsys, 0.0);
  if (wall_heights)
    for (int s = 0; s < nsys; s++) height_u_[s] = geometry[s] ? wall_heights[s] : 0.0;
  uoff_.assign(nsys + 1, 0);
  for (int s = 0; s < nsys; s++) uoff_[s + 1] = uoff_[s] + sizes[s];
  auto bucket = [](int n) {
    int b = 0;
    while ((2 << b) <= n) b++;
    return b;  // 2^b <= n < 2^(b+1)
  };
  order_.resize(nsys);
  for (int s = 0; s < nsys; s++) order_[s] = s;
  std::stable_sort(order_.begin(), order_.end(), [&](int x, int y) {
    if (geometry[x] != geometry[y]) return geometry[x] < geometry[y];
    return bucket(sizes[x]) < bucket(sizes[y]);
  });
  ioff_.assign(nsys + 1, 0);
  pad_.assign(nsys, 0);
  for (int q = 0; q < nsys; q++) {
    const int s = order_[q];
    pad_[q] = (sizes[s] + kPad - 1) / kPad * kPad;
    ioff_[q + 1] = ioff_[q] + pad_[q];
  }
  // groups of consecutive internal systems with the same geometry and bucket
  groups_.clear();
  for (int q = 0; q < nsys;) {
    auto g = std::make_unique<Group>();
    const int s = order_[q];
    g->geom = geometry[s];
    g->bucket = bucket(sizes[s]);
    g->s0 = q;
    while (q < nsys && geometry[order_[q]] == g->geom && bucket(sizes[order_[q]]) == g->bucket)
      q++;
    g->s1 = q;
    g->p0 = ioff_[g->s0];
    g->p1 = ioff_[g->s1];
    std::vector<int> sb(g->s1 - g->s0 + 1);
    for (int k = g->s0; k <= g->s1; k++) sb[k - g->s0] = ioff_[k] - g->p0;
    for (int k = g->s0; k < g->s1; k++) {
      g->span = std::max(g->span, pad_[k]);
      g->work += (double)pad_[k] * pad_[k] * (g->geom ? 160.0 : 36.0);
    }
    int *d = g->sys_begin.ensure(sb.size());
    LMG_CUDA(cudaMemcpy(d, sb.data(), sb.size() * sizeof(int), cudaMemcpyHostToDevice));
    groups_.push_back(std::move(g));
  }
  // branches: the largest products first, each onto the least loaded stream
  {
    std::vector<int> ord(groups_.size());
    for (size_t q = 0; q < ord.size(); q++) ord[q] = (int)q;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int a, int b) { return groups_[a]->work > groups_[b]->work; });
    std::vector<double> load(std::min<size_t>(groups_.size(), kEnsBranches), 0.0);
    for (int q : ord) {
      const size_t b = (size_t)(std::min_element(load.begin(), load.end()) - load.begin());
      groups_[q]->branch = (int)b;
      load[b] += groups_[q]->work;
    }
  }
  // per internal particle: caller's particle index (-1 for dummies), system
  std::vector<int> imap(npad_, -1), psys(npad_), sgeom(nsys), off3(nsys), nn(nsys);
  std::vector<double> sh(nsys);
  for (int q = 0; q < nsys; q++) {
    const int s = order_[q];
    for (int k = 0; k < pad_[q]; k++) {
      psys[ioff_[q] + k] = q;
      if (k < sizes[s]) imap[ioff_[q] + k] = uoff_[s] + k;
    }
    sgeom[q] = geometry[s];
    sh[q] = height_u_[s];
    off3[q] = 3 * ioff_[q];
    nn[q] = 3 * sizes[s];
  }
  int maxn = 1;
  for (int q = 0; q < nsys; q++) maxn = std::max(maxn, nn[q]);
  est_chunks_ = (maxn + kEstChunk - 1) / kEstChunk;
  est_part_.ensure((size_t)nsys * est_chunks_ * 2);
  if (est_ticket_.count < (size_t)nsys) {
    est_ticket_.ensure(nsys);
    LMG_CUDA(cudaMemset(est_ticket_.ptr, 0, est_ticket_.count * sizeof(unsigned)));
  }
  step_part_.ensure((size_t)nsys * est_chunks_);
  if (step_ticket_.count < (size_t)nsys) {
    step_ticket_.ensure(nsys);
    LMG_CUDA(cudaMemset(step_ticket_.ptr, 0, step_ticket_.count * sizeof(unsigned)));
  }
  auto up = [](DeviceBuffer<int> &b, const std::vector<int> &v) {
    int *d = b.ensure(v.size());
    LMG_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice));
  };
  up(imap_, imap);
  up(psys_, psys);
  up(sgeom_, sgeom);
  up(off3_, off3);
  up(nn_, nn);
  double *dh = sheight_.ensure(nsys);
  LMG_CUDA(cudaMemcpy(dh, sh.data(), nsys * sizeof(double), cudaMemcpyHostToDevice));
  check_steps_.assign(nsys, 3);
  have_pos_ = false;
}

template <class R>
void Ensemble<R>::initialize(double eta, double a, double tol, uint64_t seed, bool autotune) {
  if (!(eta > 0) || !(a > 0) || !(tol > 0))
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] viscosity, radius and tolerance must be positive");
  eta_ = eta;
  a_ = a;
  tol_ = tol;
  autotune_ = autotune;
  // NBody::initialize, mobility.h:101-106
  t0_ = 1.0 / (6.0 * M_PI * eta * a);
  rt0_ = 1.0 / (8.0 * M_PI * eta * a * a);
  r0_ = 1.0 / (8.0 * M_PI * eta * a * a * a);
  if (seed == 0) seed = std::random_device()();
  eng_ = std::mt19937((uint32_t)seed);
  init_ = true;
  for (auto &g : groups_) g->tuned = false;
  drop_graph();
}

template <class R> void Ensemble<R>::set_positions(const void *pos, size_t n) {
  if (nsys_ == 0)
    throw Error(LMG_ERR_INVALID_ARGUMENT, "[libmobility_gb300] the ensemble has no systems");
  if (!init_)
    throw Error(LMG_ERR_NOT_INITIALIZED,
                "[libmobility_gb300] initialize the ensemble before setting positions");
  if (!pos || n != 3 * (size_t)ntot_)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] positions must hold 3 values per particle of the ensemble");
  cudaStream_t st = stream();
  const R *src = to_device_user(pos, n, ustage_);
  R *p = pos_.ensure(3 * (size_t)npad_);
  int *below = below_.ensure(1);
  LMG_CUDA(cudaMemsetAsync(below, 0, sizeof(int), st));
  ens_gather_pos<R><<<grid(npad_), 256, 0, st>>>(src, imap_.ptr, psys_.ptr, sgeom_.ptr,
                                                 sheight_.ptr, p, npad_, (R)(kDummyFar * a_),
                                                 (R)a_, below);
  count_launch();
  LMG_CUDA(cudaGetLastError());
  int hb = 0;
  LMG_CUDA(cudaMemcpyAsync(&hb, below, sizeof(int), cudaMemcpyDeviceToHost, st));
  LMG_CUDA(cudaStreamSynchronize(st));
  if (hb) {
    have_pos_ = false;
    throw Error(LMG_ERR_BELOW_WALL,
                "[Mobility] The center of a particle has fallen below the wall. Check your "
                "configuration and forces to ensure particle centers stay above the wall.");
  }
  have_pos_ = true;
}

template <class R> void Ensemble<R>::ensure_plans() {
  bool any = false;
  for (auto &gp : groups_) any = any || !gp->tuned;
  if (!any) return;
  cudaStream_t st = stream();
  R *x = in_.ensure(3 * (size_t)npad_);
  R *y = out_.ensure(3 * (size_t)npad_);
  LMG_CUDA(cudaMemsetAsync(x, 0, 3 * (size_t)npad_ * sizeof(R), st));
  for (auto &gp : groups_) {
    Group &g = *gp;
    if (g.tuned) continue;
    const int N = g.p1 - g.p0;
    MdotPlan base;
    LMG_CUDA(mdot_plan<R>(shape(g), N, g.span, sms(), 1, 0, base));
    g.plan = base;
    g.trials.clear();
    if (autotune_) {
      std::vector<int> cand = {base.nsplit};
      for (int c : {1, 2, 4, 8, 16, 32, 64})
        if (c <= std::max(1, g.span / kPad)) cand.push_back(c);
      // targets per thread (1 or 2) x source splits
      std::vector<MdotPlan> plans;
      for (int tpt : {1, 2}) {
        for (int c : cand) {
          MdotPlan p;
          if (mdot_plan<R>(shape(g), N, g.span, sms(), tpt, c, p) != cudaSuccess) {
            (void)cudaGetLastError();
            continue;
          }
          bool dup = false;
          for (auto &q : plans) dup = dup || (q.nsplit == p.nsplit && q.tpt == p.tpt);
          if (!dup) plans.push_back(p);
        }
      }
      double best = 1e300;
      for (auto &p : plans) {
        ensure_scratch(p);
        g.plan = p;
        launch_group(g, x, y, nullptr, st);  // warm-up
        LMG_CUDA(cudaEventRecord(ev_t0_, st));
        for (int r = 0; r < 3; r++) launch_group(g, x, y, nullptr, st);
        LMG_CUDA(cudaEventRecord(ev_t1_, st));
        LMG_CUDA(cudaEventSynchronize(ev_t1_));
        float ms = 0;
        LMG_CUDA(cudaEventElapsedTime(&ms, ev_t0_, ev_t1_));
        g.trials.emplace_back(p.tpt * 1000 + p.nsplit, ms / 3.0);
        if (ms < best) {
          best = ms;
          base = p;
        }
      }
      g.plan = base;
    }
    ensure_scratch(g.plan);
    g.tuned = true;
  }
  // disjoint scratch per group (the tuning above ran the groups one at a time
  // on the start of the buffers); new tickets start at zero
  size_t part = 0, tick = 0;
  for (auto &gp : groups_) {
    gp->part_off = part;
    gp->ticket_off = tick;
    part += gp->plan.part_elems;
    tick += gp->plan.tickets;
  }
  part_.ensure(std::max<size_t>(part, 1));
  if (tickets_.count < std::max<size_t>(tick, 1)) tickets_.ensure(std::max<size_t>(tick, 1));
  LMG_CUDA(cudaMemsetAsync(tickets_.ptr, 0, tickets_.count * sizeof(unsigned), st));
  drop_graph();
}

// The per-iteration work captured once (on a private stream): every group's
// all-pairs launch on the current basis vector (active systems only), the
// vector update of all systems, and the iteration counter.  Re-captured
// whenever a buffer or plan it names changes.
template <class R> void Ensemble<R>::build_graph(R *V, size_t ldv) {
  const std::vector<const void *> key = {V,          w_.ptr,     vcur_.ptr,   iter_.ptr,
                                         off3_.ptr,  nn_.ptr,    active_.ptr, normz_.ptr,
                                         alpha_.ptr, beta_.ptr,  hab_.device_ptr(),
                                         pos_.ptr,   part_.ptr,  tickets_.ptr,
                                         step_part_.ptr, step_ticket_.ptr};
  if (graph_ && graph_key_ == key) return;
  drop_graph();
  cudaStream_t st = cap_;
  cudaGraph_t g = nullptr;
  LMG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  try {
    launch_groups(vcur_.ptr, w_.ptr, active_.ptr, st);
    const dim3 cg(nsys_, est_chunks_);
    ens_step_alpha<R><<<cg, kEnsThreads, 0, st>>>(w_.ptr, V, ldv, iter_.ptr, off3_.ptr, nn_.ptr,
                                                  active_.ptr, beta_.ptr, alpha_.ptr, kEnsLimit,
                                                  step_part_.ptr, step_ticket_.ptr);
    ens_step_beta<R><<<cg, kEnsThreads, 0, st>>>(w_.ptr, V, ldv, iter_.ptr, off3_.ptr, nn_.ptr,
                                                 active_.ptr, normz_.ptr, alpha_.ptr, beta_.ptr,
                                                 kEnsLimit, hab_.device_ptr(), step_part_.ptr,
                                                 step_ticket_.ptr);
    ens_step_next<R><<<cg, kEnsThreads, 0, st>>>(w_.ptr, V, vcur_.ptr, ldv, iter_.ptr,
                                                 off3_.ptr, nn_.ptr, active_.ptr, beta_.ptr,
                                                 kEnsLimit);
    ens_iter_inc<<<1, 1, 0, st>>>(iter_.ptr);
    LMG_CUDA(cudaGetLastError());
  } catch (...) {
    cudaStreamEndCapture(st, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  // the group launches above were captured, not run
  g_launches.fetch_sub(groups_.size(), std::memory_order_relaxed);
  const cudaError_t e = cudaStreamEndCapture(st, &g);
  if (e != cudaSuccess) throw_cuda(e, "cudaStreamEndCapture");
  const cudaError_t ei = cudaGraphInstantiate(&graph_, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) {
    graph_ = nullptr;
    throw_cuda(ei, "cudaGraphInstantiate");
  }
  graph_key_ = key;
}

template <class R> void Ensemble<R>::mdot(const void *F, size_t nF, void *U, size_t nU) {
  NvtxRange nvtx_range_("lmg ensemble Mdot");
  require_ready();
  const size_t n3 = 3 * (size_t)ntot_;
  if (!F || nF != n3 || !U || nU != n3)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] forces and velocities must hold 3 values per particle");
  ensure_events();
  ensure_plans();
  cudaStream_t st = stream();
  const R *src = to_device_user(F, nF, ustage_);
  R *x = in_.ensure(3 * (size_t)npad_);
  R *y = out_.ensure(3 * (size_t)npad_);
  ens_gather_vec<R><<<grid(npad_), 256, 0, st>>>(src, imap_.ptr, x, npad_);
  count_launch();
  matvec(x, y, nullptr);
  const bool udev = ens_is_device_ptr(U);
  R *dst = udev ? static_cast<R *>(U) : ustage2_.ensure(n3);
  ens_scatter<R><<<grid(npad_), 256, 0, st>>>(y, 0, nullptr, imap_.ptr, psys_.ptr, dst, npad_,
                                              R(1), 0);
  count_launch();
  LMG_CUDA(cudaGetLastError());
  if (!udev) {
    R *h = pin_.ensure(n3);
    LMG_CUDA(cudaMemcpyAsync(h, dst, n3 * sizeof(R), cudaMemcpyDeviceToHost, st));
    LMG_CUDA(cudaStreamSynchronize(st));
    std::memcpy(U, h, n3 * sizeof(R));
  }
}

template <class R>
void Ensemble<R>::sqrt_mdot_w(const void *dW, size_t ndW, void *U, size_t nU, double pf,
                              int *its, double *errs, double *ms_out) {
  NvtxRange nvtx_range_("lmg ensemble sqrtMdotW");
  if (pf == 0) return;  // MobilityInterface.h:150
  require_ready();
  const size_t n3 = 3 * (size_t)ntot_;
  if (!U || nU != n3)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] velocities must hold 3 values per particle");
  if (dW && ndW != n3)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] dW must hold 3 values per particle");
  const auto t_start = std::chrono::steady_clock::now();
  ensure_events();
  ensure_plans();
  cudaStream_t st = stream();
  cudaStream_t sd = side_;
  const size_t ld = 3 * (size_t)npad_;
  const int lim = kEnsLimit;
  // storage; the basis is zeroed when allocated, and padding entries are
  // never written afterwards, so they stay 0
  const size_t vcount = (size_t)(lim + 1) * ld;
  const bool fresh = V_.count < vcount || vcur_.count < ld;
  R *V = V_.ensure(vcount);
  R *vc = vcur_.ensure(ld);
  if (fresh) {
    LMG_CUDA(cudaMemsetAsync(V, 0, vcount * sizeof(R), st));
    LMG_CUDA(cudaMemsetAsync(vc, 0, ld * sizeof(R), st));
  }
  w_.ensure(ld);
  R *z = z_.ensure(ld);
  R *yb = yb_.ensure(2 * ld);
  double *nz = normz_.ensure(nsys_);
  alpha_.ensure((size_t)nsys_ * lim);
  beta_.ensure((size_t)nsys_ * lim);
  hab_.ensure(2 * (size_t)nsys_ * lim);
  double *coef = coef_.ensure((size_t)nsys_ * lim);
  double *errh = err_.ensure(nsys_);
  int *due = due_.ensure(nsys_);
  int *act = active_.ensure(nsys_);
  int *par = parity_.ensure(nsys_);
  int *iter = iter_.ensure(1);
  // pinned flags: two slots for active-flag uploads used in turn (an upload
  // issued at one check has run before its slot is reused two checks later:
  // the host has waited meanwhile for an event recorded after it), and one
  // slot for the final buffer parities
  int *hf = hflags_.ensure(3 * (size_t)nsys_);
  int slot = 0;
  // noise in the caller's order, gathered
  const R *zu;
  if (dW) {
    zu = to_device_user(dW, ndW, ustage_);
  } else {
    R *d = ustage_.ensure(n3);
    const uint32_t s1 = std::uniform_int_distribution<uint32_t>(0, UINT32_MAX)(eng_);
    const uint32_t s2 = std::uniform_int_distribution<uint32_t>(0, UINT32_MAX)(eng_);
    gauss_fill_kernel<R><<<(int)std::min<size_t>((n3 / 4 + 256) / 256, 4096), 256, 0, st>>>(
        d, n3, s1, s2);
    count_launch();
    zu = d;
  }
  ens_gather_vec<R><<<grid(npad_), 256, 0, st>>>(zu, imap_.ptr, z, npad_);
  count_launch();
  // all systems active, iteration 0
  for (int q = 0; q < nsys_; q++) hf[q] = 1;
  LMG_CUDA(cudaMemcpyAsync(act, hf, nsys_ * sizeof(int), cudaMemcpyHostToDevice, st));
  LMG_CUDA(cudaMemsetAsync(iter, 0, sizeof(int), st));
  ens_first<R><<<nsys_, kEnsThreads, 0, st>>>(z, V, vc, off3_.ptr, nn_.ptr, nz);
  count_launch();
  LMG_CUDA(cudaGetLastError());
  build_graph(V, ld);
  const int per_iter = (int)groups_.size() + 4;  // groups, three step kernels, counter
  auto issue = [&](int i) {
    LMG_CUDA(cudaGraphLaunch(graph_, st));
    for (int k = 0; k < per_iter; k++) count_launch();
    LMG_CUDA(cudaEventRecord(ev_iter_[i & 1], st));
  };
  std::vector<int> active(nsys_, 1), have_prev(nsys_, 0), done(nsys_, -1);
  std::vector<double> err(nsys_, 0.0), when(nsys_, 0.0);
  std::vector<int> due_list;
  int nactive = nsys_;
  issue(0);
  for (int i = 0; i < lim; i++) {
    if (i + 1 < lim) issue(i + 1);  // the GPU runs ahead while this check is made
    due_list.clear();
    for (int q = 0; q < nsys_; q++)
      if (active[q] && i >= std::min(check_steps_[q], lim - 2)) due_list.push_back(q);
    if (due_list.empty()) continue;
    const int m = i + 1;
    LMG_CUDA(cudaEventSynchronize(ev_iter_[i & 1]));
    for (int q = 0; q < nsys_; q++) due[q] = 0;
    const double *hab = hab_.ptr;
    pool_.run((int)due_list.size(), [&](int k) {
      const int q = due_list[k];
      thread_local std::vector<double> al, be, d, e, q0, out, qw;
      thread_local std::vector<double2> cs;
      thread_local std::vector<int> idx;
      al.resize(m);
      be.resize(m);
      d.resize(m);
      e.resize(m);
      q0.resize(m);
      out.resize(m);
      qw.resize(18 * (size_t)m);
      for (int t = 0; t < m; t++) {
        al[t] = hab[2 * ((size_t)q * lim + t)];
        be[t] = hab[2 * ((size_t)q * lim + t) + 1];
      }
      // the quadrature form (O(nodes m), independent tridiagonal solves)
      // unless T is not positive definite or too ill-conditioned for it
      if (tridiag_sqrt_e1_quad(al.data(), be.data(), m, qw.data(), out.data()) == 0) {
        for (int t = 0; t < m; t++) coef[(size_t)q * lim + t] = out[t];
        return;
      }
      int rc = 2;
      // rotations logged: about m^2; the log grows if a case needs more
      for (size_t cap = 4 * (size_t)m * m + 1024; rc == 2 && cap <= 64 * (size_t)m * m + 1024;
           cap *= 4) {
        if (cs.size() < cap) {
          cs.resize(cap);
          idx.resize(cap);
        }
        RotLog log{cs.data(), idx.data(), (int)cap};
        rc = tridiag_sqrt_e1(al.data(), be.data(), m, d.data(), e.data(), q0.data(), log,
                             out.data());
      }
      for (int t = 0; t < m; t++) coef[(size_t)q * lim + t] = rc == 0 ? out[t] : std::nan("");
    });
    for (int q : due_list) due[q] = 1;
    LMG_CUDA(cudaStreamWaitEvent(sd, ev_iter_[i & 1], 0));
    ens_estimate<R><<<dim3(nsys_, est_chunks_), kEnsThreads, 0, sd>>>(
        V, ld, m, coef_.device_ptr(), lim, due_.device_ptr(), nz, off3_.ptr, nn_.ptr,
        yb + (size_t)(i & 1) * ld, yb + (size_t)((i + 1) & 1) * ld, est_part_.ptr,
        est_ticket_.ptr, err_.device_ptr());
    count_launch();
    LMG_CUDA(cudaGetLastError());
    LMG_CUDA(cudaEventRecord(ev_check_, sd));
    LMG_CUDA(cudaEventSynchronize(ev_check_));
    const double now_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start)
            .count();
    bool changed = false;
    for (int q : due_list) {
      if (have_prev[q]) {  // the reference never tests the first estimate
        err[q] = errh[q];
        if (std::isnan(err[q])) {
          LMG_CUDA(cudaStreamSynchronize(st));
          LMG_CUDA(cudaStreamSynchronize(sd));
          throw Error(LMG_ERR_NAN, "[Lanczos] Unknown error (found NaN in result guess)");
        }
        if (err[q] <= tol_) {
          active[q] = 0;
          done[q] = i;
          when[q] = now_ms;
          nactive--;
          changed = true;
          // registerRequiredStepsForConverge, per system
          if (i - 2 > check_steps_[q])
            check_steps_[q] += 1;
          else
            check_steps_[q] = std::max(1, check_steps_[q] - 2);
        }
      }
      have_prev[q] = 1;
    }
    if (nactive == 0) break;
    if (changed) {
      slot ^= 1;
      int *h = hf + (size_t)slot * nsys_;
      for (int q = 0; q < nsys_; q++) h[q] = active[q];
      LMG_CUDA(cudaMemcpyAsync(act, h, nsys_ * sizeof(int), cudaMemcpyHostToDevice, st));
    }
  }
  if (nactive > 0) {
    LMG_CUDA(cudaStreamSynchronize(st));
    LMG_CUDA(cudaStreamSynchronize(sd));
    throw Error(LMG_ERR_NO_CONVERGENCE, "[Lanczos] Could not converge");
  }
  // out += prefactor * y, each system from the buffer of its last check
  int *hp = hf + 2 * (size_t)nsys_;
  for (int q = 0; q < nsys_; q++) hp[q] = done[q] & 1;
  LMG_CUDA(cudaMemcpyAsync(par, hp, nsys_ * sizeof(int), cudaMemcpyHostToDevice, st));
  LMG_CUDA(cudaEventRecord(ev_side_, sd));
  LMG_CUDA(cudaStreamWaitEvent(st, ev_side_, 0));
  const bool udev = ens_is_device_ptr(U);
  R *dst;
  if (udev) {
    dst = static_cast<R *>(U);
  } else {
    dst = ustage2_.ensure(n3);
    R *h = pin_.ensure(n3);
    std::memcpy(h, U, n3 * sizeof(R));
    LMG_CUDA(cudaMemcpyAsync(dst, h, n3 * sizeof(R), cudaMemcpyHostToDevice, st));
  }
  ens_scatter<R><<<grid(npad_), 256, 0, st>>>(yb, ld, par, imap_.ptr, psys_.ptr, dst, npad_,
                                              (R)pf, 1);
  count_launch();
  LMG_CUDA(cudaGetLastError());
  if (!udev) {
    R *h = pin_.ensure(n3);
    LMG_CUDA(cudaMemcpyAsync(h, dst, n3 * sizeof(R), cudaMemcpyDeviceToHost, st));
    LMG_CUDA(cudaStreamSynchronize(st));
    std::memcpy(U, h, n3 * sizeof(R));
  } else {
    LMG_CUDA(cudaStreamSynchronize(st));
  }
  for (int q = 0; q < nsys_; q++) {
    const int s = order_[q];
    if (its) its[s] = done[q];
    if (errs) errs[s] = err[q];
    if (ms_out) ms_out[s] = when[q];
  }
}

template <class R> std::string Ensemble<R>::describe() const {
  std::ostringstream o;
  o << "{\"precision\": \"" << (sizeof(R) == 4 ? "float" : "double") << "\", \"systems\": "
    << nsys_ << ", \"particles\": " << ntot_ << ", \"padded_particles\": " << npad_
    << ", \"groups\": [";
  for (size_t k = 0; k < groups_.size(); k++) {
    const Group &g = *groups_[k];
    o << (k ? ", " : "") << "{\"geometry\": \"" << (g.geom ? "wall" : "open")
      << "\", \"size_range\": [" << (1 << g.bucket) << ", " << (2 << g.bucket) - 1
      << "], \"systems\": " << (g.s1 - g.s0) << ", \"padded_particles\": " << (g.p1 - g.p0)
      << ", \"tuned\": " << (g.tuned ? "true" : "false") << ", \"targets_per_tile\": "
      << g.plan.threads * g.plan.tpt << ", \"source_splits\": " << g.plan.nsplit
      << ", \"sources_per_split\": " << g.plan.chunk << ", \"trials_ms\": [";
    for (size_t t = 0; t < g.trials.size(); t++)
      o << (t ? ", " : "") << "[" << g.trials[t].first / 1000 << ", "
        << g.trials[t].first % 1000 << ", " << g.trials[t].second << "]";
    o << "]}";
  }
  o << "]}";
  return o.str();
}

}  // namespace

EnsembleBase *make_ensemble(int precision) {
  if (precision == LMG_PRECISION_DOUBLE) return new Ensemble<double>();
  if (precision == LMG_PRECISION_FLOAT) return new Ensemble<float>();
  throw Error(LMG_ERR_INVALID_ARGUMENT,
              "[libmobility_gb300] precision must be 0 (float) or 1 (double)");
}

}  // namespace lmg
