// SelfMobility on the same C ABI: the mobility is the identity scaled by
// 1/(6 pi eta a) (translation) and 1/(8 pi eta a^3) (rotation), with no
// hydrodynamic interaction between particles.  Follows libMobility
// solvers/SelfMobility/mobility.h:17-111, which computes on the host: so does
// this class (device buffers are staged through the host), and its noise is
// the reference's: std::normal_distribution<real>{0, 1} drawn from
// std::mt19937 seeded with the user seed (mobility.h:39-42, 91-109).
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "solver.hpp"

namespace lmg {

namespace {
bool on_device(const void *p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// host view of a caller buffer: device buffers are copied in (and back out)
template <class R> struct HostView {
  void *user;
  size_t n;
  bool dev;
  std::vector<R> tmp;
  R *ptr;
  HostView(const void *u, size_t n_, bool copy_in) : user(const_cast<void *>(u)), n(n_) {
    dev = on_device(u);
    if (dev) {
      tmp.resize(n);
      if (copy_in) LMG_CUDA(cudaMemcpy(tmp.data(), u, n * sizeof(R), cudaMemcpyDeviceToHost));
      ptr = tmp.data();
    } else {
      ptr = static_cast<R *>(user);
    }
  }
  void write_back() {
    if (dev) LMG_CUDA(cudaMemcpy(user, tmp.data(), n * sizeof(R), cudaMemcpyHostToDevice));
  }
};
}  // namespace

template <class R> class SelfMobility final : public SolverBase {
 public:
  SelfMobility(Periodicity x, Periodicity y, Periodicity z) : SolverBase(NoNBodyRules{}) {
    if (x != Periodicity::open || y != Periodicity::open || z != Periodicity::open)
      throw Error(LMG_ERR_INVALID_ARGUMENT, "[Mobility] This is an open boundary solver");
  }
  const char *precision() const override { return sizeof(R) == 4 ? "float" : "double"; }

  void init_self(uint64_t seed_in) {
    uint64_t seed = seed_in ? seed_in : std::random_device()();
    rng_ = std::mt19937((std::mt19937::result_type)seed);
    lin_ = (R)(t0_);
    ang_mob_ = (R)(r0_);
  }

  void set_positions(const void *, size_t n) override {
    N_ = (int64_t)(n / 3);  // SelfMobility only counts particles (mobility.h:56-59)
  }

  void mdot(const void *F, size_t nF, const void *T, size_t nT, void *U, size_t nU, void *W,
            size_t nW) override {
    if (!F) nF = 0;
    if (!T) nT = 0;
    const size_t n3 = 3 * (size_t)N_;
    if (nF > 0 && nF != n3)
      throw Error(LMG_ERR_INVALID_ARGUMENT, "The forces array must have size 3*N.");
    if (nT > 0 && nT != n3)
      throw Error(LMG_ERR_INVALID_ARGUMENT, "The torques array must have size 3*N.");
    if (!ang_ && nT > 0)
      throw Error(LMG_ERR_INVALID_ARGUMENT,
                  "The solver was configured without including angular velocities. "
                  "Set includeAngular to true when initializing if you want to use "
                  "torques");
    if (nF) {
      HostView<R> f(F, n3, true), u(U, n3, false);
      for (size_t i = 0; i < n3; i++) u.ptr[i] = f.ptr[i] * lin_;
      u.write_back();
    }
    if (nT && W && nW) {
      HostView<R> t(T, n3, true), w(W, n3, false);
      for (size_t i = 0; i < n3; i++) w.ptr[i] = t.ptr[i] * ang_mob_;
      w.write_back();
    }
  }

  void sqrt_mdot_w(void *U, size_t nU, void *W, size_t nW, double prefactor, const void *dW,
                   size_t ndW, int *iterations, double *residual) override {
    if (iterations) *iterations = 0;
    if (residual) *residual = 0;
    const size_t n3 = 3 * (size_t)N_;
    std::normal_distribution<R> d{0, 1};
    const R pf = (R)prefactor;
    const R *given = nullptr;
    std::vector<R> gz;
    if (dW) {
      HostView<R> z(dW, ndW, true);
      gz.assign(z.ptr, z.ptr + ndW);
      given = gz.data();
    }
    size_t k = 0;
    if (U && nU) {
      HostView<R> u(U, n3, true);
      for (size_t i = 0; i < n3; i++) {
        const R z = given ? given[k++] : d(rng_);
        u.ptr[i] += pf * std::sqrt(lin_) * z;
      }
      u.write_back();
    }
    if (W && nW) {
      HostView<R> w(W, n3, true);
      for (size_t i = 0; i < n3; i++) {
        const R z = given ? given[k++] : d(rng_);
        w.ptr[i] += pf * std::sqrt(ang_mob_) * z;
      }
      w.write_back();
    }
  }

  void div_m(void *, size_t, void *, size_t, double) override {}  // Mobility::divM default
  void clean() override {}
  void set_preconditioner(const std::string &kind, const float *, size_t) override {
    if (kind != "none")
      throw Error(LMG_ERR_INVALID_ARGUMENT,
                  "[libmobility_gb300] SelfMobility has no preconditioner");
  }
  void on_initialized(uint64_t user_seed) override { init_self(user_seed); }

 private:
  std::mt19937 rng_;
  R lin_ = 0, ang_mob_ = 0;
};

SolverBase *make_self_mobility(Periodicity x, Periodicity y, Periodicity z, int precision) {
  if (precision == LMG_PRECISION_DOUBLE) return new SelfMobility<double>(x, y, z);
  if (precision == LMG_PRECISION_FLOAT) return new SelfMobility<float>(x, y, z);
  throw Error(LMG_ERR_INVALID_ARGUMENT,
              "[libmobility_gb300] precision must be 0 (float) or 1 (double)");
}

}  // namespace lmg
