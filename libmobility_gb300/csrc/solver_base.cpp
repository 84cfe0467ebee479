// Precision-independent part of the solver: parameter rules, seeding, error
// messages.  Every message that the reference's tests match is kept verbatim.
#include <cmath>
#include <limits>
#include <vector>

#include "solver.hpp"

namespace lmg {

Periodicity parse_periodicity(const std::string &s) {
  if (s == "open") return Periodicity::open;
  if (s == "unspecified") return Periodicity::unspecified;
  if (s == "single_wall") return Periodicity::single_wall;
  if (s == "two_walls") return Periodicity::two_walls;
  if (s == "periodic") return Periodicity::periodic;
  throw Error(LMG_ERR_INVALID_ARGUMENT, "[libMobility] Invalid periodicity");
}

// NBody::NBody, mobility.h:37-47
SolverBase::SolverBase(Periodicity x, Periodicity y, Periodicity z) {
  if (x != Periodicity::open || y != Periodicity::open)
    throw Error(LMG_ERR_INVALID_ARGUMENT, "[Mobility] NBody must be open in the plane");
  if (z == Periodicity::open)
    wall_ = false;
  else if (z == Periodicity::single_wall)
    wall_ = true;
  else
    throw Error(LMG_ERR_INVALID_ARGUMENT, "[Mobility] Invalid periodicity");
}

SolverBase::~SolverBase() {
  if (own_) cudaStreamDestroy(own_);
}

void SolverBase::set_parameters(int nbatch, int nper, std::optional<double> wall_height,
                                double delta) {
  if (wall_) {
    if (!wall_height)
      throw Error(LMG_ERR_INVALID_ARGUMENT,
                  "[Mobility] Wall height parameter is required for a bottom wall. "
                  "If you want to use a wall, set the wallHeight parameter.");
  } else if (wall_height) {
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[Mobility] Wall height parameter is only valid for bottom wall. If "
                "you want to use a wall, set periodicityZ to single_wall in the "
                "configuration.");
  }
  nbatch_ = nbatch;
  nper_ = nper;
  if (wall_height) wall_height_ = *wall_height;
  delta_ = delta;
}

void SolverBase::initialize(double viscosity, double radius, bool include_angular,
                            double tolerance, uint64_t seed, lmg_lanczos_callback cb,
                            void *user) {
  if (!(radius > 0) || !(viscosity > 0))
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] viscosity and hydrodynamicRadius must be positive");
  // Mobility::initialize cleans a solver that was already initialised
  if (initialized_) clean();
  a_ = radius;
  t0_ = 1.0 / (6.0 * M_PI * viscosity * radius);
  rt0_ = 1.0 / (8.0 * M_PI * viscosity * radius * radius);
  r0_ = 1.0 / (8.0 * M_PI * viscosity * radius * radius * radius);
  // seeding chain of mobility.h:107-111 and MobilityInterface.h:106-110
  const uint64_t user_seed = seed;
  if (seed == 0) seed = std::random_device()();
  nbody_rng_ = std::mt19937((std::mt19937::result_type)seed);
  uint64_t seed2 = nbody_rng_();
  if (seed2 == 0) seed2 = std::random_device()();
  base_rng_ = std::mt19937((std::mt19937::result_type)seed2);
  initialized_ = true;
  lanczos_seed_ = (uint32_t)base_rng_();
  tol_ = tolerance;
  cb_ = cb;
  cb_user_ = user;
  ang_ = include_angular;
  on_initialized(user_seed);
}

void SolverBase::check_positions_set(const char *who) const {
  (void)who;
  if (N_ <= 0)
    throw Error(LMG_ERR_NO_POSITIONS,
                "[Mobility] Positions have 0 particles. Did you call setPositions?");
}

// pythonify.h:109-149 (setup_arrays) and NbodyRPY.cu:234-235
void SolverBase::check_mdot_args(size_t nF, size_t nT, size_t nU, size_t nW) const {
  check_positions_set("Mdot");
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
  if (nU > 0 && nU != n3)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libMobility] The number of linear velocities does not match the "
                "number of particles");
  if (nW > 0 && nW != n3)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libMobility] The number of angular velocities does not match the "
                "number of particles");
}

void SolverBase::lanczos_register(int steps) {
  if (steps - 2 > check_steps_)
    check_steps_ += 1;
  else
    check_steps_ = std::max(1, check_steps_ - 2);
}

// Mobility::sqrtMdotW creates LanczosStochasticVelocities on first use
// (MobilityInterface.h:157-160) seeded with lanczosSeed.
void SolverBase::ensure_lanczos() {
  if (!lanczos_alive_) {
    lanczos_engine_ = std::mt19937(lanczos_seed_);
    check_steps_ = 3;
    lanczos_alive_ = true;
  }
}

// lanczos.h:49-50: two 32-bit seeds per call
void SolverBase::draw_noise_seeds(uint32_t &s1, uint32_t &s2) {
  s1 = std::uniform_int_distribution<uint32_t>(0, UINT32_MAX)(lanczos_engine_);
  s2 = std::uniform_int_distribution<uint32_t>(0, UINT32_MAX)(lanczos_engine_);
}

void SolverBase::langevin(double dt, double kbt, const void *F, size_t nF, const void *T,
                          size_t nT, void *U, size_t nU, void *W, size_t nW) {
  if ((F && nF) || (T && nT)) mdot(F, nF, T, nT, U, nU, W, nW);
  if (kbt != 0) {
    const double pf = std::sqrt(2.0 * kbt / dt);
    sqrt_mdot_w(U, nU, W, nW, pf, nullptr, 0, nullptr, nullptr);
    div_m(U, nU, W, nW, kbt);
  }
}

void SolverBase::set_stream(cudaStream_t s) {
  stream_ = s;
  have_stream_ = true;
  own_stream_ = false;
}

void SolverBase::use_own_stream() {
  have_stream_ = false;
  own_stream_ = false;
}

cudaStream_t SolverBase::stream() {
  if (!have_stream_) {
    if (!own_) LMG_CUDA(cudaStreamCreateWithFlags(&own_, cudaStreamNonBlocking));
    stream_ = own_;
    have_stream_ = true;
    own_stream_ = true;
  }
  return stream_;
}

// LanczosAlgorithm.h:272-274 (the reference default is 200)
void SolverBase::set_iteration_limit(int limit) {
  if (limit < 3 || limit > kMaxLanczosIterations)
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] the Lanczos iteration limit must be in [3, " +
                    std::to_string(kMaxLanczosIterations) + "]");
  hard_limit_ = limit;
}

void SolverBase::synchronize() {
  if (have_stream_) LMG_CUDA(cudaStreamSynchronize(stream_));
}

}  // namespace lmg
