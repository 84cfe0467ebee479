// Host C++ mirror of libMobility's Mobility interface and NBody solver.
//
//   libmobility::Mobility      include/MobilityInterface/MobilityInterface.h:56-224
//   NBody                      solvers/NBody/mobility.h:11-237
//
// The non-numeric behaviour (parameter rules, error messages, seeding chain,
// argument validation) lives in SolverBase and is identical for both
// precisions; the numeric work is in Solver<R> (solver.cu).  Validation that
// needs no GPU runs before any CUDA call, so it also works on a machine
// without one.
#pragma once
#include <cstdint>
#include <optional>
#include <random>
#include <string>

#include "common.hpp"

namespace lmg {

// Size of the FP64 scalar arrays of a Lanczos solve (the iteration limit can
// be raised up to this; the reference default is 200).
constexpr int kMaxLanczosIterations = 250;

enum class Periodicity { single_wall, two_walls, open, periodic, unspecified };

Periodicity parse_periodicity(const std::string &s);  // pythonify.h:38-52

class SolverBase {
 public:
  explicit SolverBase(Periodicity x, Periodicity y, Periodicity z);
  struct NoNBodyRules {};
  explicit SolverBase(NoNBodyRules) {}
  virtual ~SolverBase();

  // NBody::setParametersNBody, mobility.h:78-97 (algorithm already parsed)
  void set_parameters(int nbatch, int nper, std::optional<double> wall_height, double delta);
  // NBody::initialize + Mobility::initialize, mobility.h:99-114,
  // MobilityInterface.h:102-114
  void initialize(double viscosity, double radius, bool include_angular, double tolerance,
                  uint64_t seed, lmg_lanczos_callback cb, void *user);

  virtual void set_positions(const void *pos, size_t n) = 0;
  virtual void mdot(const void *F, size_t nF, const void *T, size_t nT, void *U, size_t nU,
                    void *W, size_t nW) = 0;
  // Rows [row_begin, row_end) of M.[F;T] (F, T of all N particles; U, W of
  // the rows only): the product of one rank of a row-partitioned solve.
  virtual void mdot_rows(int64_t row_begin, int64_t row_end, const void *F, size_t nF,
                         const void *T, size_t nT, void *U, size_t nU, void *W, size_t nW) {
    (void)row_begin; (void)row_end; (void)F; (void)nF; (void)T; (void)nT;
    (void)U; (void)nU; (void)W; (void)nW;
    throw Error(LMG_ERR_INVALID_ARGUMENT,
                "[libmobility_gb300] row products are available for NBody solvers only");
  }
  virtual void sqrt_mdot_w(void *U, size_t nU, void *W, size_t nW, double prefactor,
                           const void *dW, size_t ndW, int *iterations, double *residual) = 0;
  virtual void div_m(void *U, size_t nU, void *W, size_t nW, double prefactor) = 0;
  virtual void clean() = 0;
  virtual const char *precision() const = 0;
  // learned sparse preconditioner for sqrtMdotW (no counterpart in the
  // reference): kind "none" or "mlp" with the network's parameters
  virtual void set_preconditioner(const std::string &kind, const float *params, size_t n) = 0;
  int last_solve_iterations() const { return last_inner_iters_; }
  // Lanczos phase timing (no counterpart in the reference), off by default:
  // device time of the Krylov vector updates that follow each matvec (on the
  // solver stream) and of the convergence checks (estimate y = |z| V c and
  // the error norm, on the side stream, overlapping the next matvec), with
  // the algorithmic bytes each moves, summed over converged solves.
  struct PhaseTimes {
    double vector_ms = 0, vector_bytes = 0, check_ms = 0, check_bytes = 0;
    long iterations = 0, checks = 0, solves = 0;
    // the operator of each iteration (M v, or P M P^T v), and with the
    // learned preconditioner its build and the final P solve (spans on the
    // solver stream, idle gaps included)
    double operator_ms = 0, build_ms = 0, psolve_ms = 0;
  };
  void set_phase_timing(bool on) {
    timing_ = on;
    phase_ = PhaseTimes{};
  }
  const PhaseTimes &phase_times() const { return phase_; }
  // called at the end of initialize() with the seed as the caller gave it
  virtual void on_initialized(uint64_t user_seed) { (void)user_seed; }

  // Mobility::LangevinVelocities, MobilityInterface.h:191-206
  void langevin(double dt, double kbt, const void *F, size_t nF, const void *T, size_t nT,
                void *U, size_t nU, void *W, size_t nW);

  int64_t number_particles() const { return N_; }
  bool include_angular() const { return ang_; }
  void set_stream(cudaStream_t s);   // s is used as given (0 = default stream)
  void use_own_stream();
  cudaStream_t stream();
  void set_iteration_limit(int limit);  // lanczos::Solver::setIterationHardLimit
  void synchronize();

  std::string last_error;

 protected:
  bool wall_ = false;
  // setParametersNBody
  int nbatch_ = -1, nper_ = -1;
  double wall_height_ = 0.0;
  double delta_ = 1e-3;
  // initialize
  bool initialized_ = false;
  double a_ = 1.0, t0_ = 0, r0_ = 0, rt0_ = 0, tol_ = 1e-4;
  bool ang_ = false;
  std::mt19937 nbody_rng_;   // NBody::rng, draws the divM seeds
  std::mt19937 base_rng_;    // Mobility::rng
  uint32_t lanczos_seed_ = 0;
  // LanczosStochasticVelocities state (lanczos.h:26-59), recreated after clean()
  bool lanczos_alive_ = false;
  std::mt19937 lanczos_engine_;
  int check_steps_ = 3;      // lanczos::Solver::check_convergence_steps
  int hard_limit_ = 200;     // lanczos::Solver::iterationHardLimit
  lmg_lanczos_callback cb_ = nullptr;
  int last_inner_iters_ = 0;  // BiCGSTAB iterations of the last preconditioned solve
  bool timing_ = false;
  PhaseTimes phase_;
  void *cb_user_ = nullptr;
  // positions
  int64_t N_ = 0;
  int batch_count() const { return nbatch_ < 0 ? 1 : nbatch_; }
  int batch_size() const { return nper_ < 0 ? (int)N_ : nper_; }
  // stream: the caller's (set_stream, 0 = CUDA default stream) or, until
  // one is set, a private non-blocking stream created on first use
  cudaStream_t stream_ = nullptr;
  bool have_stream_ = false;
  bool own_stream_ = false;
  cudaStream_t own_ = nullptr;

  // shared argument checks (messages of pythonify.h / mobility.h)
  void check_positions_set(const char *who) const;
  void check_mdot_args(size_t nF, size_t nT, size_t nU, size_t nW) const;
  void lanczos_register(int steps);  // LanczosAlgorithm.cu:224-232
  void ensure_lanczos();
  void draw_noise_seeds(uint32_t &s1, uint32_t &s2);
};

SolverBase *make_solver(Periodicity x, Periodicity y, Periodicity z, int precision);
// SelfMobility (solvers/SelfMobility/mobility.h): no hydrodynamic interactions
SolverBase *make_self_mobility(Periodicity x, Periodicity y, Periodicity z, int precision);

// internal test hook: T^{1/2} e1 for a symmetric tridiagonal matrix (FP64,
// host build of the device solver).  Returns 0 on success.
int tridiag_sqrt_e1_host(const double *alpha, const double *beta, int m, double *out);
// the same by quadrature (the ensemble's routine): 0, or 2 when the caller
// must fall back to the exact one
int tridiag_sqrt_e1_quad_host(const double *alpha, const double *beta, int m, double *out);

}  // namespace lmg
