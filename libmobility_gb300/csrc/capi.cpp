// extern "C" boundary: every entry point of include/libmobility_gb300.h.
// Exceptions never cross it; they become an lmg_status plus a message.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>

#include "ensemble.hpp"
#include "solver.hpp"

struct lmg_solver {
  std::unique_ptr<lmg::SolverBase> impl;
};

struct lmg_ensemble {
  std::unique_ptr<lmg::EnsembleBase> impl;
};

namespace {
thread_local std::string g_create_error;

template <class H, class F> lmg_status guarded(H *h, F &&f) {
  if (!h || !h->impl) return LMG_ERR_INVALID_ARGUMENT;
  try {
    f(*h->impl);
    h->impl->last_error.clear();
    return LMG_OK;
  } catch (const lmg::Error &e) {
    h->impl->last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    h->impl->last_error = "[libmobility_gb300] out of host memory";
    return LMG_ERR_INTERNAL;
  } catch (const std::exception &e) {
    h->impl->last_error = e.what();
    return LMG_ERR_INTERNAL;
  }
}
}  // namespace

extern "C" {

const char *lmg_version(void) { return "1.1"; }

const char *lmg_last_error(const lmg_solver *h) {
  if (!h || !h->impl) return "invalid handle";
  return h->impl->last_error.c_str();
}

const char *lmg_create_error(void) { return g_create_error.c_str(); }

lmg_status lmg_create(const char *px, const char *py, const char *pz, int precision,
                      lmg_solver **out) {
  if (!out) return LMG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  try {
    if (!px || !py || !pz) throw lmg::Error(LMG_ERR_INVALID_ARGUMENT, "[libMobility] Invalid periodicity");
    auto x = lmg::parse_periodicity(px);
    auto y = lmg::parse_periodicity(py);
    auto z = lmg::parse_periodicity(pz);
    auto *h = new lmg_solver;
    h->impl.reset(lmg::make_solver(x, y, z, precision));
    *out = h;
    g_create_error.clear();
    return LMG_OK;
  } catch (const lmg::Error &e) {
    g_create_error = e.what();
    return e.code;
  } catch (const std::exception &e) {
    g_create_error = e.what();
    return LMG_ERR_INTERNAL;
  }
}

lmg_status lmg_create_self_mobility(const char *px, const char *py, const char *pz,
                                    int precision, lmg_solver **out) {
  if (!out) return LMG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  try {
    if (!px || !py || !pz) throw lmg::Error(LMG_ERR_INVALID_ARGUMENT, "[libMobility] Invalid periodicity");
    auto x = lmg::parse_periodicity(px);
    auto y = lmg::parse_periodicity(py);
    auto z = lmg::parse_periodicity(pz);
    auto *h = new lmg_solver;
    h->impl.reset(lmg::make_self_mobility(x, y, z, precision));
    *out = h;
    g_create_error.clear();
    return LMG_OK;
  } catch (const lmg::Error &e) {
    g_create_error = e.what();
    return e.code;
  } catch (const std::exception &e) {
    g_create_error = e.what();
    return LMG_ERR_INTERNAL;
  }
}

lmg_status lmg_destroy(lmg_solver *h) {
  if (!h) return LMG_ERR_INVALID_ARGUMENT;
  delete h;
  return LMG_OK;
}

lmg_status lmg_set_stream(lmg_solver *h, void *s) {
  return guarded(h, [&](lmg::SolverBase &m) {
    if (s == LMG_OWN_STREAM)
      m.use_own_stream();
    else
      m.set_stream((cudaStream_t)s);
  });
}

lmg_status lmg_set_lanczos_iteration_limit(lmg_solver *h, int limit) {
  return guarded(h, [&](lmg::SolverBase &m) { m.set_iteration_limit(limit); });
}

lmg_status lmg_set_parameters_nbody(lmg_solver *h, const char *algorithm, int Nbatch,
                                    int NperBatch, int has_wall_height, double wallHeight,
                                    double delta) {
  return guarded(h, [&](lmg::SolverBase &m) {
    // string2NBodyAlgorithm, solvers/NBody/python_wrapper.cu:35-47.  All four
    // schedules run the same GB300 kernel.
    std::string a = algorithm ? algorithm : "advise";
    if (a != "naive" && a != "fast" && a != "block" && a != "advise")
      throw lmg::Error(LMG_ERR_INVALID_ARGUMENT, "Invalid algorithm selected");
    std::optional<double> wh;
    if (has_wall_height) wh = wallHeight;
    m.set_parameters(Nbatch, NperBatch, wh, delta);
  });
}

lmg_status lmg_initialize(lmg_solver *h, double viscosity, double radius, int includeAngular,
                          double tolerance, uint64_t seed, lmg_lanczos_callback cb, void *user) {
  return guarded(h, [&](lmg::SolverBase &m) {
    m.initialize(viscosity, radius, includeAngular != 0, tolerance, seed, cb, user);
  });
}

lmg_status lmg_set_positions(lmg_solver *h, const void *pos, size_t n) {
  return guarded(h, [&](lmg::SolverBase &m) { m.set_positions(pos, pos ? n : 0); });
}

lmg_status lmg_get_number_particles(const lmg_solver *h, int64_t *out) {
  if (!h || !h->impl || !out) return LMG_ERR_INVALID_ARGUMENT;
  *out = h->impl->number_particles();
  return LMG_OK;
}

lmg_status lmg_get_include_angular(const lmg_solver *h, int *out) {
  if (!h || !h->impl || !out) return LMG_ERR_INVALID_ARGUMENT;
  *out = h->impl->include_angular() ? 1 : 0;
  return LMG_OK;
}

lmg_status lmg_mdot(lmg_solver *h, const void *F, size_t nF, const void *T, size_t nT, void *U,
                    size_t nU, void *W, size_t nW) {
  return guarded(h, [&](lmg::SolverBase &m) { m.mdot(F, nF, T, nT, U, nU, W, nW); });
}

lmg_status lmg_mdot_rows(lmg_solver *h, int64_t row_begin, int64_t row_end, const void *F,
                         size_t nF, const void *T, size_t nT, void *U, size_t nU, void *W,
                         size_t nW) {
  return guarded(h, [&](lmg::SolverBase &m) {
    m.mdot_rows(row_begin, row_end, F, nF, T, nT, U, nU, W, nW);
  });
}

lmg_status lmg_sqrt_mdot_w(lmg_solver *h, void *U, size_t nU, void *W, size_t nW,
                           double prefactor) {
  return guarded(h, [&](lmg::SolverBase &m) {
    m.sqrt_mdot_w(U, nU, W, nW, prefactor, nullptr, 0, nullptr, nullptr);
  });
}

lmg_status lmg_sqrt_mdot_w_noise(lmg_solver *h, const void *dW, size_t n_dW, void *U, size_t nU,
                                 void *W, size_t nW, double prefactor, int *iterations,
                                 double *residual) {
  return guarded(h, [&](lmg::SolverBase &m) {
    if (!dW || n_dW == 0)
      throw lmg::Error(LMG_ERR_INVALID_ARGUMENT, "[libmobility_gb300] dW is required");
    m.sqrt_mdot_w(U, nU, W, nW, prefactor, dW, n_dW, iterations, residual);
  });
}

lmg_status lmg_langevin_velocities(lmg_solver *h, double dt, double kbt, const void *F,
                                   size_t nF, const void *T, size_t nT, void *U, size_t nU,
                                   void *W, size_t nW) {
  return guarded(h, [&](lmg::SolverBase &m) { m.langevin(dt, kbt, F, nF, T, nT, U, nU, W, nW); });
}

lmg_status lmg_div_m(lmg_solver *h, void *U, size_t nU, void *W, size_t nW, double prefactor) {
  return guarded(h, [&](lmg::SolverBase &m) { m.div_m(U, nU, W, nW, prefactor); });
}

lmg_status lmg_set_preconditioner(lmg_solver *h, const char *kind, const float *params,
                                  size_t n_params) {
  return guarded(h, [&](lmg::SolverBase &m) {
    m.set_preconditioner(kind ? kind : "none", params, n_params);
  });
}

lmg_status lmg_get_preconditioner_solve_iterations(const lmg_solver *h, int *out) {
  if (!h || !h->impl || !out) return LMG_ERR_INVALID_ARGUMENT;
  *out = h->impl->last_solve_iterations();
  return LMG_OK;
}

lmg_status lmg_clean(lmg_solver *h) {
  return guarded(h, [&](lmg::SolverBase &m) { m.clean(); });
}

lmg_status lmg_synchronize(lmg_solver *h) {
  return guarded(h, [&](lmg::SolverBase &m) { m.synchronize(); });
}

const char *lmg_precision_name(const lmg_solver *h) {
  if (!h || !h->impl) return "";
  return h->impl->precision();
}

// Internal test hook (not part of the public header): FP64 T^{1/2} e1 of a
// symmetric tridiagonal matrix with the solver's own QL routine, on the host.
int lmg_internal_tridiag_sqrt_e1(const double *alpha, const double *beta, int m, double *out) {
  return lmg::tridiag_sqrt_e1_host(alpha, beta, m, out);
}

// The quadrature form used by the ensembles (0, or 2: use the exact form).
int lmg_internal_tridiag_sqrt_e1_quad(const double *alpha, const double *beta, int m,
                                      double *out) {
  return lmg::tridiag_sqrt_e1_quad_host(alpha, beta, m, out);
}

// Internal measurement hooks (not part of the public header): switch the
// Lanczos phase timing on or off (either resets the sums), and read the sums
// as out[10] = {vector_ms, vector_bytes, check_ms, check_bytes, iterations,
// checks, solves, operator_ms, build_ms, psolve_ms}.
int lmg_internal_lanczos_phase_timing(lmg_solver *h, int on) {
  return guarded(h, [&](lmg::SolverBase &m) { m.set_phase_timing(on != 0); });
}

int lmg_internal_lanczos_phase_times(lmg_solver *h, double *out) {
  if (!h || !h->impl || !out) return LMG_ERR_INVALID_ARGUMENT;
  const auto &p = h->impl->phase_times();
  const double v[10] = {p.vector_ms,         p.vector_bytes,   p.check_ms,
                        p.check_bytes,       (double)p.iterations, (double)p.checks,
                        (double)p.solves,    p.operator_ms,    p.build_ms,
                        p.psolve_ms};
  for (int q = 0; q < 10; q++) out[q] = v[q];
  return LMG_OK;
}


lmg_status lmg_ensemble_create(int precision, lmg_ensemble **out) {
  if (!out) return LMG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  try {
    auto *h = new lmg_ensemble;
    h->impl.reset(lmg::make_ensemble(precision));
    *out = h;
    g_create_error.clear();
    return LMG_OK;
  } catch (const lmg::Error &e) {
    g_create_error = e.what();
    return e.code;
  } catch (const std::exception &e) {
    g_create_error = e.what();
    return LMG_ERR_INTERNAL;
  }
}

lmg_status lmg_ensemble_destroy(lmg_ensemble *h) {
  delete h;
  return LMG_OK;
}

const char *lmg_ensemble_last_error(const lmg_ensemble *h) {
  if (!h || !h->impl) return "invalid handle";
  return h->impl->last_error.c_str();
}

lmg_status lmg_ensemble_set_stream(lmg_ensemble *h, void *s) {
  return guarded(h, [&](lmg::EnsembleBase &m) {
    if (s == LMG_OWN_STREAM)
      m.use_own_stream();
    else
      m.set_stream((cudaStream_t)s);
  });
}

lmg_status lmg_ensemble_set_systems(lmg_ensemble *h, int nsys, const int *sizes,
                                    const int *geometry, const double *wall_heights) {
  return guarded(h, [&](lmg::EnsembleBase &m) {
    m.set_systems(nsys, sizes, geometry, wall_heights);
  });
}

lmg_status lmg_ensemble_initialize(lmg_ensemble *h, double viscosity,
                                   double hydrodynamicRadius, double tolerance, uint64_t seed,
                                   int autotune) {
  return guarded(h, [&](lmg::EnsembleBase &m) {
    m.initialize(viscosity, hydrodynamicRadius, tolerance, seed, autotune != 0);
  });
}

lmg_status lmg_ensemble_set_positions(lmg_ensemble *h, const void *pos, size_t n) {
  return guarded(h, [&](lmg::EnsembleBase &m) { m.set_positions(pos, n); });
}

lmg_status lmg_ensemble_mdot(lmg_ensemble *h, const void *F, size_t nF, void *U, size_t nU) {
  return guarded(h, [&](lmg::EnsembleBase &m) { m.mdot(F, nF, U, nU); });
}

lmg_status lmg_ensemble_sqrt_mdot_w(lmg_ensemble *h, const void *dW, size_t ndW, void *U,
                                    size_t nU, double prefactor, int *iterations,
                                    double *errors, double *completion_ms) {
  return guarded(h, [&](lmg::EnsembleBase &m) {
    m.sqrt_mdot_w(dW, ndW, U, nU, prefactor, iterations, errors, completion_ms);
  });
}

lmg_status lmg_ensemble_describe(const lmg_ensemble *h, char *buf, size_t len) {
  if (!h || !h->impl || !buf || len == 0) return LMG_ERR_INVALID_ARGUMENT;
  const std::string d = h->impl->describe();
  const size_t k = std::min(len - 1, d.size());
  std::memcpy(buf, d.data(), k);
  buf[k] = 0;
  return d.size() < len ? LMG_OK : LMG_ERR_INVALID_ARGUMENT;
}

}  // extern "C"
