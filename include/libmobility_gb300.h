/*
 * libmobility_gb300 -- C ABI of the GB300-native NBody mobility solver.
 *
 * One handle is one solver object with the behaviour of libMobility's
 * `NBody` class (solvers/NBody/mobility.h) behind the `libmobility::Mobility`
 * interface (include/MobilityInterface/MobilityInterface.h:56-224).  Every
 * entry point below replaces one member of that interface; the reference
 * location is cited beside each declaration.
 *
 * Conventions
 *   - Every call returns an lmg_status; 0 is success.  After a failure,
 *     lmg_last_error(h) holds the message (the reference's exception text
 *     where it has one, e.g. "...has fallen below the wall...").
 *   - Real-valued buffers hold `real` values: float for a handle created with
 *     LMG_PRECISION_FLOAT, double for LMG_PRECISION_DOUBLE (the reference's
 *     compile-time `real`, include/MobilityInterface/defines.h:5-14, made a
 *     run-time choice).
 *   - A buffer is a (pointer, count) pair: the count of `real` values, as in
 *     the reference's device_span (include/memory/container.h:24-57).  A count
 *     of 0 (or a NULL pointer) means the array is absent.
 *   - Pointers may be host memory or CUDA device memory of the current device;
 *     the library finds out which (cudaPointerGetAttributes) and stages host
 *     buffers itself, as the reference's device_adapter does
 *     (include/memory/container.h:59-110).  The caller keeps ownership of
 *     every buffer; the library never frees them.
 *   - Work is issued on the handle's CUDA stream (see lmg_set_stream).  Calls
 *     that take or return host memory, and calls that must report an error
 *     found on the GPU (setPositions, sqrtMdotW), synchronise that stream
 *     before returning; Mdot on device buffers does not.
 *   - A handle is not thread-safe; distinct handles are independent.
 */
#ifndef LIBMOBILITY_GB300_H
#define LIBMOBILITY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lmg_solver lmg_solver;

typedef enum {
  LMG_OK = 0,
  LMG_ERR_INVALID_ARGUMENT = 1, /* bad periodicity, shape, batch, parameter */
  LMG_ERR_NOT_INITIALIZED = 2,  /* initialize() has not been called */
  LMG_ERR_NO_POSITIONS = 3,     /* setPositions() has not been called */
  LMG_ERR_BELOW_WALL = 4,       /* a particle centre is below the wall */
  LMG_ERR_NO_CONVERGENCE = 5,   /* Lanczos reached its iteration limit */
  LMG_ERR_NAN = 6,              /* NaN in the Lanczos result estimate */
  LMG_ERR_TIMEOUT = 7,          /* a device-side wait ran out */
  LMG_ERR_CUDA = 8,             /* CUDA runtime error */
  LMG_ERR_NO_DEVICE = 9,        /* no CUDA device visible */
  LMG_ERR_INTERNAL = 10
} lmg_status;

typedef enum { LMG_PRECISION_FLOAT = 0, LMG_PRECISION_DOUBLE = 1 } lmg_precision;

/* Lanczos progress callback: iteration index and current residual, the
 * reference's Parameters::lanczosCallback (MobilityInterface.h:42). */
typedef void (*lmg_lanczos_callback)(int iteration, double residual, void *user);

/* Interface version string, LIBMOBILITYVERSION ("1.1"),
 * include/MobilityInterface/defines.h:4. */
const char *lmg_version(void);

/* Message of the last failed call on h (never NULL). */
const char *lmg_last_error(const lmg_solver *h);

/* NBody(Configuration) -- solvers/NBody/mobility.h:37-47 with the periodicity
 * strings of include/MobilityInterface/pythonify.h:38-61 ("open",
 * "single_wall", "two_walls", "periodic", "unspecified").  X and Y must be
 * "open"; Z "open" selects the open-boundary RPY kernel, "single_wall" the
 * Rotne-Prager-Blake kernel.  On failure *out is NULL and the message is
 * available from lmg_create_error(). */
lmg_status lmg_create(const char *periodicityX, const char *periodicityY,
                      const char *periodicityZ, int precision, lmg_solver **out);
const char *lmg_create_error(void);

/* SelfMobility(Configuration) -- solvers/SelfMobility/mobility.h:31-36: the
 * same handle API for the solver without hydrodynamic interactions (mobility
 * 1/(6 pi eta a) and 1/(8 pi eta a^3) times the identity, noise drawn on the
 * host exactly as the reference draws it).  All three periodicities must be
 * "open".  Its setParameters takes no effect (mobility.h:54). */
lmg_status lmg_create_self_mobility(const char *periodicityX, const char *periodicityY,
                                    const char *periodicityZ, int precision,
                                    lmg_solver **out);

/* Frees the handle and everything it owns. */
lmg_status lmg_destroy(lmg_solver *h);

/* Issue the handle's work on this CUDA stream.  cuda_stream is a
 * cudaStream_t used as given, so NULL/0 is CUDA's default stream;
 * LMG_OWN_STREAM selects the handle's private non-blocking stream (created on
 * first use), which is also what a handle uses before this is ever called.
 * The solver may use one more internal stream for work that overlaps the
 * matrix-vector products of Lanczos; it is joined back before a call
 * returns. */
#define LMG_OWN_STREAM ((void *)(intptr_t)-1)
lmg_status lmg_set_stream(lmg_solver *h, void *cuda_stream);

/* lanczos::Solver::setIterationHardLimit -- include/lanczos/LanczosAlgorithm.h:
 * 272-274.  Iteration limit of sqrtMdotW (default 200, at most 250); reaching
 * it is LMG_ERR_NO_CONVERGENCE ("[Lanczos] Could not converge"). */
lmg_status lmg_set_lanczos_iteration_limit(lmg_solver *h, int limit);

/* setParametersNBody -- solvers/NBody/mobility.h:78-97 and the Python
 * setParameters of solvers/NBody/python_wrapper.cu:50-61.  algorithm is one
 * of "fast", "naive", "block", "advise" (all run the same GB300 kernel;
 * anything else is an error).  Nbatch/NperBatch < 0 mean "all particles in
 * one batch".  has_wall_height says whether wallHeight was given: required for
 * a single wall, forbidden for open Z.  delta: random-finite-difference step
 * in units of the radius. */
lmg_status lmg_set_parameters_nbody(lmg_solver *h, const char *algorithm,
                                    int Nbatch, int NperBatch,
                                    int has_wall_height, double wallHeight,
                                    double delta);

/* Mobility::initialize + NBody::initialize -- MobilityInterface.h:102-114,
 * mobility.h:99-114.  seed 0 draws a random seed.  callback may be NULL. */
lmg_status lmg_initialize(lmg_solver *h, double viscosity,
                          double hydrodynamicRadius, int includeAngular,
                          double tolerance, uint64_t seed,
                          lmg_lanczos_callback callback, void *user);

/* NBody::setPositions -- mobility.h:116-162.  pos holds n_pos = 3N reals,
 * [x1,y1,z1,x2,...]. */
lmg_status lmg_set_positions(lmg_solver *h, const void *pos, size_t n_pos);

/* NBody::getNumberParticles -- mobility.h:164. */
lmg_status lmg_get_number_particles(const lmg_solver *h, int64_t *out);

/* Mobility::getIncludeAngular -- MobilityInterface.h:217. */
lmg_status lmg_get_include_angular(const lmg_solver *h, int *out);

/* NBody::Mdot -- mobility.h:166-182 / NbodyRPY.cu:254-287.  U (and W when
 * includeAngular) are OVERWRITTEN with M.[F;T]. */
lmg_status lmg_mdot(lmg_solver *h, const void *F, size_t nF, const void *T,
                    size_t nT, void *U, size_t nU, void *W, size_t nW);

/* Rows [row_begin, row_end) of NBody::Mdot (mobility.h:166-182): F and T hold
 * all N particles (3N values each, either may be NULL), U and W receive the
 * rows only (3 * (row_end - row_begin) values each, OVERWRITTEN).  Row i of
 * the result sums every particle of i's batch, exactly like lmg_mdot; it is
 * the matrix-vector product of one rank of a row-partitioned Lanczos solve
 * (the reference's Lanczos is single-device: include/lanczos/
 * LanczosAlgorithm.cu:173-232 calls the whole Mdot).  NBody solvers only. */
lmg_status lmg_mdot_rows(lmg_solver *h, int64_t row_begin, int64_t row_end,
                         const void *F, size_t nF, const void *T, size_t nT,
                         void *U, size_t nU, void *W, size_t nW);

/* Mobility::sqrtMdotW -- MobilityInterface.h:132-188 with the Lanczos solver
 * of include/lanczos/LanczosAlgorithm.cu:173-232.  ADDS prefactor*sqrt(M) dW
 * into U (and W), dW drawn from the handle's seeded generator. */
lmg_status lmg_sqrt_mdot_w(lmg_solver *h, void *U, size_t nU, void *W,
                           size_t nW, double prefactor);

/* Same with the Gaussian vector dW given by the caller (n_dW = 3N, or 6N with
 * includeAngular, in the layout [dW_F; dW_T]); the reference draws dW inside
 * (include/MobilityInterface/lanczos.h:43-58).  iterations / residual (may be
 * NULL) receive the Lanczos iteration index at return and the last
 * successive-iterate error. */
lmg_status lmg_sqrt_mdot_w_noise(lmg_solver *h, const void *dW, size_t n_dW,
                                 void *U, size_t nU, void *W, size_t nW,
                                 double prefactor, int *iterations,
                                 double *residual);

/* Mobility::LangevinVelocities -- MobilityInterface.h:191-206:
 * U,W = M.[F;T] (if F or T given) + sqrt(2 kbt/dt) sqrt(M) dW + kbt divM. */
lmg_status lmg_langevin_velocities(lmg_solver *h, double dt, double kbt,
                                   const void *F, size_t nF, const void *T,
                                   size_t nT, void *U, size_t nU, void *W,
                                   size_t nW);

/* NBody::divM -- mobility.h:184-236 (random finite differences,
 * include/MobilityInterface/random_finite_differences.h:30-63).  ADDS
 * prefactor * div M into U (and W); nothing for open Z. */
lmg_status lmg_div_m(lmg_solver *h, void *U, size_t nU, void *W, size_t nW,
                     double prefactor);

/* No counterpart in the reference: learned sparse preconditioner for
 * sqrtMdotW.  kind "none" (default: plain Lanczos as in the reference) or
 * "mlp": Lanczos then runs on S = P M P^T, where P approximates M^{-1/2}
 * row by row over each particle's 16 nearest neighbours (an MLP on their
 * relative positions), and the sample is P^{-1} S^{1/2} dW, whose covariance is
 * M exactly; P changes the iteration count, not the statistics.  params holds
 * the network (n_params floats, the layout of libmobility_gb300/precond.py).
 * Needs precision float; batches of fewer than 17 particles use plain
 * Lanczos. */
lmg_status lmg_set_preconditioner(lmg_solver *h, const char *kind, const float *params,
                                  size_t n_params);
/* Iterations of the last preconditioner solve P x = S^{1/2} dW. */
lmg_status lmg_get_preconditioner_solve_iterations(const lmg_solver *h, int *out);

/* Mobility::clean -- MobilityInterface.h:220-223: frees the solver's
 * Lanczos storage and scratch. */
lmg_status lmg_clean(lmg_solver *h);

/* Waits for the handle's stream. */
lmg_status lmg_synchronize(lmg_solver *h);

/* Precision of the handle: "float" or "double" (Mobility::precision,
 * MobilityInterface.h:73-77). */
const char *lmg_precision_name(const lmg_solver *h);

/* No counterpart in the reference.  Mdot (FP32) that allocates nothing, for
 * callers that may not allocate device memory: programs whose device memory is
 * owned by their own pool with no other allocations allowed, or loops that
 * cannot take the device-wide synchronisation of cudaMalloc/cudaFree.  No
 * handle: every input and output is a caller-owned DEVICE buffer of 3N floats
 * (positions measured from the wall, z = 0 at the wall, when single_wall;
 * no below-the-wall check is made); one of F and T may be NULL (not both: a
 * call without forces and torques is rejected), W is required with
 * includeAngular; U and W are overwritten as by lmg_mdot.  Buffers must live
 * on the current GPU.  NperBatch <= 0
 * means one batch.  The kernel's scratch is a static device array of
 * LMG_MDOT_NOALLOC_SCRATCH_BYTES held by every GPU that loads the library;
 * numberParticles above LMG_MDOT_NOALLOC_MAX_PARTICLES is rejected.  Every call
 * looks up the scratch address on the current device; the first call on a
 * device also loads the library's device code there (make it before any
 * stream capture); calls share the scratch, so calls that overlap on the GPU
 * race.
 * Work is issued on cuda_stream (0 = default stream), nothing is synchronised.
 * On failure a message is written to err (err_len bytes, may be NULL). */
#define LMG_MDOT_NOALLOC_SCRATCH_BYTES ((size_t)8 << 20)
#define LMG_MDOT_NOALLOC_MAX_PARTICLES ((int64_t)1 << 24)
lmg_status lmg_mdot_noalloc_f32(const float *pos, const float *F, const float *T,
                                float *U, float *W, int64_t numberParticles,
                                int64_t NperBatch, int single_wall, double viscosity,
                                double hydrodynamicRadius, int includeAngular,
                                void *cuda_stream, char *err, size_t err_len);

/* ------------------------------------------------------------------------
 * Ensembles: no counterpart in the reference, whose NBody batches
 * (Nbatch x NperBatch, mobility.h:52-60) are equal in size and share one
 * geometry.  An ensemble holds many independent systems of uneven size, each
 * open or above its own bottom wall, with one viscosity and radius, forces
 * only (no torques).  Every system behaves as its own NBody solver; Mdot and
 * sqrtMdotW run all systems together: one all-pairs launch per group of
 * systems of the same geometry and size bucket per matrix-vector product,
 * one launch for all systems' Lanczos vector updates, each system stopping
 * at its own convergence (LanczosAlgorithm.cu:202-222 per system).
 * Buffers follow the conventions above, all systems concatenated in the
 * order given to lmg_ensemble_set_systems (3 values per particle).
 * ------------------------------------------------------------------------ */
typedef struct lmg_ensemble lmg_ensemble;

lmg_status lmg_ensemble_create(int precision, lmg_ensemble **out);
lmg_status lmg_ensemble_destroy(lmg_ensemble *h);
const char *lmg_ensemble_last_error(const lmg_ensemble *h);
/* As lmg_set_stream. */
lmg_status lmg_ensemble_set_stream(lmg_ensemble *h, void *cuda_stream);
/* sizes[s] >= 1 particles; geometry[s] 0 = open, 1 = bottom wall;
 * wall_heights (may be NULL: 0) gives the wall position of wall systems
 * (ignored for open ones), as NBody's wallHeight. */
lmg_status lmg_ensemble_set_systems(lmg_ensemble *h, int nsys, const int *sizes,
                                    const int *geometry, const double *wall_heights);
/* As lmg_initialize without includeAngular.  autotune != 0 times the
 * candidate launch plans of each group of systems on first use and keeps the
 * fastest (plans differ only in summation order); 0 keeps the planner's. */
lmg_status lmg_ensemble_initialize(lmg_ensemble *h, double viscosity,
                                   double hydrodynamicRadius, double tolerance, uint64_t seed,
                                   int autotune);
/* As lmg_set_positions: every wall system is shifted by its wall height and
 * checked against its wall ("fallen below the wall"). */
lmg_status lmg_ensemble_set_positions(lmg_ensemble *h, const void *pos, size_t n);
/* U = M F per system; U is overwritten. */
lmg_status lmg_ensemble_mdot(lmg_ensemble *h, const void *F, size_t nF, void *U, size_t nU);
/* U += prefactor * M^{1/2} dW per system (dW NULL: noise drawn as
 * lmg_sqrt_mdot_w does, one stream for the whole ensemble).  Per system (in
 * the caller's order, each array may be NULL): Lanczos iterations, last
 * successive-iterate error, and the host time in ms from the start of the
 * call until that system's result was known. */
lmg_status lmg_ensemble_sqrt_mdot_w(lmg_ensemble *h, const void *dW, size_t ndW, void *U,
                                    size_t nU, double prefactor, int *iterations,
                                    double *errors, double *completion_ms);
/* Groups, their chosen plans and the timings behind them, as JSON text
 * (written to buf, at most len bytes with the terminating 0). */
lmg_status lmg_ensemble_describe(const lmg_ensemble *h, char *buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* LIBMOBILITY_GB300_H */
