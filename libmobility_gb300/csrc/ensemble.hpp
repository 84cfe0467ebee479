// Ensembles of independent NBody systems of uneven size (open and bottom-wall
// geometries mixed): the object behind the lmg_ensemble_* entry points.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "common.hpp"

namespace lmg {

class EnsembleBase {
 public:
  virtual ~EnsembleBase() = default;
  std::string last_error;

  virtual void set_stream(cudaStream_t s) = 0;
  virtual void use_own_stream() = 0;
  virtual void set_systems(int nsys, const int *sizes, const int *geometry,
                           const double *wall_heights) = 0;
  virtual void initialize(double viscosity, double radius, double tolerance, uint64_t seed,
                          bool autotune) = 0;
  virtual void set_positions(const void *pos, size_t n) = 0;
  virtual void mdot(const void *F, size_t nF, void *U, size_t nU) = 0;
  virtual void sqrt_mdot_w(const void *dW, size_t ndW, void *U, size_t nU, double prefactor,
                           int *iterations, double *errors, double *completion_ms) = 0;
  virtual std::string describe() const = 0;
};

EnsembleBase *make_ensemble(int precision);

}  // namespace lmg
