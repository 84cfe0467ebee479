/*
 * libmobility_gb300::NBody -- this library as a libmobility::Mobility.
 *
 * The class a libMobility code base adds to run the NBody path on this
 * library behind the reference's own C++ interface: it derives from
 * libmobility::Mobility (include/MobilityInterface/MobilityInterface.h:56-224)
 * and forwards every member that the reference's NBody
 * (solvers/NBody/mobility.h:11-236) implements to the matching entry point of
 * libmobility_gb300.h.  A device_span becomes pointer + count; the library
 * finds out itself whether the memory is on the host or the device.
 *
 * It needs the reference's include/ directory on the include path (for
 * MobilityInterface.h) and links with -llmg_gb300.  Errors are thrown as
 * std::runtime_error with the library's message, which is the reference's
 * exception text where the reference has one.
 */
#pragma once

#include <cstdint>
#include <functional>
#include <optional>
#include <stdexcept>

#include <MobilityInterface/MobilityInterface.h>

#include "libmobility_gb300.h"

namespace libmobility_gb300 {

class NBody : public libmobility::Mobility {
 public:
  // NBody(Configuration) -- solvers/NBody/mobility.h:37-47
  explicit NBody(libmobility::Configuration c) {
    const lmg_status s =
        lmg_create(name(c.periodicityX), name(c.periodicityY), name(c.periodicityZ),
                   sizeof(libmobility::real) == 8 ? LMG_PRECISION_DOUBLE : LMG_PRECISION_FLOAT,
                   &h_);
    if (s != LMG_OK) throw std::runtime_error(lmg_create_error());
  }
  ~NBody() { lmg_destroy(h_); }
  NBody(const NBody &) = delete;
  NBody &operator=(const NBody &) = delete;

  // setParametersNBody -- solvers/NBody/mobility.h:78-97 (algorithm "fast",
  // "naive", "block" or "advise"; wallHeight required for a single wall)
  void setParametersNBody(const char *algorithm, int Nbatch, int NperBatch,
                          std::optional<double> wallHeight, double delta = 1e-3) {
    check(lmg_set_parameters_nbody(h_, algorithm, Nbatch, NperBatch, wallHeight.has_value(),
                                   wallHeight.value_or(0.0), delta));
  }

  // NBody::initialize -- mobility.h:99-114; the Lanczos callback receives
  // (iteration, residual) as Parameters::lanczosCallback does
  void initialize(libmobility::Parameters p) override {
    Mobility::initialize(p);
    callback_ = p.lanczosCallback;
    check(lmg_initialize(h_, p.viscosity, p.hydrodynamicRadius.at(0), p.includeAngular,
                         p.tolerance, p.seed, callback_ ? &forward_callback : nullptr, this));
  }

  // NBody::setPositions -- mobility.h:116-162
  void setPositions(libmobility::device_span<const libmobility::real> x) override {
    check(lmg_set_positions(h_, x.data(), x.size()));
  }

  // NBody::getNumberParticles -- mobility.h:164
  uint getNumberParticles() override {
    int64_t n = 0;
    check(lmg_get_number_particles(h_, &n));
    return static_cast<uint>(n);
  }

  // NBody::Mdot -- mobility.h:166-182 (U and W overwritten)
  void Mdot(libmobility::device_span<const libmobility::real> F,
            libmobility::device_span<const libmobility::real> T,
            libmobility::device_span<libmobility::real> U,
            libmobility::device_span<libmobility::real> W) override {
    check(lmg_mdot(h_, F.data(), F.size(), T.data(), T.size(), U.data(), U.size(), W.data(),
                   W.size()));
  }

  // Mobility::sqrtMdotW -- MobilityInterface.h:132-188 (adds prefactor B dW)
  void sqrtMdotW(libmobility::device_span<libmobility::real> U,
                 libmobility::device_span<libmobility::real> W,
                 libmobility::real prefactor) override {
    check(lmg_sqrt_mdot_w(h_, U.data(), U.size(), W.data(), W.size(), prefactor));
  }

  // Mobility::LangevinVelocities -- MobilityInterface.h:191-206, composed in
  // the library in the same order (Mdot, then sqrtMdotW and divM if kbt != 0)
  void LangevinVelocities(libmobility::real dt, libmobility::real kbt,
                          libmobility::device_span<const libmobility::real> F,
                          libmobility::device_span<const libmobility::real> T,
                          libmobility::device_span<libmobility::real> U,
                          libmobility::device_span<libmobility::real> W) override {
    check(lmg_langevin_velocities(h_, dt, kbt, F.data(), F.size(), T.data(), T.size(),
                                  U.data(), U.size(), W.data(), W.size()));
  }

  // NBody::divM -- mobility.h:184-236 (adds prefactor div M; zero for open Z)
  void divM(libmobility::device_span<libmobility::real> U,
            libmobility::device_span<libmobility::real> W,
            libmobility::real prefactor) override {
    check(lmg_div_m(h_, U.data(), U.size(), W.data(), W.size(), prefactor));
  }

  // Mobility::clean -- MobilityInterface.h:220-223
  void clean() override {
    Mobility::clean();
    check(lmg_clean(h_));
  }

  // The handle, for the library's own extras (lmg_set_stream,
  // lmg_set_preconditioner, lmg_sqrt_mdot_w_noise, ...).
  lmg_solver *handle() const { return h_; }

 private:
  lmg_solver *h_ = nullptr;
  std::function<void(int, float)> callback_;

  static void forward_callback(int iteration, double residual, void *self) {
    static_cast<NBody *>(self)->callback_(iteration, static_cast<float>(residual));
  }
  void check(lmg_status s) const {
    if (s != LMG_OK) throw std::runtime_error(lmg_last_error(h_));
  }
  // the periodicity strings of include/MobilityInterface/pythonify.h:38-61
  static const char *name(libmobility::periodicity_mode m) {
    switch (m) {
      case libmobility::periodicity_mode::open: return "open";
      case libmobility::periodicity_mode::single_wall: return "single_wall";
      case libmobility::periodicity_mode::two_walls: return "two_walls";
      case libmobility::periodicity_mode::periodic: return "periodic";
      default: return "unspecified";
    }
  }
};

}  // namespace libmobility_gb300
