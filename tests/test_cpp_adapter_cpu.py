"""The C++ adapter include/libmobility_gb300_mobility.hpp (this library as a
libmobility::Mobility) compiles against the reference's own interface header
(include/MobilityInterface/MobilityInterface.h), and the class it defines is
concrete: every pure virtual of the reference's interface is implemented.
Compile only (nvcc for sm_103a, no GPU needed); needs the reference checkout,
whose headers are not copied here.  The stand-ins of oracle/ref_shim supply
cblas/lapacke and the interface of UAMMD's Saru generator, which the
reference does not vendor."""
import shutil
import subprocess

import pytest

from conftest import REFERENCE, ROOT

TU = r"""
#include "libmobility_gb300_mobility.hpp"
#include <type_traits>
static_assert(!std::is_abstract_v<libmobility_gb300::NBody>,
              "a pure virtual of libmobility::Mobility is not implemented");
static_assert(std::is_base_of_v<libmobility::Mobility, libmobility_gb300::NBody>);
static_assert(!std::is_copy_constructible_v<libmobility_gb300::NBody>);
// the members a caller of the reference's NBody uses
using N = libmobility_gb300::NBody;
[[maybe_unused]] static auto p1 = &N::setParametersNBody;
[[maybe_unused]] static auto p2 = &N::handle;
#include <memory>
// the call sequence the integration notes show (compiled, not run)
[[maybe_unused]] static void usage(libmobility::device_span<const libmobility::real> positions,
                                   libmobility::device_span<const libmobility::real> forces,
                                   libmobility::device_span<const libmobility::real> torques,
                                   libmobility::device_span<libmobility::real> linear,
                                   libmobility::device_span<libmobility::real> angular) {
  libmobility::Configuration conf{libmobility::periodicity_mode::open,
                                  libmobility::periodicity_mode::open,
                                  libmobility::periodicity_mode::single_wall};
  auto solver = std::make_unique<libmobility_gb300::NBody>(conf);
  solver->setParametersNBody("advise", -1, -1, /*wallHeight=*/0.0, 1e-3);
  libmobility::Parameters par;
  par.hydrodynamicRadius = {1.0};
  par.viscosity = 1.0;
  par.tolerance = 1e-4;
  par.includeAngular = true;
  solver->initialize(par);
  solver->setPositions(positions);
  solver->Mdot(forces, torques, linear, angular);
  solver->sqrtMdotW(linear, angular, 1.0);
}
"""


def test_adapter_compiles_against_reference_interface(tmp_path):
    iface = REFERENCE / "include" / "MobilityInterface" / "MobilityInterface.h"
    if not iface.exists():
        pytest.skip("reference checkout not present on this machine")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "adapter.cu"
    src.write_text(TU)
    cmd = [nvcc, "-std=c++20", "--expt-relaxed-constexpr", "-extended-lambda",
           "-gencode", "arch=compute_103a,code=sm_103a",
           f"-I{ROOT / 'include'}", f"-I{ROOT / 'oracle' / 'ref_shim'}",
           f"-I{REFERENCE / 'include'}", "-c", str(src), "-o", str(tmp_path / "adapter.o")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
