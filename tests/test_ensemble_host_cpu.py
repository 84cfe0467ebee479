"""Host-side rules of the batched ensemble, checked without a GPU: every
argument error is raised before any device work (the same checks the GPU
test of the ensemble makes on a device)."""
import pytest


@pytest.fixture(scope="module")
def Ensemble():
    from libmobility_gb300 import _build
    _build.build()
    from libmobility_gb300.ensemble import Ensemble
    return Ensemble


def test_precision_must_be_float_or_double(Ensemble):
    with pytest.raises(RuntimeError, match="precision"):
        Ensemble(precision="half")


@pytest.mark.parametrize("sizes,geometry,heights,match", [
    ([10, 0], ["open", "open"], None, "at least one particle"),
    ([10, -3], ["open", "open"], None, "at least one particle"),
    ([10], ["periodic"], None, "'open' or 'single_wall'"),
    ([10, 20], ["open"], None, "one entry per system"),
    ([10, 20], ["open", "single_wall"], [0.0], "one entry per system"),
])
def test_bad_systems_are_refused(Ensemble, sizes, geometry, heights, match):
    e = Ensemble(precision="float")
    with pytest.raises(RuntimeError, match=match):
        e.setSystems(sizes, geometry, heights)


@pytest.mark.parametrize("viscosity,radius,tolerance", [
    (0.0, 1.0, 1e-4), (1.0, -1.0, 1e-4), (1.0, 1.0, 0.0), (float("nan"), 1.0, 1e-4),
])
def test_bad_constants_are_refused(Ensemble, viscosity, radius, tolerance):
    e = Ensemble(precision="double")
    with pytest.raises(RuntimeError, match="must be positive"):
        e.initialize(viscosity=viscosity, hydrodynamicRadius=radius, tolerance=tolerance)
    e.initialize(viscosity=1.0, hydrodynamicRadius=1.0, tolerance=1e-4)
