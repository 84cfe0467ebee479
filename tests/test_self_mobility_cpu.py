"""SelfMobility through the C ABI, on the host (no GPU needed), ported from
libMobility's tests for that solver: self mobility values
(test_mobility_matrix.py:194-221), periodicity rule, shapes, prefactor
linearity with a shared seed (test_interface.py:384-418), kbt = 0 Langevin
equals Mdot, zero divM, and fluctuation-dissipation (KS per component)."""
import numpy as np
import pytest

from libmobility_gb300 import SelfMobility


@pytest.fixture(scope="module", autouse=True)
def built():
    from libmobility_gb300 import _build
    _build.build()


@pytest.mark.parametrize("precision", ["float", "double"])
@pytest.mark.parametrize("ang", [True, False])
def test_self_mobility_values(precision, ang):
    s = SelfMobility("open", "open", "open", precision=precision)
    s.setParameters(parameter=5.0)
    a, eta = 0.9123, 1.123
    s.initialize(viscosity=eta, hydrodynamicRadius=a, includeAngular=ang)
    s.setPositions(np.zeros((1, 3)))
    f = np.ones(3)
    m0 = 1.0 / (6 * np.pi * eta * a)
    if ang:
        lin, angv = s.Mdot(f, np.ones(3))
        assert np.allclose(angv, np.ones(3) / (8 * np.pi * eta * a ** 3), rtol=0, atol=1e-7)
    else:
        lin, _ = s.Mdot(f)
    assert np.allclose(lin, m0 * f, rtol=0, atol=1e-7)


def test_periodicity_and_shapes():
    with pytest.raises(RuntimeError, match="open boundary solver"):
        SelfMobility("open", "open", "single_wall")
    s = SelfMobility("open", "open", "open")
    s.setParameters(1.0)
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
    s.setPositions(np.random.rand(4, 3))
    u, w = s.Mdot(np.random.rand(4, 3))
    assert u.shape == (4, 3) and w is None
    with pytest.raises(RuntimeError):
        s.Mdot(np.random.rand(4, 3), np.random.rand(4, 3))  # torques without angular
    assert s.sqrtMdotW()[0].shape == (4, 3)
    assert not s.divM()[0].any()
    f = np.random.rand(4, 3)
    assert np.allclose(s.LangevinVelocities(1.0, 0.0, f)[0], s.Mdot(f)[0])


@pytest.mark.parametrize("ang", [True, False])
def test_prefactor_and_seed(ang):
    out = []
    for pf in (2.45, 1.0):
        s = SelfMobility("open", "open", "open")
        s.setParameters(1.0)
        s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, includeAngular=ang, seed=1234)
        s.setPositions(np.random.rand(3, 3))
        out.append(s.sqrtMdotW(prefactor=pf))
    (a1, b1), (a0, b0) = out
    assert np.allclose(a1, 2.45 * a0, atol=1e-5)
    if ang:
        assert np.allclose(b1, 2.45 * b0, atol=1e-5)


def test_fluctuation_dissipation():
    from scipy.stats import kstest, norm
    s = SelfMobility("open", "open", "open", precision="double")
    s.setParameters(1.0)
    eta, a = 1.0, 0.95
    s.initialize(viscosity=eta, hydrodynamicRadius=a, includeAngular=True, seed=99)
    N = 2
    s.setPositions(np.random.rand(N, 3))
    n = 6 * N
    mu_alpha = 0.999 ** (1 / n)
    Ns = int(round(2 * (norm.ppf(mu_alpha) / 0.05) ** 2))
    X = np.array([np.concatenate([x.ravel() for x in s.sqrtMdotW()]) for _ in range(Ns)])
    scale = np.concatenate([np.full(3 * N, 1 / np.sqrt(1 / (6 * np.pi * eta * a))),
                            np.full(3 * N, 1 / np.sqrt(1 / (8 * np.pi * eta * a ** 3)))])
    for m in range(n):
        _, p = kstest(X[:, m] * scale[m], "norm")
        assert p > 1 - mu_alpha
