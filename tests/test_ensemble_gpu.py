"""Ensembles of uneven systems (open and bottom wall mixed), through the C ABI.

Every system of an ensemble must behave as its own NBody solver:
  * Mdot per system against the FP64 oracle (FP32 within 1e-5, FP64 within
    1e-12 of the largest output, as the single-system tests), with and without
    the autotuner, sizes on both sides of the 128-particle padding;
  * sqrtMdotW per system against the exact M^{1/2} dW (within 20 x tol) and
    against one NBody solver per system on the same dW (samples and Lanczos
    iteration counts);
  * noise drawn from the seed is reproducible; prefactor scales; results
    accumulate into the output; below-the-wall positions raise.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = {"float": 1e-5, "double": 1e-12}


def rel_err(x, ref):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.abs(x - ref).max() / np.abs(ref).max()


def _ensemble(rng, sizes, geoms, heights, phi=0.1):
    """Positions of each system: open ones uniform in a cube sized for phi,
    wall ones with x, y uniform and z uniform in [1.5, 12] above their wall."""
    out = []
    for n, g, h in zip(sizes, geoms, heights):
        if g:
            L = np.sqrt(n * 4.19 / (10.5 * phi))
            p = np.column_stack([rng.uniform(0, L, n), rng.uniform(0, L, n),
                                 h + rng.uniform(1.5, 12, n)])
        else:
            L = (n * 4.19 / phi) ** (1 / 3)
            p = rng.uniform(0, L, (n, 3))
        out.append(p)
    return out


def _make(precision, sizes, geoms, heights, tol=1e-6, autotune=True, seed=3):
    from libmobility_gb300.ensemble import Ensemble
    e = Ensemble(precision=precision)
    e.setSystems(sizes, geoms, heights)
    e.initialize(viscosity=0.9, hydrodynamicRadius=1.1, tolerance=tol, seed=seed,
                 autotune=autotune)
    return e


SIZES = [1, 5, 127, 128, 129, 300, 700, 40, 255, 256, 513, 2]
GEOMS = [0, 1, 1, 0, 1, 0, 1, 1, 0, 1, 0, 1]
HEIGHTS = [0.0, 0.0, -3.5, 0.0, 2.0, 0.0, 0.0, 10.0, 0.0, -1.0, 0.0, 0.5]


@pytest.mark.parametrize("precision", ["float", "double"])
@pytest.mark.parametrize("autotune", [True, False])
def test_mdot_per_system_matches_oracle(cuda, oracle, precision, autotune):
    rng = np.random.default_rng(1 + autotune)
    systems = _ensemble(rng, SIZES, GEOMS, HEIGHTS)
    e = _make(precision, SIZES, GEOMS, HEIGHTS, autotune=autotune)
    pos = np.concatenate(systems)
    F = rng.normal(size=pos.shape)
    e.setPositions(pos)
    for rep in range(2):  # the second call reuses plans and buffers
        U = e.Mdot(F)
        off = 0
        for n, g, h, p in zip(SIZES, GEOMS, HEIGHTS, systems):
            Uo, _ = oracle.mdot(p, F[off:off + n], None, a=1.1, viscosity=0.9, wall=bool(g),
                                wall_height=h)
            assert rel_err(U[off:off + n], Uo) <= TOL[precision], (n, g, rep)
            off += n
    d = e.describe()
    assert d["systems"] == len(SIZES) and d["particles"] == sum(SIZES)
    assert all(gr["padded_particles"] % 128 == 0 for gr in d["groups"])
    assert all(gr["tuned"] for gr in d["groups"])
    if autotune:
        assert all(len(gr["trials_ms"]) >= 1 for gr in d["groups"])


def test_mdot_torch_cuda_buffers(cuda, oracle):
    import torch
    rng = np.random.default_rng(5)
    sizes, geoms, heights = [200, 333, 90], [1, 0, 1], [0.0, 0.0, 1.0]
    systems = _ensemble(rng, sizes, geoms, heights)
    pos = np.concatenate(systems)
    F = rng.normal(size=pos.shape)
    e = _make("float", sizes, geoms, heights)
    e.setPositions(torch.tensor(pos, device="cuda", dtype=torch.float32))
    U = e.Mdot(torch.tensor(F, device="cuda", dtype=torch.float32))
    assert U.is_cuda and tuple(U.shape) == pos.shape
    U = U.cpu().numpy()
    off = 0
    for n, g, h, p in zip(sizes, geoms, heights, systems):
        Uo, _ = oracle.mdot(p, F[off:off + n], None, a=1.1, viscosity=0.9, wall=bool(g),
                            wall_height=h)
        assert rel_err(U[off:off + n], Uo) <= 1e-5
        off += n


@pytest.mark.parametrize("precision,tol", [("float", 1e-6), ("double", 1e-8)])
def test_sqrt_per_system_matches_exact_root(cuda, oracle, precision, tol):
    rng = np.random.default_rng(7)
    sizes = [60, 130, 7, 250, 128, 90, 1]
    geoms = [0, 1, 1, 0, 1, 0, 0]
    heights = [0.0, 0.0, 2.5, 0.0, -4.0, 0.0, 0.0]
    systems = _ensemble(rng, sizes, geoms, heights, phi=0.15)
    e = _make(precision, sizes, geoms, heights, tol=tol)
    pos = np.concatenate(systems)
    e.setPositions(pos)
    for call in range(2):  # the adaptive check schedule moves between calls
        dW = rng.normal(size=pos.shape)
        U, its, errs, ms = e.sqrtMdotW(dW, prefactor=1.0)
        off = 0
        for k, (n, g, h, p) in enumerate(zip(sizes, geoms, heights, systems)):
            M = oracle.dense(p, a=1.1, viscosity=0.9, wall=bool(g), wall_height=h)
            z = dW[off:off + n].ravel()
            ex = oracle.sqrtm_dense(M) @ z
            y = U[off:off + n].ravel()
            assert np.linalg.norm(y - ex) / np.linalg.norm(ex) < 20 * tol, (k, n, g)
            assert errs[k] <= tol and ms[k] > 0
            off += n
        assert (its > 0).all()


# The ensemble sums each product in another order (its own source splits).
# Lanczos without reorthogonalisation is sensitive to such rounding once the
# basis loses orthogonality: for the N = 400, phi = 0.2 system below the
# FP64 oracle restatement itself stops anywhere between 69 and 78 iterations
# at 1e-8 when M is perturbed by 1e-15 of its largest entry.  So the stopping
# steps agree to max(3, 15 %); the samples agree to the tolerance scale.
@pytest.mark.parametrize("precision,tol,dsample",
                         [("double", 1e-8, 4e-7), ("float", 1e-6, 2e-5)])
def test_iterations_match_single_system_solver(cuda, precision, tol, dsample):
    """The same dW through an ensemble and through one NBody per system."""
    from libmobility_gb300 import NBody
    rng = np.random.default_rng(9)
    sizes, geoms, heights = [150, 400, 64, 300], [1, 0, 0, 1], [0.0, 0.0, 0.0, 3.0]
    systems = _ensemble(rng, sizes, geoms, heights, phi=0.2)
    pos = np.concatenate(systems)
    e = _make(precision, sizes, geoms, heights, tol=tol)
    e.setPositions(pos)
    dW = rng.normal(size=pos.shape)
    U, its, _, _ = e.sqrtMdotW(dW)
    off = 0
    for k, (n, g, h, p) in enumerate(zip(sizes, geoms, heights, systems)):
        s = NBody("open", "open", "single_wall" if g else "open", precision=precision)
        if g:
            s.setParameters(wallHeight=h)
        else:
            s.setParameters()
        s.initialize(viscosity=0.9, hydrodynamicRadius=1.1, tolerance=tol)
        s.setPositions(p)
        u, _, it, _ = s.sqrtMdotW_noise(dW[off:off + n])
        assert abs(it - its[k]) <= max(3, 0.15 * it), (k, it, its[k])
        assert np.linalg.norm(U[off:off + n] - u) / np.linalg.norm(u) < dsample
        off += n


def test_noise_seed_prefactor_and_accumulation(cuda):
    rng = np.random.default_rng(11)
    sizes, geoms, heights = [100, 257, 33], [0, 1, 0], [0.0, 0.0, 0.0]
    pos = np.concatenate(_ensemble(rng, sizes, geoms, heights))
    a = _make("float", sizes, geoms, heights, seed=42)
    b = _make("float", sizes, geoms, heights, seed=42)
    a.setPositions(pos)
    b.setPositions(pos)
    ua, _, _, _ = a.sqrtMdotW(prefactor=1.0)
    ub, _, _, _ = b.sqrtMdotW(prefactor=2.0)
    assert np.isfinite(ua).all() and np.abs(ua).max() > 0
    assert np.allclose(ub, 2.0 * ua, rtol=1e-5, atol=1e-6)
    # the next draw of the same stream differs; out= accumulates
    uc, _, _, _ = a.sqrtMdotW(prefactor=1.0, out=np.full(pos.shape, 0.5, dtype=np.float32))
    assert not np.allclose(uc - 0.5, ua)
    dW = rng.normal(size=pos.shape)
    u1, _, _, _ = a.sqrtMdotW(dW)
    u2, _, _, _ = a.sqrtMdotW(dW, out=np.full(pos.shape, 0.5, dtype=np.float32))
    assert np.allclose(u2 - 0.5, u1, atol=1e-5)


def test_errors(cuda):
    from libmobility_gb300.ensemble import Ensemble
    e = Ensemble(precision="float")
    with pytest.raises(RuntimeError):
        e.setSystems([10, 0], [0, 1])
    with pytest.raises(RuntimeError):
        e.setSystems([10, 5], [0, 2])
    e.setSystems([10, 5], ["open", "single_wall"], [0.0, 1.0])
    e.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
    with pytest.raises(RuntimeError):
        e.setPositions(np.zeros((14, 3)))
    pos = np.zeros((15, 3))
    pos[:, 0] = np.arange(15) * 3.0
    pos[10:, 2] = 0.5  # wall at 1.0: below it
    with pytest.raises(RuntimeError, match="fallen below the wall"):
        e.setPositions(pos)
    pos[10:, 2] = 3.0
    e.setPositions(pos)
    with pytest.raises(RuntimeError):
        e.Mdot(np.zeros((14, 3)))
    U = e.Mdot(np.ones((15, 3)))
    assert np.isfinite(U).all()
