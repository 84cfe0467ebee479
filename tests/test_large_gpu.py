"""Large single-wall system with torques (N = 262144; x, y uniform in
[0, 1024)^2, z uniform in [1.5a, 40a], forces and torques N(0, 1)):

  * FP32 Mdot against the FP64 oracle on 4096 target rows (each summed over
    all 262144 sources), both on the same FP32 inputs: within 1e-5 of the
    largest output;
  * fluctuation-dissipation on a dense window of the same configuration
    (the ~1000 particles with x, y in [0, 64)^2): over 1000 sqrtMdotW draws
    with torques, the sample variance of q.y for random unit vectors q
    matches q^T M q (M from the oracle), each within 6 standard errors of a
    variance estimate from 1000 samples, and on average within 2 % -- with
    plain Lanczos and with the learned wall preconditioner on;
  * the learned wall preconditioner cuts the Lanczos iterations of the same
    layout at N = 65536 (x, y in [0, 512)^2, same density) below half.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_LARGE = 262144


def _config(seed=31):
    rng = np.random.default_rng(seed)
    pos = np.column_stack([rng.uniform(0, 1024, N_LARGE), rng.uniform(0, 1024, N_LARGE),
                           rng.uniform(1.5, 40, N_LARGE)])
    F = rng.normal(size=(N_LARGE, 3))
    T = rng.normal(size=(N_LARGE, 3))
    return pos, F, T


def _solver(precision="float", tol=1e-6, seed=0):
    from libmobility_gb300 import NBody
    s = NBody("open", "open", "single_wall", precision=precision)
    s.setParameters(wallHeight=0.0)
    s.initialize(viscosity=1 / (6 * np.pi), hydrodynamicRadius=1.0, includeAngular=True,
                 tolerance=tol, seed=seed)
    return s


def test_mdot_262k_wall_rows_vs_fp64_oracle(cuda, oracle):
    """On the same inputs: the oracle gets the FP32 values the kernel works
    on.  (Rounding the positions themselves to FP32 moves them by up to 6e-5
    at x ~ 1000, which changes the exact result by ~2e-5 of its largest
    entry; that is the input's precision, not the kernel's.)"""
    pos, F, T = (np.asarray(v, np.float32).astype(np.float64) for v in _config())
    s = _solver()
    s.setPositions(pos)
    U, W = s.Mdot(F, T)
    rows = 4096
    Uo, Wo = oracle.mdot(pos, F, T, a=1.0, viscosity=1 / (6 * np.pi), wall=True,
                         include_angular=True, rows=(0, rows))
    for got, ref in ((U[:rows], Uo), (W[:rows], Wo)):
        err = np.abs(np.asarray(got, np.float64) - ref).max() / np.abs(ref).max()
        assert err <= 1e-5, err


@pytest.mark.parametrize("prec", ["none", "mlp"])
def test_fluctuation_dissipation_dense_window(cuda, oracle, prec):
    pos, _, _ = _config()
    win = pos[(pos[:, 0] < 64) & (pos[:, 1] < 64)]
    n = win.shape[0]
    assert 800 < n < 1300
    M = oracle.dense(win, a=1.0, viscosity=1 / (6 * np.pi), wall=True, include_angular=True)
    s = _solver(seed=123)
    s.setPreconditioner(prec)
    s.setPositions(win)
    draws = 1000
    Y = np.empty((draws, 6 * n))
    for k in range(draws):
        u, w = s.sqrtMdotW(prefactor=1.0)
        Y[k, :3 * n] = np.asarray(u).ravel()
        Y[k, 3 * n:] = np.asarray(w).ravel()
    assert np.abs(Y.mean(0)).max() < 6 * np.sqrt(np.diag(M).max() / draws)
    rng = np.random.default_rng(5)
    ratios = []
    for _ in range(64):
        q = rng.normal(size=6 * n)
        q /= np.linalg.norm(q)
        var_ref = q @ M @ q
        var = np.var(Y @ q)
        ratios.append(var / var_ref)
    ratios = np.array(ratios)
    se = np.sqrt(2.0 / draws)  # relative standard error of a sample variance
    assert np.abs(ratios - 1).max() < 6 * se, ratios
    assert abs(ratios.mean() - 1) < 0.02, ratios.mean()


def test_wall_preconditioner_halves_iterations(cuda):
    from libmobility_gb300 import precond
    if not precond.default_weights(wall=True).name.startswith("precond_wall"):
        pytest.skip("no wall network shipped")
    rng = np.random.default_rng(31)
    N = 65536
    pos = np.column_stack([rng.uniform(0, 512, N), rng.uniform(0, 512, N),
                           rng.uniform(1.5, 40, N)])
    its = {}
    for prec in ("none", "mlp"):
        s = _solver(seed=3)
        s.setPreconditioner(prec)
        s.setPositions(pos)
        its[prec] = [s.sqrtMdotW_noise(np.random.default_rng(40 + k).normal(size=6 * N))[2]
                     for k in range(2)]
    assert np.mean(its["mlp"]) < 0.5 * np.mean(its["none"]), its
