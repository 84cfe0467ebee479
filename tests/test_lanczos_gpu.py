"""sqrtMdotW parity on the GPU, through the C ABI.

* with a given dW, against the reference lanczos::Solver fixtures and the
  oracle's restatement: the result agrees within the Lanczos tolerance scale
  and the iteration count matches (FP64 kernel path) or is within one;
* fluctuation-dissipation: M^{-1/2} sqrtMdotW() samples are N(0,1) per
  component (Kolmogorov-Smirnov, test_fluctuation_dissipation.py:19-59);
* seeded noise: the same seed gives the same noise, the prefactor scales it;
* the error paths (non-convergence) report an error and keep the context.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from test_mdot_gpu import compute_M, make_solver

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("precision", ["double", "float"])
def test_against_reference_lanczos_fixture(cuda, oracle, precision):
    z = np.load(GOLDEN / "ref_lanczos_cases.npz")
    metas = json.loads(str(z["meta"]))
    for si, s in enumerate(metas):
        pos = z[f"s{si}_pos"]
        for run in s["runs"]:
            if run["dtype"] != "float64" or run["tol"] < 1e-6:
                continue
            solver = make_solver(s["wall"], s["ang"], s["a"], s["eta"], precision)
            # tolerance is an initialize() parameter
            solver.initialize(viscosity=s["eta"], hydrodynamicRadius=s["a"],
                              includeAngular=bool(s["ang"]), tolerance=run["tol"])
            solver.setPositions(pos)
            for call in range(3):
                zz = z[run["tag"] + "_z"][call]
                u, w, it, res = solver.sqrtMdotW_noise(zz)
                y = np.concatenate([u.ravel(), w.ravel()]) if s["ang"] else u.ravel()
                yr = z[run["tag"] + "_y"][call]
                rel = np.linalg.norm(y - yr) / np.linalg.norm(yr)
                it_ref = z[run["tag"] + "_it"][call]
                if precision == "double":
                    assert it == it_ref, (si, call, it, it_ref)
                    assert rel < 1e-8, (si, call, rel)
                else:
                    assert abs(it - it_ref) <= 1, (si, call, it, it_ref)
                    assert rel < 10 * run["tol"], (si, call, rel)
                assert res <= run["tol"]


@pytest.mark.parametrize("wall", [0, 1])
def test_matches_oracle_restatement_and_exact_root(cuda, oracle, wall):
    rng = np.random.default_rng(21 + wall)
    N = 200
    p = rng.uniform(0, 25, (N, 3))
    if wall:
        p[:, 2] = rng.uniform(1.5, 10, N)
    a, eta = 1.0, 1 / (6 * np.pi)
    M = oracle.dense(p, a=a, viscosity=eta, wall=wall, include_angular=True)
    S = oracle.sqrtm_dense(M)
    ref = oracle.Lanczos()
    for precision, tol in (("double", 1e-8), ("float", 1e-6)):
        s = make_solver(wall, 1, a, eta, precision)
        s.initialize(viscosity=eta, hydrodynamicRadius=a, includeAngular=True, tolerance=tol)
        s.setPositions(p)
        zz = rng.normal(size=6 * N)
        u, w, it, res = s.sqrtMdotW_noise(zz, prefactor=1.0)
        y = np.concatenate([u.ravel(), w.ravel()])
        ex = S @ zz
        assert np.linalg.norm(y - ex) / np.linalg.norm(ex) < 20 * tol
        yo, ito = oracle.Lanczos().run(lambda v: M @ v, zz, tol)
        assert abs(it - ito) <= 1


def _ks_fdt(M, draw):
    """fluctuation_dissipation_KS of the reference tests."""
    from scipy.stats import kstest, norm
    lam, Q = np.linalg.eigh(M)
    inv_half = (Q / np.sqrt(np.clip(lam, 1e-300, None))).T
    n = lam.size
    mu_alpha = 0.999 ** (1 / n)
    Ns = int(round(2 * (norm.ppf(mu_alpha) / 0.05) ** 2))
    X = np.array([draw() for _ in range(Ns)]).T
    Y = inv_half @ X
    for m in range(n):
        if lam[m] < 1e-6:
            continue
        _, pval = kstest(Y[m], "norm")
        assert pval > 1 - mu_alpha, (m, pval)


@pytest.mark.parametrize("pz", ["open", "single_wall"])
@pytest.mark.parametrize("ang", [False, True])
@pytest.mark.parametrize("N", [1, 2, 10])
def test_fluctuation_dissipation(cuda, pz, ang, N):
    from libmobility_gb300 import NBody
    s = NBody("open", "open", pz, precision="double")
    s.setParameters(**({"wallHeight": 0.0} if pz == "single_wall" else {}))
    s.initialize(viscosity=1.0, hydrodynamicRadius=0.95, includeAngular=ang, seed=1234 + N)
    rng = np.random.default_rng(N)
    p = rng.random((N, 3)) - 0.5
    p[:, 2] += 0.5
    s.setPositions(p * 10)
    M = compute_M(s, N, ang)

    def draw():
        u, w = s.sqrtMdotW(prefactor=1.0)
        return np.concatenate([u.ravel(), w.ravel()]) if ang else u.ravel()

    _ks_fdt(M, draw)


@pytest.mark.parametrize("ang", [False, True])
def test_prefactor_and_seed(cuda, ang):
    from libmobility_gb300 import NBody
    out = []
    for pf in (2.45, 1.0):
        s = NBody("open", "open", "single_wall")
        s.setParameters(wallHeight=0.0)
        s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, includeAngular=ang, seed=4321)
        s.setPositions(np.array([[1.0, 2.0, 3.0], [2.5, 2.0, 3.5]]))
        out.append((s.sqrtMdotW(prefactor=pf), s.divM(prefactor=pf)))
    (a1, d1), (a0, d0) = out
    assert np.allclose(a1[0], 2.45 * a0[0], atol=1e-4)
    assert np.allclose(d1[0], 2.45 * d0[0], atol=1e-4)
    if ang:
        assert np.allclose(a1[1], 2.45 * a0[1], atol=1e-4)
        assert np.allclose(d1[1], 2.45 * d0[1], atol=1e-4)


def test_callback_and_nonconvergence(cuda):
    """Reaching the iteration limit (setIterationHardLimit of the reference
    solver) raises "Could not converge" and leaves the handle usable; the
    callback sees every check from iteration 1 on."""
    s = make_solver(0, 0, 1.0, 1.0, "float")
    seen = []
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, tolerance=1e-12,
                 lanczos_callback=lambda i, e: seen.append((i, e)))
    s.setPositions(np.random.default_rng(1).random((300, 3)) * 30)
    s.setLanczosIterationLimit(6)
    with pytest.raises(RuntimeError, match="Could not converge"):
        s.sqrtMdotW()
    assert [i for i, _ in seen] == [1, 2, 3, 4, 5]
    with pytest.raises(RuntimeError):
        s.setLanczosIterationLimit(1000)
    s.setLanczosIterationLimit(200)
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, tolerance=1e-4)
    s.setPositions(np.random.default_rng(1).random((20, 3)) * 10)
    u, _ = s.sqrtMdotW()
    assert np.isfinite(u).all() and np.abs(u).max() > 0


def test_adaptive_check_schedule_matches_reference(cuda, oracle):
    """Without a callback the first convergence check moves with the
    iterations the previous solves needed (LanczosAlgorithm.cu:224-232); the
    iteration counts over a sequence of solves equal the oracle's, which
    follows the same schedule."""
    rng = np.random.default_rng(8)
    N = 40
    p = rng.uniform(0, 12, (N, 3))
    M = oracle.dense(p, a=1.0, viscosity=1.0, include_angular=False)
    s = make_solver(0, 0, 1.0, 1.0, "double")
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, tolerance=1e-6)
    s.setPositions(p)
    ref = oracle.Lanczos()
    for _ in range(6):
        zz = rng.normal(size=3 * N)
        _, _, it, _ = s.sqrtMdotW_noise(zz)
        _, ito = ref.run(lambda v: M @ v, zz, 1e-6)
        assert it == ito


def test_phase_timing_counts_and_leaves_results_unchanged(cuda):
    """The measurement hook only records events: two solvers with the same
    history, one timed, give bitwise the same results; the sums count every
    issued iteration (up to 3 issued ahead of the check being evaluated at
    this size, and the checks are read one check late: up to 5 past the
    stopping step per solve) and the algorithmic bytes 4 n s per
    iteration."""
    rng = np.random.default_rng(12)
    N = 300
    p = np.column_stack([rng.uniform(0, 40, (N, 2)), rng.uniform(1.5, 10, N)])
    dWs = [rng.normal(size=6 * N) for _ in range(4)]
    out = []
    for timed in (False, True):
        s = make_solver(1, 1, 1.0, 1.0, "float")
        s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, includeAngular=True,
                     tolerance=1e-6)
        s.setPositions(p)
        if timed:
            s._lanczos_phase_timing(True)
        out.append([s.sqrtMdotW_noise(z) for z in dWs])
    t = s._lanczos_phase_times()
    its = 0
    for a, b in zip(*out):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]
        its += b[2]
    assert t["solves"] == 4 and t["checks"] >= 4
    assert its <= t["iterations"] <= its + 4 * 5
    assert t["vector_bytes"] == 4 * (6 * N) * 4 * t["iterations"]
    assert t["check_bytes"] > 0 and t["vector_ms"] > 0 and t["check_ms"] > 0
    assert t["operator_ms"] > 0 and t["build_ms"] == 0 and t["psolve_ms"] == 0
    s._lanczos_phase_timing(False)
    assert s._lanczos_phase_times()["solves"] == 0  # switching resets the sums


def test_grid_barrier_wait_is_bounded(cuda):
    """The fused Lanczos step waits at grid barriers; a wait that nothing
    ends gives up after about a second, reports, and leaves the context
    usable (two blocks meeting at a barrier that cannot complete)."""
    import ctypes
    import time
    from libmobility_gb300 import _capi
    lib = _capi.load()
    gave_up = ctypes.c_int()
    t0 = time.perf_counter()
    assert lib.lmg_internal_barrier_timeout_probe(ctypes.byref(gave_up)) == 0
    assert gave_up.value == 2
    assert time.perf_counter() - t0 < 30
    s = make_solver(0, 0, 1.0, 1.0, "float")
    s.setPositions(np.random.default_rng(2).uniform(0, 10, (30, 3)))
    u, _ = s.sqrtMdotW()
    assert np.isfinite(u).all() and np.abs(u).max() > 0


@pytest.mark.parametrize("precision", ["float", "double"])
def test_nan_in_noise_reports_and_handle_stays_usable(cuda, precision):
    """A NaN in the dW given to sqrtMdotW_noise (injected on the host) ends the
    solve with the reference's error (LanczosAlgorithm.cu:210-213), and the
    same handle then solves a clean dW exactly as a fresh handle does."""
    rng = np.random.default_rng(321)
    N = 200
    p = rng.uniform(0, 20, (N, 3))
    z = rng.normal(size=3 * N)
    bad = z.copy()
    bad[17] = np.nan

    def fresh():
        s = make_solver(0, 0, 1.0, 1 / (6 * np.pi), precision)
        s.setPositions(p)
        return s

    s = fresh()
    with pytest.raises(RuntimeError, match=r"found NaN in result guess"):
        s.sqrtMdotW_noise(bad)
    u, _, it, _ = s.sqrtMdotW_noise(z)
    u2, _, it2, _ = fresh().sqrtMdotW_noise(z)
    assert it == it2
    assert np.array_equal(np.asarray(u), np.asarray(u2))


@pytest.mark.parametrize("precision", ["float", "double"])
@pytest.mark.parametrize("wall", [0, 1])
def test_device_and_host_square_roots_agree(cuda, precision, wall):
    """T^{1/2} e1 at the convergence checks by quadrature on the host (the
    default), by the exact QL on the host, or by quadrature on the device:
    the same stopping step and the same result (FP64 within 1e-12, FP32
    within 1e-6), on fresh handles."""
    from libmobility_gb300 import _capi
    lib = _capi.load()
    rng = np.random.default_rng(90 + wall)
    N = 300
    p = rng.uniform(0, 25, (N, 3))
    if wall:
        p[:, 2] = rng.uniform(1.2, 10, N)
    zs = [rng.normal(size=3 * N) for _ in range(3)]
    out = {}
    try:
        for mode in (1, 0, 2):
            assert lib.lmg_internal_lanczos_device_sqrt(mode) == 0
            s = make_solver(wall, 0, 1.0, 1 / (6 * np.pi), precision)
            s.setPositions(p)
            out[mode] = [s.sqrtMdotW_noise(z) for z in zs]
    finally:
        lib.lmg_internal_lanczos_device_sqrt(2)
    tol = 1e-12 if precision == "double" else 1e-6
    for mode in (1, 2):
        for (u1, _, it1, _), (u0, _, it0, _) in zip(out[mode], out[0]):
            assert it1 == it0
            u1, u0 = np.asarray(u1, np.float64), np.asarray(u0, np.float64)
            assert np.abs(u1 - u0).max() <= tol * np.abs(u0).max()


@pytest.mark.parametrize("precision", ["float", "double"])
def test_lookahead_changes_nothing(cuda, precision):
    """Issuing 1 or 3 iterations ahead of the check being evaluated, and
    starting each check kernel after its own iteration or after the next
    iteration's product, only change how busy the GPU is: same stopping
    step, bitwise the same result (the checks read nothing a later iteration
    writes)."""
    from libmobility_gb300 import _capi
    lib = _capi.load()
    rng = np.random.default_rng(33)
    N = 500
    p = rng.uniform(0, 30, (N, 3))
    zs = [rng.normal(size=3 * N) for _ in range(3)]
    out = {}
    try:
        for ahead, wait in ((1, 0), (3, 0), (1, 1), (3, 1)):
            assert lib.lmg_internal_lanczos_lookahead(ahead) == 0
            assert lib.lmg_internal_lanczos_check_wait(wait) == 0
            s = make_solver(0, 0, 1.0, 1 / (6 * np.pi), precision)
            s.setPositions(p)
            out[ahead, wait] = [s.sqrtMdotW_noise(z) for z in zs]
    finally:
        lib.lmg_internal_lanczos_lookahead(0)
        lib.lmg_internal_lanczos_check_wait(0)
    assert lib.lmg_internal_lanczos_check_wait(2) != 0
    for key in ((3, 0), (1, 1), (3, 1)):
        for (u1, _, it1, r1), (u3, _, it3, r3) in zip(out[1, 0], out[key]):
            assert it1 == it3 and r1 == r3
            assert np.array_equal(np.asarray(u1), np.asarray(u3))


@pytest.mark.parametrize("precision,wall,ang,N", [
    ("float", 0, 0, 300),      # one element a thread or none (registers)
    ("float", 0, 0, 4096),     # the open N = 4096 workload
    ("float", 1, 1, 8000),     # 48000 elements: four a thread
    ("float", 0, 0, 40000),    # eight a thread
    ("float", 0, 0, 60000),    # streamed through memory
    ("double", 1, 1, 6000),    # FP64, four a thread
    ("double", 0, 0, 22000),   # FP64, streamed
])
def test_cluster_and_grid_steps_agree(cuda, precision, wall, ang, N):
    """The Lanczos vector step as one thread-block cluster (the default) and
    as the cooperative grid-wide launch: the same per-element arithmetic,
    inner products summed in another order (and in double-float instead of
    FP64 for FP32 vectors), for vector lengths that take each register path
    of the cluster kernel and the streamed one.

    In FP32 the FP64 scalars agree far below FP32 rounding, so the vectors
    and results come out bitwise equal.  In FP64 the differences of the
    scalars (1e-16) reach the vectors, and Lanczos without
    reorthogonalisation amplifies them once the basis loses orthogonality
    (measured on these systems: successive-iterate errors equal to 1e-13 over
    the first 12 iterations, results 4e-4 apart after 23 at tolerance 1e-3).
    So the check is: the same stopping step, the errors of the first 8
    iterations (reported by a callback) within 1e-9 relative, the results
    within 2 x tol.  A wrong element or a lost partial shows in the first
    errors."""
    from libmobility_gb300 import _capi
    lib = _capi.load()
    rng = np.random.default_rng(N + 7 * wall)
    side = int(np.ceil(N ** (1 / 3)))
    g = np.stack(np.meshgrid(*(np.arange(side),) * 3, indexing="ij"), -1).reshape(-1, 3)[:N]
    p = 3.0 * g + rng.uniform(-0.4, 0.4, (N, 3))
    if wall:
        p[:, 2] += 1.5
    zs = [rng.normal(size=(6 if ang else 3) * N) for _ in range(2)]
    tol = 1e-3
    out = {}
    try:
        for mode in (0, 1):
            assert lib.lmg_internal_lanczos_step_mode(mode) == 0
            errs = []
            s = make_solver(wall, ang, 1.0, 1 / (6 * np.pi), precision)
            s.initialize(viscosity=1 / (6 * np.pi), hydrodynamicRadius=1.0,
                         includeAngular=bool(ang), tolerance=tol,
                         lanczos_callback=lambda i, e, errs=errs: errs.append(e))
            s.setPositions(p)
            out[mode] = ([s.sqrtMdotW_noise(z) for z in zs], errs)
    finally:
        lib.lmg_internal_lanczos_step_mode(0)
    (res0, errs0), (res1, errs1) = out[0], out[1]
    n8 = min(8, len(errs1))
    assert np.allclose(errs0[:n8], errs1[:n8], rtol=1e-9, atol=0)
    for (u1, w1, it1, _), (u0, w0, it0, _) in zip(res0, res1):
        assert it1 == it0
        for a, b in ((u1, u0), (w1, w0)) if ang else ((u1, u0),):
            a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
            if precision == "float":
                assert np.array_equal(a, b)
            else:
                assert np.abs(a - b).max() <= 2 * tol * np.abs(b).max()
