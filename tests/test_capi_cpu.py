"""The C-ABI library on a machine without a GPU: it loads, exports every entry
point the public header declares, and its host-side rules (periodicity,
parameters, batches, the wall check, error messages) work before any CUDA
call.  The FP64 tridiagonal square root used by Lanczos is checked on the host
build of the same routine."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "libmobility_gb300.h"


@pytest.fixture(scope="module")
def lib():
    from libmobility_gb300 import _build
    _build.build()
    from libmobility_gb300 import _capi
    return _capi.load()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lmg_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported(lib):
    from libmobility_gb300 import _capi
    names = declared_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
        assert n in _capi.SIGNATURES, n
    assert lib.lmg_version().decode() == "1.1"


def _solver(pz="open", precision="float"):
    from libmobility_gb300 import NBody
    return NBody("open", "open", pz, precision=precision)


def test_periodicity_rules(lib):
    from libmobility_gb300 import NBody
    for bad in (("periodicasdas", "periodic", "open"), ("periodic", "periodic", "open"),
                ("open", "open", "periodic"), ("open", "open", "two_walls")):
        with pytest.raises(RuntimeError):
            NBody(*bad)
    NBody("open", "open", "open")
    NBody("open", "open", "single_wall")


def test_wall_height_parameter_rules(lib):
    s = _solver("open")
    with pytest.raises(RuntimeError, match="only valid for bottom wall"):
        s.setParameters(wallHeight=0.5)
    s.setParameters("advise")
    w = _solver("single_wall")
    with pytest.raises(RuntimeError, match="required for a bottom wall"):
        w.setParameters("advise")
    w.setParameters(wallHeight=0.5)
    with pytest.raises(RuntimeError, match="Invalid algorithm"):
        s.setParameters("fmm")
    for alg in ("naive", "fast", "block", "advise"):
        s.setParameters(alg)


@pytest.mark.parametrize(("nbatch", "nper", "n"), [(5, 1, 10), (2, -1, 8)])
def test_bad_batch_parameters(lib, nbatch, nper, n):
    s = _solver()
    s.setParameters("advise", nbatch, nper)
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.5)
    with pytest.raises(RuntimeError, match="Invalid batch parameters"):
        s.setPositions(np.random.rand(n, 3))


def test_below_wall_rejected_on_host(lib):
    s = _solver("single_wall")
    s.setParameters(wallHeight=1.0)
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
    with pytest.raises(RuntimeError, match="fallen below the wall"):
        s.setPositions(np.array([1.0, 2.0, 0.5]))


@pytest.mark.parametrize("shape", [(4, 6), (3, 1), (1, 4)])
def test_bad_positions_shape(lib, shape):
    s = _solver()
    s.setParameters()
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
    with pytest.raises(RuntimeError):
        s.setPositions(np.random.rand(*shape))


def test_calls_before_positions(lib):
    s = _solver()
    s.setParameters()
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
    with pytest.raises(RuntimeError):
        s.Mdot(np.random.rand(1, 3))
    with pytest.raises(RuntimeError):
        s.sqrtMdotW()
    with pytest.raises(RuntimeError):
        s.LangevinVelocities(dt=1.0, kbt=1.0)
    with pytest.raises(RuntimeError):
        s.divM()


def test_precision_switch(lib):
    assert _solver(precision="float").precision == "float"
    assert _solver(precision="double").precision == "double"
    from libmobility_gb300 import NBody
    assert NBody.precision in ("float", "double")
    h = _solver(precision="double")
    assert lib.lmg_precision_name(h._h).decode() == "double"


def test_status_codes_and_messages(lib):
    h = ctypes.c_void_p()
    st = lib.lmg_create(b"open", b"open", b"bogus", 0, ctypes.byref(h))
    assert st == 1 and not h.value
    assert b"Invalid periodicity" in lib.lmg_create_error()
    st = lib.lmg_create(b"open", b"open", b"open", 7, ctypes.byref(h))
    assert st == 1
    st = lib.lmg_create(b"open", b"open", b"open", 0, ctypes.byref(h))
    assert st == 0 and h.value
    n = ctypes.c_int64(-1)
    assert lib.lmg_get_number_particles(h, ctypes.byref(n)) == 0 and n.value == 0
    # a NULL handle is rejected, not dereferenced
    assert lib.lmg_mdot(None, None, 0, None, 0, None, 0, None, 0) == 1
    assert lib.lmg_destroy(h) == 0


def _tridiag_sqrt_reference(a, b):
    from scipy.linalg import eigh_tridiagonal
    if len(a) == 1:
        return np.array([np.sqrt(a[0])])
    lam, Q = eigh_tridiagonal(a, b)
    return Q @ (np.sqrt(lam) * Q[0])


@pytest.mark.parametrize("m", [1, 2, 3, 7, 50, 120, 200])
def test_tridiagonal_sqrt_e1(lib, m):
    rng = np.random.default_rng(m)
    a = rng.uniform(1.0, 3.0, m)
    b = rng.uniform(-0.4, 0.4, max(m - 1, 1))[: m - 1] if m > 1 else np.zeros(0)
    # diagonally dominant -> positive definite
    out = np.zeros(m)
    rc = lib.lmg_internal_tridiag_sqrt_e1(a.ctypes.data, (b if m > 1 else np.zeros(1)).ctypes.data,
                                          m, out.ctypes.data)
    assert rc == 0
    ref = _tridiag_sqrt_reference(a, b)
    assert np.allclose(out, ref, rtol=1e-12, atol=1e-13)


def test_tridiagonal_lanczos_like_spectrum(lib):
    """Clustered and widely spread eigenvalues, as Lanczos produces (ghost
    copies of converged eigenvalues)."""
    rng = np.random.default_rng(3)
    m = 60
    lam = np.concatenate([np.full(20, 2.0) + 1e-12 * rng.normal(size=20),
                          np.logspace(-3, 3, 40)])
    Q, _ = np.linalg.qr(rng.normal(size=(m, m)))
    A = Q @ np.diag(lam) @ Q.T
    # Householder tridiagonalisation via Lanczos on A with full reorthogonalisation
    v = rng.normal(size=m)
    v /= np.linalg.norm(v)
    V = [v]
    al, be = [], []
    w = A @ v
    for k in range(m):
        al.append(V[-1] @ w)
        w = w - al[-1] * V[-1] - (be[-1] * V[-2] if k else 0)
        for u in V:
            w -= (u @ w) * u
        if k == m - 1:
            break
        be.append(np.linalg.norm(w))
        V.append(w / be[-1])
        w = A @ V[-1]
    a = np.array(al)
    b = np.array(be)
    out = np.zeros(m)
    assert lib.lmg_internal_tridiag_sqrt_e1(a.ctypes.data, b.ctypes.data, m, out.ctypes.data) == 0
    ref = _tridiag_sqrt_reference(a, b)
    assert np.allclose(out, ref, rtol=1e-9, atol=1e-11)


def test_tridiagonal_negative_eigenvalue_gives_nan(lib):
    a = np.array([1.0, -2.0, 1.0])
    b = np.array([0.1, 0.1])
    out = np.zeros(3)
    lib.lmg_internal_tridiag_sqrt_e1(a.ctypes.data, b.ctypes.data, 3, out.ctypes.data)
    assert np.isnan(out).any()


def _lanczos_tridiagonal(lam, m, rng):
    """Lanczos (full reorthogonalisation) on a matrix with spectrum lam."""
    n = len(lam)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    A = Q @ np.diag(lam) @ Q.T
    v = rng.normal(size=n)
    V = [v / np.linalg.norm(v)]
    al, be = [], []
    for k in range(m):
        w = A @ V[-1]
        al.append(V[-1] @ w)
        for u in V:
            w -= (u @ w) * u
        if k == m - 1:
            break
        be.append(np.linalg.norm(w))
        V.append(w / be[-1])
    return np.array(al), np.array(be)


@pytest.mark.parametrize("m", [1, 2, 3, 7, 50, 120, 200])
def test_tridiagonal_sqrt_e1_quadrature(lib, m):
    """The ensembles' quadrature form of T^{1/2} e1 against the eigen-solution."""
    rng = np.random.default_rng(100 + m)
    a = rng.uniform(1.0, 3.0, m)
    b = rng.uniform(-0.4, 0.4, m)
    out = np.zeros(m)
    assert lib.lmg_internal_tridiag_sqrt_e1_quad(a.ctypes.data, b.ctypes.data, m,
                                                 out.ctypes.data) == 0
    ref = _tridiag_sqrt_reference(a, b[: m - 1])
    assert np.linalg.norm(out - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("kappa", [1e2, 1e4, 1e6, 1e7])
def test_tridiagonal_quadrature_condition_numbers(lib, kappa):
    """Spectra over [1, kappa] with a cluster, as Lanczos produces.  The rule
    itself is within 1e-13 of 1/sqrt(lambda); the product T (T^{-1/2} e1)
    adds rounding of order sqrt(kappa) eps, so the bound grows with kappa.
    (The condition number is bounded from above by Gershgorin and a Sturm
    search in factors of 4, so a true kappa of ~1e7 already meets the 1e8
    limit of the node sets.)"""
    rng = np.random.default_rng(int(np.log10(kappa)))
    lam = np.concatenate([np.logspace(0, np.log10(kappa), 50), np.full(10, 2.0)])
    a, b = _lanczos_tridiagonal(lam, 60, rng)
    out = np.zeros(60)
    assert lib.lmg_internal_tridiag_sqrt_e1_quad(a.ctypes.data, b.ctypes.data, 60,
                                                 out.ctypes.data) == 0
    ref = _tridiag_sqrt_reference(a, b)
    bound = 1e-13 * max(1.0, np.sqrt(kappa) / 100)
    assert np.linalg.norm(out - ref) <= bound * np.linalg.norm(ref)


def test_tridiagonal_quadrature_defers_to_exact_form(lib):
    """Not positive definite, or beyond kappa = 1e8: return 2 (the caller
    then takes the exact routine, which gives NaN for a negative eigenvalue)."""
    out = np.zeros(3)
    a, b = np.array([1.0, -2.0, 1.0]), np.array([0.1, 0.1])
    assert lib.lmg_internal_tridiag_sqrt_e1_quad(a.ctypes.data, b.ctypes.data, 3,
                                                 out.ctypes.data) == 2
    a1 = np.array([-1.0])
    assert lib.lmg_internal_tridiag_sqrt_e1_quad(a1.ctypes.data, b.ctypes.data, 1,
                                                 out.ctypes.data) == 2
    a, b = _lanczos_tridiagonal(np.logspace(0, 11, 40), 40, np.random.default_rng(7))
    out = np.zeros(40)
    assert lib.lmg_internal_tridiag_sqrt_e1_quad(a.ctypes.data, b.ctypes.data, 40,
                                                 out.ctypes.data) == 2


def test_buffers_of_another_gpu_are_refused():
    """The decision behind every buffer check, for given pointer attributes
    (cudaMemoryType: 0 unregistered, 1 host, 2 device, 3 managed): device
    memory of another GPU is refused (-1), never read on the host or through
    peer access."""
    from libmobility_gb300 import _capi
    lib = _capi.load()
    f = lib.lmg_internal_classify_pointer
    assert f(0, -1, 0) == 0 and f(1, 0, 0) == 0      # host memory
    assert f(2, 0, 0) == 1 and f(2, 3, 3) == 1       # this GPU's memory
    assert f(2, 1, 0) == -1 and f(2, 0, 5) == -1     # another GPU's memory
    assert f(3, 1, 0) == 1                           # managed memory


def test_solver_selectors_check_their_arguments(lib):
    """The process-wide selectors of the single-system Lanczos and the
    preconditioner build take only their documented values (each one sets a
    setting, no device work) and are left at their defaults."""
    cases = [
        (lib.lmg_internal_lanczos_step_mode, (0, 1), (-1, 2), 0),
        (lib.lmg_internal_lanczos_device_sqrt, (0, 1, 2), (-1, 3), 2),
        (lib.lmg_internal_lanczos_lookahead, (0, 1, 4), (-1, 5), 0),
        (lib.lmg_internal_lanczos_check_wait, (0, 1), (-1, 2), 0),
        (lib.lmg_internal_precond_tc, (0, 1), (-1, 2), 0),
    ]
    try:
        for fn, good, bad, _ in cases:
            for v in good:
                assert fn(v) == 0, (fn.__name__, v)
            for v in bad:
                assert fn(v) != 0, (fn.__name__, v)
        shape = lib.lmg_internal_lanczos_step_shape
        assert shape(16, 256) == 0 and shape(1, 32) == 0 and shape(0, 0) == 0
        for ctas, threads in ((17, 256), (0, 256), (4, 16), (4, 100), (4, 2048)):
            assert shape(ctas, threads) != 0, (ctas, threads)
    finally:
        for fn, _, _, default in cases:
            fn(default)
        lib.lmg_internal_lanczos_step_shape(0, 0)


def test_iteration_limit_and_preconditioner_rules(lib):
    """lanczos::Solver::setIterationHardLimit's range here ([3, 250]), and the
    learned preconditioner's host rules: kind "none" or "mlp", FP32 handles
    only, a parameter vector of a supported network size, and no network
    trained above a wall on an open handle.  All refused before device work."""
    import ctypes
    from libmobility_gb300 import precond as pc
    s = _solver()
    for bad in (2, 251):
        with pytest.raises(RuntimeError, match="iteration limit"):
            s.setLanczosIterationLimit(bad)
    s.setLanczosIterationLimit(3)
    s.setLanczosIterationLimit(250)
    with pytest.raises(RuntimeError, match='"none" or "mlp"'):
        s.setPreconditioner("bogus")
    s.setPreconditioner("none")
    with pytest.raises(RuntimeError, match="needs precision float"):
        _solver(precision="double").setPreconditioner("mlp")
    junk = np.zeros(1000, np.float32)
    rc = s._lib.lmg_set_preconditioner(s._h, b"mlp", ctypes.c_void_p(junk.ctypes.data), junk.size)
    assert rc != 0
    assert "not the size of a network" in s._lib.lmg_last_error(s._h).decode()
    wall = pc.load_weights(pc.default_weights(True), wall=True).astype(np.float32)
    rc = s._lib.lmg_set_preconditioner(s._h, b"mlp", ctypes.c_void_p(wall.ctypes.data), wall.size)
    assert rc != 0
    assert "trained above a wall" in s._lib.lmg_last_error(s._h).decode()


def test_noalloc_argument_rules(lib):
    """lmg_mdot_noalloc_f32 refuses bad arguments before any device work:
    particle count, batch size, constants, missing buffers, torques without
    includeAngular, includeAngular without W, and host buffers (it cannot
    stage them without allocating)."""
    import ctypes
    err = ctypes.create_string_buffer(256)
    a = np.zeros((12, 3), np.float32)
    p = ctypes.c_void_p(a.ctypes.data)

    def call(pos=p, F=p, T=None, U=p, W=None, N=12, nper=-1, wall=0, eta=1.0, rad=1.0, ang=0):
        rc = lib.lmg_mdot_noalloc_f32(pos, F, T, U, W, N, nper, wall, eta, rad, ang, None,
                                      err, 256)
        return rc, err.value.decode()

    for kw, msg in (
        (dict(N=0), "numberParticles must be in"),
        (dict(N=(1 << 24) + 1), "numberParticles must be in"),
        (dict(nper=5), "Invalid batch parameters"),
        (dict(eta=0.0), "must be positive"),
        (dict(rad=-1.0), "must be positive"),
        (dict(pos=None), "needs pos, U and F and/or T"),
        (dict(U=None), "needs pos, U and F and/or T"),
        (dict(F=None), "needs pos, U and F and/or T"),
        (dict(T=p), "includeAngular to true"),
        (dict(ang=1), "needs W when includeAngular"),
        (dict(), "device buffers only"),
    ):
        rc, text = call(**kw)
        assert rc == 1 and msg in text, (kw, rc, text)
