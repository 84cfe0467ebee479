"""Mdot parity on the GPU, called through the C ABI (via the Python class).

Tolerances (stated by the specification of this path): FP32 results within
1e-5 relative of FP64 (error measured as max|u - u_ref| / max|u_ref| over the
whole output), FP64 results within 1e-12.  References:
  * the committed fixtures of the reference's own pair code (make_golden.py);
  * the FP64 oracle (pinned against libMobility's golden arrays);
  * the reference's own CUDA kernel on the same GPU, when its cubin is here.
"""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
TOL = {"float": 1e-5, "double": 1e-12}


def rel_err(x, ref):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    s = np.abs(ref).max()
    if s == 0:
        return np.abs(x).max()
    return np.abs(x - ref).max() / s


def make_solver(wall, ang, a, eta, precision, N=None, nper=None, wall_height=0.0):
    from libmobility_gb300 import NBody
    s = NBody("open", "open", "single_wall" if wall else "open", precision=precision)
    nb = -1 if (nper is None or N is None) else N // nper
    np_ = -1 if nper is None else nper
    if wall:
        s.setParameters("advise", nb, np_, wallHeight=wall_height)
    else:
        s.setParameters("advise", nb, np_)
    s.initialize(viscosity=eta, hydrodynamicRadius=a, includeAngular=bool(ang))
    return s


@pytest.mark.parametrize("precision", ["float", "double"])
def test_reference_fixture_cases(cuda, precision):
    z = np.load(GOLDEN / "ref_mdot_cases.npz")
    metas = json.loads(str(z["meta"]))
    for i, m in enumerate(metas):
        s = make_solver(m["wall"], m["ang"], m["a"], m["eta"], precision, m["N"], m["nper"],
                        m["wall_height"])
        s.setPositions(z[f"c{i}_pos"])
        F = z[f"c{i}_F"] if m["hasF"] else None
        T = z[f"c{i}_T"] if m["hasT"] else None
        U, W = s.Mdot(F, T)
        assert rel_err(U, z[f"c{i}_U_d"]) <= TOL[precision], (i, m)
        if m["ang"]:
            assert rel_err(W, z[f"c{i}_W_d"]) <= TOL[precision], (i, m)
        else:
            assert W is None


def _system(rng, N, wall, box=None, phi=0.05):
    if box is None:
        box = (N * 4 * np.pi / 3 / phi) ** (1 / 3)
    p = rng.uniform(0, box, (N, 3))
    if wall:
        p[:, 2] = rng.uniform(0.5, 12.0, N)
    return p


@pytest.mark.parametrize("precision", ["float", "double"])
@pytest.mark.parametrize("wall", [0, 1])
@pytest.mark.parametrize("blocks", ["F", "F+ang", "T+ang", "FT+ang"])
def test_random_systems_vs_oracle(cuda, oracle, precision, wall, blocks):
    seed = 1000 * (precision == "double") + 100 * wall + ["F", "F+ang", "T+ang", "FT+ang"].index(blocks)
    rng = np.random.default_rng(seed)
    ang = "ang" in blocks
    for N, nper in ((1, 1), (2, 2), (3, 3), (31, 31), (33, 11), (257, 257), (1000, 250),
                    (1537, 1537)):
        p = _system(rng, N, wall)
        F = rng.normal(size=(N, 3)) if "F" in blocks else None
        T = rng.normal(size=(N, 3)) if "T" in blocks else None
        s = make_solver(wall, ang, 1.1, 0.9, precision, N, nper)
        s.setPositions(p)
        U, W = s.Mdot(F, T)
        Uo, Wo = oracle.mdot(p, F, T, a=1.1, viscosity=0.9, wall=wall, include_angular=ang,
                             nper_batch=nper)
        assert rel_err(U, Uo) <= TOL[precision], (N, nper)
        if ang:
            assert rel_err(W, Wo) <= TOL[precision], (N, nper)


@pytest.mark.parametrize("precision", ["float", "double"])
@pytest.mark.parametrize("wall", [0, 1])
def test_every_launch_plan_agrees(cuda, oracle, precision, wall):
    """Targets per thread (1, 2) and source splits (1, 3, 8, planner's) only
    change the order of summation: every plan matches the oracle.  The wall
    case with all blocks runs the packed two-sources-at-a-time evaluation,
    with overlapping pairs (r < 2a) and particles below the radius mixed in."""
    from libmobility_gb300 import _capi
    lib = _capi.load()
    rng = np.random.default_rng(21 + wall)
    cases = ((1537, 1537), (3000, 1000))
    try:
        for N, nper in cases:
            p = _system(rng, N, wall, phi=0.15)
            F = rng.normal(size=(N, 3))
            T = rng.normal(size=(N, 3))
            Uo, Wo = oracle.mdot(p, F, T, a=1.1, viscosity=0.9, wall=wall, include_angular=1,
                                 nper_batch=nper)
            for tpt in (1, 2):
                for split in (0, 1, 3, 8):
                    assert lib.lmg_internal_mdot_plan_override(tpt, split) == 0
                    s = make_solver(wall, 1, 1.1, 0.9, precision, N, nper)
                    s.setPositions(p)
                    U, W = s.Mdot(F, T)
                    assert rel_err(U, Uo) <= TOL[precision], (N, tpt, split)
                    assert rel_err(W, Wo) <= TOL[precision], (N, tpt, split)
    finally:
        lib.lmg_internal_mdot_plan_override(0, 0)


@pytest.mark.parametrize("precision", ["float", "double"])
def test_large_open_and_wall_subsample(cuda, oracle, precision):
    """N = 4096 open (UF) and N = 16384 wall (all blocks): rows 0..511 against
    the FP64 oracle summed over every source."""
    rng = np.random.default_rng(11)
    for wall, N, ang in ((0, 4096, 0), (1, 16384, 1)):
        if wall:
            p = np.column_stack([rng.uniform(0, 128, N), rng.uniform(0, 128, N),
                                 rng.uniform(1.5, 20, N)])
        else:
            L = (N * 4 * np.pi / 3 / 0.05) ** (1 / 3)
            p = rng.uniform(0, L, (N, 3))
        F = rng.normal(size=(N, 3))
        T = rng.normal(size=(N, 3)) if ang else None
        s = make_solver(wall, ang, 1.0, 1 / (6 * np.pi), precision)
        s.setPositions(p)
        U, W = s.Mdot(F, T)
        Uo, Wo = oracle.mdot(p, F, T, a=1.0, viscosity=1 / (6 * np.pi), wall=wall,
                             include_angular=ang, rows=(0, 512))
        assert rel_err(U[:512], Uo) <= TOL[precision]
        if ang:
            assert rel_err(W[:512], Wo) <= TOL[precision]


def test_torch_cuda_buffers_and_stream(cuda, oracle):
    import torch
    rng = np.random.default_rng(2)
    N = 700
    p = _system(rng, N, 1)
    F = rng.normal(size=(N, 3))
    T = rng.normal(size=(N, 3))
    s = make_solver(1, 1, 1.0, 1.0, "float")
    s.setPositions(torch.tensor(p, device="cuda"))
    U, W = s.Mdot(torch.tensor(F, device="cuda"), torch.tensor(T, device="cuda"))
    assert U.is_cuda and W.is_cuda and U.dtype == torch.float32 and U.shape == (N, 3)
    Uo, Wo = oracle.mdot(p, F, T, a=1.0, viscosity=1.0, wall=1, include_angular=1)
    torch.cuda.synchronize()
    assert rel_err(U.cpu().numpy(), Uo) <= 1e-5
    assert rel_err(W.cpu().numpy(), Wo) <= 1e-5


def test_ordered_on_callers_stream(cuda, oracle):
    """Results are ordered on the caller's current torch stream (the default
    stream included): reading them right away, without a synchronize, sees
    the finished values."""
    import torch
    rng = np.random.default_rng(12)
    N = 4096
    p = _system(rng, N, 0)
    F = rng.normal(size=(N, 3))
    s = make_solver(0, 0, 1.0, 1.0, "float")
    s.setPositions(torch.tensor(p, device="cuda"))
    dF = torch.tensor(F, device="cuda", dtype=torch.float32)
    Uo, _ = oracle.mdot(p, F, None, a=1.0, viscosity=1.0, rows=(0, 256))
    for stream in (torch.cuda.default_stream(), torch.cuda.Stream()):
        with torch.cuda.stream(stream):
            U, _ = s.Mdot(dF)
            V = U[:256].clone() * 1.0  # consumer on the same stream
        stream.synchronize()
        assert rel_err(V.cpu().numpy(), Uo) <= 1e-5


def test_no_forces_no_torques_and_overwrite(cuda):
    s = make_solver(0, 1, 1.0, 1.0, "float")
    s.setPositions(np.random.rand(5, 3) * 5)
    U1, W1 = s.Mdot(np.ones((5, 3)))
    U2, W2 = s.Mdot(np.ones((5, 3)))
    assert np.array_equal(U1, U2) and np.array_equal(W1, W2)  # overwritten, not added
    U3, W3 = s.Mdot(np.zeros((5, 3)), np.zeros((5, 3)))
    assert not U3.any() and not W3.any()


def _ref_gpu():
    from oracle import build as ob
    here = Path(ob.__file__).resolve().parent
    cub = {p: here / "_ref" / f"ref_nbody_{p}.cubin" for p in "fd"}
    if not all(c.exists() for c in cub.values()):
        pytest.skip("reference kernel cubin not present")
    ob.build_oracle()
    import ctypes
    lib = ctypes.CDLL(str(here / "_build" / "libref_gpu_launcher.so"))
    lib.ref_gpu_last_error.restype = ctypes.c_char_p
    for dbl, key in ((0, "f"), (1, "d")):
        if lib.ref_gpu_load(dbl, str(cub[key]).encode()) != 0:
            pytest.skip("cannot load reference cubin: " + lib.ref_gpu_last_error().decode())
    return lib


@pytest.mark.parametrize("precision", ["float", "double"])
def test_against_reference_cuda_kernel(cuda, precision):
    """Same inputs through libMobility's own computeRPYBatchedFastGPU and
    through this library, on the same GPU."""
    import ctypes
    import torch
    lib = _ref_gpu()
    dt = torch.float32 if precision == "float" else torch.float64
    rng = np.random.default_rng(9)
    for wall, ang, hasT, N, nper in ((0, 0, 0, 4096, 4096), (0, 1, 1, 1024, 256),
                                     (1, 1, 1, 2048, 2048), (1, 0, 0, 999, 333)):
        p = _system(rng, N, wall)
        F = rng.normal(size=(N, 3))
        T = rng.normal(size=(N, 3)) if hasT else None
        a, eta = 1.0, 1 / (6 * np.pi)
        t0 = 1 / (6 * np.pi * eta * a)
        rt0 = 1 / (8 * np.pi * eta * a * a)
        r0 = 1 / (8 * np.pi * eta * a ** 3)
        dp = torch.tensor(p, dtype=dt, device="cuda")
        dF = torch.tensor(F, dtype=dt, device="cuda")
        dT = torch.tensor(T, dtype=dt, device="cuda") if hasT else None
        U = torch.zeros((N, 3), dtype=dt, device="cuda")
        W = torch.zeros((N, 3), dtype=dt, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        rc = lib.ref_gpu_mdot(ctypes.c_int(precision == "double"), ctypes.c_int(wall),
                              ctypes.c_void_p(dp.data_ptr()), ctypes.c_void_p(dF.data_ptr()),
                              ctypes.c_void_p(dT.data_ptr() if hasT else None),
                              ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(W.data_ptr()),
                              ctypes.c_int(N // nper), ctypes.c_int(nper), ctypes.c_double(t0),
                              ctypes.c_double(r0), ctypes.c_double(rt0), ctypes.c_double(a),
                              ctypes.c_int(ang), ctypes.c_void_p(st))
        assert rc == 0, lib.ref_gpu_last_error()
        torch.cuda.synchronize()
        s = make_solver(wall, ang, a, eta, precision, N, nper)
        s.setPositions(dp)
        U2, W2 = s.Mdot(dF, dT)
        torch.cuda.synchronize()
        assert rel_err(U2.cpu().numpy(), U.cpu().numpy()) <= TOL[precision]
        if ang:
            assert rel_err(W2.cpu().numpy(), W.cpu().numpy()) <= TOL[precision]


def compute_M(solver, N, ang):
    """Dense mobility column by column through Mdot (tests/utils.py:62-84)."""
    n = (6 if ang else 3) * N
    M = np.zeros((n, n))
    I = np.identity(n)
    for i in range(n):
        f = I[: 3 * N, i].copy()
        if ang:
            t = I[3 * N:, i].copy()
            u, w = solver.Mdot(f, t)
            M[:, i] = np.concatenate([u.reshape(-1), w.reshape(-1)])
        else:
            M[:, i] = solver.Mdot(f)[0].reshape(-1)
    return M


@pytest.mark.parametrize("precision", ["float", "double"])
@pytest.mark.parametrize("wall_height", [0.0, 5.4, -10.0])
def test_wall_pair_and_self_matrices(cuda, oracle, precision, wall_height):
    """The golden configurations of test_wall_mobility.py (a pair at
    separations 3a, 4a, 8a offset in x and y, and a single particle, at heights
    down to below one radius), against the FP64 oracle, with the reference's
    tolerance 100 eps of the working precision after normalising by the
    block prefactors."""
    eta = 1 / 4 / np.sqrt(np.pi)
    tol = 100 * np.finfo(np.float32 if precision == "float" else np.float64).eps
    s = make_solver(1, 1, 1.0, eta, precision, wall_height=wall_height)
    c0 = np.array([38.4, 38.4, 0.0])
    heights = np.concatenate([np.linspace(0.2, 1.0, 5), np.linspace(1.05, 12.0, 9)])
    nm1 = np.zeros((6, 6))
    nm1[:3, :3] = 1 / (6 * np.pi * eta)
    nm1[3:, 3:] = 1 / (8 * np.pi * eta)
    nm1[3:, :3] = nm1[:3, 3:] = 1 / (6 * np.pi * eta)
    for h in heights:
        pos = (c0 + [0, 0, h + wall_height])[None, :]
        s.setPositions(pos)
        M = compute_M(s, 1, True)
        Mo = oracle.dense(pos, a=1.0, viscosity=eta, wall=True, wall_height=wall_height,
                          include_angular=True)
        assert np.allclose(M / nm1, Mo / nm1, atol=tol, rtol=tol), h
    nm2 = np.kron(np.array([[1, 1], [1, 1]]), np.ones((6, 6)))
    nm2 = np.zeros((12, 12))
    nm2[:6, :6] = 1 / (6 * np.pi * eta)
    nm2[6:, 6:] = 1 / (8 * np.pi * eta)
    nm2[6:, :6] = nm2[:6, 6:] = 1 / (6 * np.pi * eta)
    for off in (np.array([1.0, 0, 0]), np.array([0, 1.0, 0])):
        for sep in (3.0, 4.0, 8.0):
            for h in heights[::2]:
                c = c0 + [0, 0, h + wall_height]
                pos = np.array([c + sep * off / 2, c - sep * off / 2])
                s.setPositions(pos)
                M = compute_M(s, 2, True)
                Mo = oracle.dense(pos, a=1.0, viscosity=eta, wall=True, wall_height=wall_height,
                                  include_angular=True)
                assert np.allclose(M / nm2, Mo / nm2, atol=tol, rtol=tol), (sep, h)


@pytest.mark.parametrize("precision", ["float", "double"])
def test_self_mobility_and_symmetry(cuda, precision):
    """test_mobility_matrix.py: self mobility 1/(6 pi eta a), 1/(8 pi eta a^3)
    for every algorithm string, and |M - M^T| <= 5e-5."""
    from libmobility_gb300 import NBody
    a, eta = 0.9123, 1.123
    for alg in ("naive", "block", "fast", "advise"):
        s = NBody("open", "open", "open", precision=precision)
        s.setParameters(alg)
        s.initialize(viscosity=eta, hydrodynamicRadius=a, includeAngular=True)
        s.setPositions(np.zeros((1, 3)))
        lin, ang = s.Mdot(np.ones(3), 2 * np.ones(3))
        assert np.allclose(lin, np.ones(3) / (6 * np.pi * eta * a), rtol=0, atol=1e-7)
        assert np.allclose(ang, 2 * np.ones(3) / (8 * np.pi * eta * a ** 3), rtol=0, atol=1e-7)
    rng = np.random.default_rng(4)
    for pz in ("open", "single_wall"):
        for a in (1.0, 0.95, 1.12):
            for N in (1, 2, 3, 10):
                for ang in (False, True):
                    s = NBody("open", "open", pz, precision=precision)
                    s.setParameters(**({"wallHeight": 0.0} if pz == "single_wall" else {}))
                    s.initialize(viscosity=1.0, hydrodynamicRadius=a, includeAngular=ang)
                    p = rng.random((N, 3)) - 0.5
                    p[:, 2] += 0.5
                    s.setPositions(p * 10)
                    M = compute_M(s, N, ang)
                    assert np.allclose(M - M.T, 0, rtol=0, atol=5e-5)
                    assert np.all(np.linalg.eigvals(M).real > 0)
