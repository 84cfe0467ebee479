"""FP64 CPU oracle for libMobility's NBody RPY product and Lanczos sqrt(M) dW.

TEST INFRASTRUCTURE ONLY.  This module is the reference oracle for libmobility_gb300's
CUDA path.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline leg (and its ``--impl reference`` arm) import it; the product never
does.

Contents
--------
* ``mdot`` / ``dense`` -- ctypes front end of ``rpy_oracle.c`` (the pair
  physics of solvers/NBody/extra/hydrodynamicKernels.cuh:41-442 and the
  batched all-pairs loop of NbodyRPY.cu:119-147, in FP64), with the wall shift
  and below-the-wall check of solvers/NBody/mobility.h:124-148 and the block
  selection of NbodyRPY.cu:264-275.
* ``Lanczos`` -- a NumPy restatement of the reference Krylov solver
  include/lanczos/LanczosAlgorithm.cu:26-232 (same recurrence, breakdown
  rule, square root through the tridiagonal eigen-decomposition, successive
  iterate error and adaptive check schedule), in FP64 or FP32.
* ``ref_pair_mdot`` / ``RefLanczos`` -- the reference's own code compiled for
  this CPU by oracle/build.py (only where the reference checkout exists), used
  to pin the two restatements above.
"""
import ctypes
import math
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIB = None


class OracleError(RuntimeError):
    pass


def _lib():
    global _LIB
    if _LIB is None:
        path = HERE / "_build" / "liboracle.so"
        if not path.exists():
            from oracle import build as _b
            _b.build_oracle()
        _LIB = ctypes.CDLL(str(path))
        _LIB.orc_mdot.restype = ctypes.c_int
        _LIB.orc_dense.restype = ctypes.c_int
    return _LIB


class _Params(ctypes.Structure):
    _fields_ = [("t0", ctypes.c_double), ("r0", ctypes.c_double),
                ("rt0", ctypes.c_double), ("a", ctypes.c_double),
                ("wall", ctypes.c_int), ("useUF", ctypes.c_int),
                ("useUT", ctypes.c_int), ("useWT", ctypes.c_int),
                ("useWF", ctypes.c_int)]


def mobility_constants(viscosity, a):
    """t0, r0, rt0 of NBody::initialize, solvers/NBody/mobility.h:99-106."""
    t0 = 1.0 / (6.0 * math.pi * viscosity * a)
    rt0 = 1.0 / (8.0 * math.pi * viscosity * a * a)
    r0 = 1.0 / (8.0 * math.pi * viscosity * a * a * a)
    return t0, r0, rt0


def wall_frame(pos, wall, wall_height):
    """Shift z so the wall sits at 0 and reject particles below it
    (solvers/NBody/mobility.h:124-148)."""
    p = np.array(pos, dtype=np.float64).reshape(-1, 3).copy()
    if wall:
        if wall_height != 0:
            p[:, 2] -= wall_height
        if p.shape[0] and p[:, 2].min() < 0:
            raise OracleError("[Mobility] The center of a particle has fallen below the wall.")
    return p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def mdot(pos, F=None, T=None, *, a, viscosity, wall=False, wall_height=0.0,
         include_angular=False, nper_batch=None, rows=None, nthreads=None):
    """FP64 M.[F;T] -> (U, W); U, W are None when not produced.

    ``rows=(b, e)`` evaluates only target rows [b, e) (summed over all
    sources of their batch).  Output shape is (rows, 3)."""
    p = wall_frame(pos, wall, wall_height)
    N = p.shape[0]
    nb = N if nper_batch is None else int(nper_batch)
    Fa = None if F is None else np.ascontiguousarray(np.asarray(F, np.float64).reshape(N, 3))
    Ta = None if T is None else np.ascontiguousarray(np.asarray(T, np.float64).reshape(N, 3))
    t0, r0, rt0 = mobility_constants(viscosity, a)
    prm = _Params(t0, r0, rt0, a, int(bool(wall)), int(Fa is not None),
                  int(Ta is not None and include_angular),
                  int(Ta is not None and include_angular),
                  int(Fa is not None and include_angular))
    b, e = (0, N) if rows is None else rows
    U = np.zeros((e - b, 3))
    W = np.zeros((e - b, 3)) if include_angular else None
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    rc = _lib().orc_mdot(ctypes.byref(prm), _ptr(p), _ptr(Fa), _ptr(Ta), _ptr(U),
                         _ptr(W), ctypes.c_int64(N), ctypes.c_int64(nb),
                         ctypes.c_int64(b), ctypes.c_int64(e), ctypes.c_int(nthreads))
    if rc:
        raise OracleError("orc_mdot: bad arguments")
    return U, W


def dense(pos, *, a, viscosity, wall=False, wall_height=0.0,
          include_angular=False, nper_batch=None):
    """Dense FP64 mobility matrix, rows [U; W] x columns [F; T] as in the
    reference tests' compute_M (tests/utils.py:62-84)."""
    p = wall_frame(pos, wall, wall_height)
    N = p.shape[0]
    nb = N if nper_batch is None else int(nper_batch)
    n = (6 if include_angular else 3) * N
    M = np.zeros((n, n))
    t0, r0, rt0 = mobility_constants(viscosity, a)
    prm = _Params(t0, r0, rt0, a, int(bool(wall)), 1, 0, 0, 0)
    rc = _lib().orc_dense(ctypes.byref(prm), _ptr(p), ctypes.c_int64(N),
                          ctypes.c_int64(nb), ctypes.c_int(int(include_angular)), _ptr(M))
    if rc:
        raise OracleError("orc_dense: bad arguments")
    return M


def sqrtm_dense(M):
    """Symmetric square root through eigh (FP64)."""
    lam, Q = np.linalg.eigh(0.5 * (M + M.T))
    return (Q * np.sqrt(np.clip(lam, 0, None))) @ Q.T


# --------------------------------------------------------------------------
# Lanczos restatement, include/lanczos/LanczosAlgorithm.cu:26-232
# --------------------------------------------------------------------------

class LanczosNoConvergence(OracleError):
    pass


class LanczosNaN(OracleError):
    pass


def _tridiag_sqrt_e1(hdiag, hsup, dtype):
    """H^{1/2} e1 through the eigen-decomposition of the m x m tridiagonal
    matrix, KrylovSubspace::computeSquareRoot (LanczosAlgorithm.cu:48-85)."""
    from scipy.linalg import eigh_tridiagonal
    m = len(hdiag)
    d = np.asarray(hdiag, np.float64)
    e = np.asarray(hsup[: m - 1], np.float64)
    if m == 1:
        lam, P = d.copy(), np.ones((1, 1))
    else:
        lam, P = eigh_tridiagonal(d, e)
    with np.errstate(invalid="ignore"):
        s = np.sqrt(lam.astype(dtype)) * P[0, :].astype(dtype)
    return (P.astype(dtype) @ s).astype(dtype)


class Lanczos:
    """Stateful solver: keeps the adaptive convergence-check interval across
    calls as lanczos::Solver does (LanczosAlgorithm.h:266-284)."""

    def __init__(self, hard_limit=200, dtype=np.float64):
        self.hard_limit = hard_limit
        self.check_convergence_steps = 3
        self.dtype = np.dtype(dtype)

    def _register(self, steps):  # LanczosAlgorithm.cu:224-232
        if steps - 2 > self.check_convergence_steps:
            self.check_convergence_steps += 1
        else:
            self.check_convergence_steps = max(1, self.check_convergence_steps - 2)

    def run(self, matvec, z, tol, callback=None):
        """Returns (y, i): y = sqrt(M) z and the iteration index at return."""
        dt = self.dtype
        z = np.asarray(z, dt).ravel()
        n = z.size
        m_max = self.hard_limit
        V = np.zeros((m_max + 1, n), dt)
        hdiag = np.zeros(m_max + 1, dt)
        hsup = np.zeros(m_max + 1, dt)
        normz = dt.type(np.sqrt(np.dot(z.astype(np.float64), z.astype(np.float64))))
        V[0] = z * dt.type(1.0 / normz)
        old = np.zeros(n, dt)
        y = np.zeros(n, dt)
        k = min(self.check_convergence_steps, self.hard_limit - 2)
        for i in range(self.hard_limit):
            # KrylovSubspace::nextIteration, LanczosAlgorithm.cu:120-153
            w = np.asarray(matvec(V[i]), dt).ravel().copy()
            if i > 0:
                w -= hsup[i - 1] * V[i - 1]
            hdiag[i] = np.dot(w, V[i])
            w -= hdiag[i] * V[i]
            hsup[i] = dt.type(np.sqrt(np.dot(w.astype(np.float64), w.astype(np.float64))))
            tol_b = dt.type(1e-3) * hdiag[i] / normz
            if hsup[i] < tol_b:
                hsup[i] = 0
            if hsup[i] > 0:
                w *= dt.type(1.0 / hsup[i])
            else:
                w[:] = 0
                w[0] = 1
            V[i + 1] = w
            if i >= k or callback is not None:
                # computeCurrentResultEstimation, :158-167
                m = i + 1
                c = _tridiag_sqrt_e1(hdiag[:m], hsup[:m], dt)
                y = (normz * (V[:m].T @ c)).astype(dt)
                if i > 0:
                    # computeError, :202-222
                    prev = np.sqrt(np.dot(old.astype(np.float64), old.astype(np.float64)))
                    diff = np.sqrt(np.sum((old.astype(np.float64) - y) ** 2))
                    with np.errstate(divide="ignore", invalid="ignore"):
                        err = abs(diff / prev) if prev != 0 else (np.inf if diff > 0 else np.nan)
                    if np.isnan(err):
                        raise LanczosNaN("[Lanczos] Unknown error (found NaN in result guess)")
                    if callback is not None:
                        callback(i, float(err))
                    if err <= tol:
                        self._register(i)
                        return y, i
                old = y.copy()
        raise LanczosNoConvergence("[Lanczos] Could not converge")


# --------------------------------------------------------------------------
# The reference's own code compiled for this CPU (oracle/build.py)
# --------------------------------------------------------------------------

def reference_built():
    return (HERE / "_ref" / "libref_pair_d.so").exists()


_REF = {}


def _ref_lib(kind, dbl):
    key = (kind, dbl)
    if key not in _REF:
        path = HERE / "_ref" / f"libref_{kind}_{'d' if dbl else 'f'}.so"
        if not path.exists():
            raise OracleError(f"{path} not built (reference checkout absent)")
        _REF[key] = ctypes.CDLL(str(path))
    return _REF[key]


def ref_pair_mdot(pos_wall_frame, F=None, T=None, *, a, viscosity, wall=False,
                  include_angular=False, nper_batch=None, dtype=np.float64):
    """Reference pair code (hydrodynamicKernels.cuh) in `dtype` on the CPU.
    Positions must already be in the wall frame."""
    dt = np.dtype(dtype)
    lib = _ref_lib("pair", dt == np.float64)
    P = ctypes.POINTER(ctypes.c_double if dt == np.float64 else ctypes.c_float)
    p = np.ascontiguousarray(np.asarray(pos_wall_frame, dt).reshape(-1, 3))
    N = p.shape[0]
    Fa = None if F is None else np.ascontiguousarray(np.asarray(F, dt).reshape(N, 3))
    Ta = None if T is None else np.ascontiguousarray(np.asarray(T, dt).reshape(N, 3))
    U = np.zeros((N, 3), dt)
    W = np.zeros((N, 3), dt)
    t0, r0, rt0 = mobility_constants(viscosity, a)
    f = lambda x: None if x is None else x.ctypes.data_as(P)
    lib.ref_pair_mdot(ctypes.c_int(int(wall)), f(p), f(Fa), f(Ta), f(U), f(W),
                      ctypes.c_int64(N), ctypes.c_int64(N if nper_batch is None else nper_batch),
                      ctypes.c_double(t0), ctypes.c_double(r0), ctypes.c_double(rt0),
                      ctypes.c_double(a), ctypes.c_int(int(include_angular)))
    return U, (W if include_angular else None)


class RefLanczos:
    """The reference lanczos::Solver (LanczosAlgorithm.{h,cu}) compiled for
    the CPU with host stand-ins for cuBLAS/thrust/LAPACKE, on a dense M."""

    def __init__(self, dtype=np.float64, hard_limit=200):
        self.dt = np.dtype(dtype)
        self.lib = _ref_lib("lanczos", self.dt == np.float64)
        self.lib.ref_lanczos_new.restype = ctypes.c_void_p
        self.lib.ref_lanczos_free.argtypes = [ctypes.c_void_p]
        self.h = self.lib.ref_lanczos_new(ctypes.c_int(hard_limit))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_lanczos_free(ctypes.c_void_p(self.h))
            self.h = None

    def run(self, M, z, tol, with_callback=False):
        dt = self.dt
        P = ctypes.POINTER(ctypes.c_double if dt == np.float64 else ctypes.c_float)
        Ma = np.ascontiguousarray(np.asarray(M, dt))
        za = np.ascontiguousarray(np.asarray(z, dt).ravel())
        n = za.size
        y = np.zeros(n, dt)
        err = ctypes.create_string_buffer(256)
        if with_callback:
            res = np.zeros(256)
            its = np.zeros(256, np.int32)
            nres = ctypes.c_int(0)
            it = self.lib.ref_lanczos_solve(
                ctypes.c_void_p(self.h), Ma.ctypes.data_as(P), ctypes.c_int(n),
                za.ctypes.data_as(P), ctypes.c_double(tol), y.ctypes.data_as(P),
                res.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                its.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ctypes.c_int(256),
                ctypes.byref(nres), err, ctypes.c_int(256))
            k = min(nres.value, 256)
            hist = (its[:k].copy(), res[:k].copy())
        else:
            it = self.lib.ref_lanczos_solve_nocb(
                ctypes.c_void_p(self.h), Ma.ctypes.data_as(P), ctypes.c_int(n),
                za.ctypes.data_as(P), ctypes.c_double(tol), y.ctypes.data_as(P),
                err, ctypes.c_int(256))
            hist = None
        if it < 0:
            raise OracleError(err.value.decode())
        return y, it, hist
