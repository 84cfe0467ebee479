"""Python NBody class with the API of libMobility's Python module.

Mirrors ``define_module_content`` in include/MobilityInterface/pythonify.h:
364-397 (constructor with three periodicity strings, ``initialize``,
``setPositions``, ``Mdot``, ``sqrtMdotW``, ``LangevinVelocities``, ``divM``,
``clean``, ``precision``) plus the NBody ``setParameters`` of
solvers/NBody/python_wrapper.cu:50-61, including the argument defaults, the
shape rules of ``check_and_get_shape`` / ``setup_arrays`` (pythonify.h:83-149)
and the rule that outputs take the framework, device and shape of the input
(numpy arrays, and torch tensors on the CPU or on CUDA).  Every error is a
RuntimeError, as nanobind raises for the reference.

All work goes through the C ABI of ``liblmg_gb300.so`` (see _capi.py); this
module only converts arrays.
"""
import ctypes
import os

import numpy as np

from . import _capi

_PRECISIONS = {"float": 0, "double": 1}
_NP = {"float": np.float32, "double": np.float64}
_SHAPE_MSG = ("[libMobility] The input arrays for positions, forces, and torques must each "
              "have shape (N, 3) or (3*N).")
_SIZE_MSG = ("[libMobility] The input arrays for positions, forces, and torques must each "
             "have total size 3*N.")


def _default_precision():
    p = os.environ.get("LIBMOBILITY_GB300_PRECISION", "float")
    if p not in _PRECISIONS:
        raise RuntimeError(f"LIBMOBILITY_GB300_PRECISION must be float or double, not {p!r}")
    return p


def _torch():
    import torch
    return torch


def _is_torch(a):
    return type(a).__module__.startswith("torch")


class _Arr:
    """A C-contiguous array of the solver precision, with where it lives."""

    __slots__ = ("obj", "ptr", "size", "framework", "device", "shape", "is_cuda")

    def __init__(self, a, precision):
        if _is_torch(a):
            torch = _torch()
            dt = torch.float32 if precision == "float" else torch.float64
            t = a.detach()
            if t.dtype != dt:
                t = t.to(dt)
            t = t.contiguous()
            self.obj = t
            self.ptr = t.data_ptr() if t.numel() else None
            self.size = t.numel()
            self.framework = "torch"
            self.device = t.device
            self.is_cuda = t.is_cuda
            self.shape = tuple(t.shape)
        else:
            arr = np.ascontiguousarray(np.asarray(a), dtype=_NP[precision])
            self.obj = arr
            self.ptr = arr.ctypes.data if arr.size else None
            self.size = arr.size
            self.framework = "numpy"
            self.device = "cpu"
            self.is_cuda = False
            self.shape = arr.shape


def _check_and_get_shape(arr):
    """pythonify.h:83-107"""
    if arr.size == 0:
        return ()
    if arr.size % 3 != 0:
        raise RuntimeError(_SIZE_MSG)
    n = arr.size // 3
    nd = len(arr.shape)
    if (nd == 1 and arr.shape[0] != 3 * n) or (nd == 2 and arr.shape[1] != 3) or nd not in (1, 2):
        raise RuntimeError(_SHAPE_MSG)
    return tuple(arr.shape)


class NBody:
    """All-pairs Rotne-Prager-Yamakawa mobility, open space or above a single
    bottom wall, evaluated by hand-written sm_103a CUDA kernels.

    Drop-in for libMobility's ``NBody``: same constructor, methods, argument
    names and defaults.  ``precision`` ("float" or "double") is a class
    attribute as in the reference; it is taken from the environment variable
    LIBMOBILITY_GB300_PRECISION at import and can be overridden per instance
    with the ``precision=`` keyword.
    """

    precision = _default_precision()
    _create = "lmg_create"

    def __init__(self, periodicityX, periodicityY, periodicityZ, precision=None):
        lib = _capi.load()
        p = precision or type(self).precision
        if p not in _PRECISIONS:
            raise RuntimeError("precision must be 'float' or 'double'")
        self.precision = p
        self._h = None
        h = ctypes.c_void_p()
        create = getattr(lib, self._create)
        _capi.check(create(str(periodicityX).encode(), str(periodicityY).encode(),
                           str(periodicityZ).encode(), _PRECISIONS[p], ctypes.byref(h)))
        self._lib = lib
        self._h = h
        self._wall = periodicityZ == "single_wall"
        self._cb = None
        self._last_shape = ()
        self._last_framework = "numpy"
        self._last_device = "cpu"
        self._include_angular = False
        self._initialized = False

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.lmg_destroy(self._h)
            self._h = None

    # -- helpers -----------------------------------------------------------
    def _check(self, st):
        _capi.check(st, self._h)

    def _arr(self, a):
        if a is None:
            return None
        r = _Arr(a, self.precision)
        return r if r.size else None

    def _bind_stream(self, *objs):
        """Issue the work on the caller's current torch stream when CUDA
        tensors (inputs as _Arr, or output tensors) are involved, so it is
        ordered with the caller's own work (the default stream included);
        otherwise on the handle's private stream."""
        for x in objs:
            if x is None:
                continue
            cuda = x.is_cuda if isinstance(x, _Arr) else (_is_torch(x) and x.is_cuda)
            if cuda:
                stream = _torch().cuda.current_stream(x.device).cuda_stream
                self._check(self._lib.lmg_set_stream(self._h, ctypes.c_void_p(stream)))
                return
        self._check(self._lib.lmg_set_stream(self._h, _capi.LMG_OWN_STREAM))

    def setPreconditioner(self, kind="mlp", weights=None):
        """Learned sparse preconditioner for sqrtMdotW (no counterpart in
        the reference): "mlp" uses the network shipped in
        libmobility_gb300/weights for the handle's geometry (the wall network
        for a single wall when one is shipped), or the .npz given as
        `weights`; "none"
        restores plain Lanczos.  The statistics of the samples do not depend
        on it, only the number of Lanczos iterations."""
        if kind == "none":
            self._check(self._lib.lmg_set_preconditioner(self._h, b"none", None, 0))
            return
        from . import precond
        params = np.ascontiguousarray(
            precond.load_weights(weights, wall=self._wall)
            if not isinstance(weights, np.ndarray) else weights, dtype=np.float32)
        self._prec_params = params
        self._check(self._lib.lmg_set_preconditioner(self._h, str(kind).encode(),
                                                     ctypes.c_void_p(params.ctypes.data),
                                                     params.size))

    def lastPreconditionerSolveIterations(self):
        it = ctypes.c_int()
        self._check(self._lib.lmg_get_preconditioner_solve_iterations(self._h, ctypes.byref(it)))
        return it.value

    def _lanczos_phase_timing(self, on=True):
        """Measurement hook: time the Krylov vector updates and the convergence
        checks of every following sqrtMdotW on the device (resets the sums)."""
        self._check(self._lib.lmg_internal_lanczos_phase_timing(self._h, int(bool(on))))

    def _lanczos_phase_times(self):
        """Sums since the timing was switched on: milliseconds and algorithmic
        bytes of the vector updates and of the checks, iterations issued
        (including the one issued ahead of the last check), checks, solves,
        milliseconds of the operator (all iterations) and, with the learned
        preconditioner, of its build and of the final P solve."""
        out = (ctypes.c_double * 10)()
        self._check(self._lib.lmg_internal_lanczos_phase_times(self._h, out))
        keys = ("vector_ms", "vector_bytes", "check_ms", "check_bytes", "iterations",
                "checks", "solves", "operator_ms", "build_ms", "psolve_ms")
        return dict(zip(keys, list(out)))

    def setLanczosIterationLimit(self, limit):
        """lanczos::Solver::setIterationHardLimit (LanczosAlgorithm.h:272-274)."""
        self._check(self._lib.lmg_set_lanczos_iteration_limit(self._h, int(limit)))

    def _zeros(self, shape, framework, device):
        if framework == "torch":
            torch = _torch()
            dt = torch.float32 if self.precision == "float" else torch.float64
            return torch.zeros(shape, dtype=dt, device=device)
        return np.zeros(shape, dtype=_NP[self.precision])

    @staticmethod
    def _ptr(x):
        if x is None:
            return None, 0
        if _is_torch(x):
            return ctypes.c_void_p(x.data_ptr()), x.numel()
        return ctypes.c_void_p(x.ctypes.data), x.size

    # -- interface ---------------------------------------------------------
    def setParameters(self, algorithm="advise", Nbatch=-1, NperBatch=-1, wallHeight=None,
                      delta=1e-3):
        """NBody parameters (solvers/NBody/python_wrapper.cu:50-61)."""
        has_wh = wallHeight is not None
        self._check(self._lib.lmg_set_parameters_nbody(
            self._h, str(algorithm).encode(), int(Nbatch), int(NperBatch), int(has_wh),
            float(wallHeight) if has_wh else 0.0, float(delta)))

    def initialize(self, viscosity, hydrodynamicRadius, includeAngular=False, tolerance=1e-4,
                   seed=None, lanczos_callback=None):
        """pythonify.h:241-260; seed None draws a random seed."""
        cb = None
        if lanczos_callback is not None:
            user_cb = lanczos_callback

            def _trampoline(i, err, _user):
                user_cb(i, err)
            cb = _capi.LANCZOS_CALLBACK(_trampoline)
        self._cb = cb
        s = 0 if seed is None else int(seed) & 0xFFFFFFFFFFFFFFFF
        self._check(self._lib.lmg_initialize(
            self._h, float(viscosity), float(hydrodynamicRadius), int(bool(includeAngular)),
            float(tolerance), ctypes.c_uint64(s),
            cb if cb is not None else _capi.LANCZOS_CALLBACK(), None))
        self._include_angular = bool(includeAngular)
        self._initialized = True

    def setPositions(self, positions):
        """pythonify.h:262-271"""
        p = _Arr(positions, self.precision)
        shape = _check_and_get_shape(p)
        self._bind_stream(p)
        self._check(self._lib.lmg_set_positions(
            self._h, ctypes.c_void_p(p.ptr) if p.ptr else None, p.size))
        self._last_shape = shape
        self._last_framework = p.framework
        self._last_device = p.device

    def getNumberParticles(self):
        n = ctypes.c_int64()
        self._check(self._lib.lmg_get_number_particles(self._h, ctypes.byref(n)))
        return n.value

    def _setup_arrays(self, forces, torques):
        """pythonify.h:109-149"""
        N = self.getNumberParticles()
        f = self._arr(forces)
        t = self._arr(torques)
        if f is not None and f.size != 3 * N:
            raise RuntimeError("The forces array must have size 3*N.")
        if t is not None and t.size != 3 * N:
            raise RuntimeError("The torques array must have size 3*N.")
        src = f if f is not None else t
        framework = src.framework if src is not None else "numpy"
        device = src.device if src is not None else "cpu"
        f_shape = _check_and_get_shape(src) if src is not None else ()
        mf = self._zeros(f_shape, framework, device) if src is not None else None
        mt = None
        if not self._include_angular:
            if t is not None:
                raise RuntimeError(
                    "The solver was configured without including angular velocities. Set "
                    "includeAngular to true when initializing if you want to use torques")
        else:
            t_shape = f_shape if t is None else _check_and_get_shape(t)
            mt = self._zeros(t_shape, framework, device) if src is not None else None
        return f, t, mf, mt

    def Mdot(self, forces=None, torques=None):
        """M.[F;T] -> (linear, angular); angular is None without includeAngular."""
        f, t, mf, mt = self._setup_arrays(forces, torques)
        if f is None and t is None:
            if self.getNumberParticles() <= 0:
                raise RuntimeError(
                    "[Mobility] Positions have 0 particles. Did you call setPositions?")
            raise RuntimeError("[libMobility] Mdot needs forces and/or torques")
        self._bind_stream(f, t)
        up, un = self._ptr(mf)
        wp, wn = self._ptr(mt)
        self._check(self._lib.lmg_mdot(
            self._h, ctypes.c_void_p(f.ptr) if f else None, f.size if f else 0,
            ctypes.c_void_p(t.ptr) if t else None, t.size if t else 0, up, un, wp, wn))
        return mf, mt

    def Mdot_rows(self, row_begin, row_end, forces=None, torques=None):
        """Rows [row_begin, row_end) of M.[F;T] for forces/torques of all N
        particles -> (linear, angular), each of shape (row_end - row_begin, 3);
        the product of one rank of a row-partitioned solve (no counterpart in
        the reference, whose Mdot is solvers/NBody/mobility.h:166-182)."""
        f = self._arr(forces)
        t = self._arr(torques)
        N = self.getNumberParticles()
        if f is not None and f.size != 3 * N:
            raise RuntimeError("The forces array must have size 3*N.")
        if t is not None and t.size != 3 * N:
            raise RuntimeError("The torques array must have size 3*N.")
        if t is not None and not self._include_angular:
            raise RuntimeError(
                "The solver was configured without including angular velocities. Set "
                "includeAngular to true when initializing if you want to use torques")
        src = f if f is not None else t
        if src is None:
            raise RuntimeError("[libMobility] Mdot needs forces and/or torques")
        rows = int(row_end) - int(row_begin)
        shape = (max(rows, 0), 3)
        mf = self._zeros(shape, src.framework, src.device)
        mt = self._zeros(shape, src.framework, src.device) if self._include_angular else None
        self._bind_stream(f, t)
        up, un = self._ptr(mf)
        wp, wn = self._ptr(mt)
        self._check(self._lib.lmg_mdot_rows(
            self._h, int(row_begin), int(row_end),
            ctypes.c_void_p(f.ptr) if f else None, f.size if f else 0,
            ctypes.c_void_p(t.ptr) if t else None, t.size if t else 0, up, un, wp, wn))
        return mf, mt

    def _fresh_outputs(self):
        mf = self._zeros(self._last_shape, self._last_framework, self._last_device)
        mt = (self._zeros(self._last_shape, self._last_framework, self._last_device)
              if self._include_angular else None)
        return mf, mt

    def sqrtMdotW(self, prefactor=1.0):
        """prefactor * M^{1/2} dW with the shape of the last positions."""
        if self.getNumberParticles() <= 0:
            raise RuntimeError("[libMobility] The number of particles is not set. Did you "
                               "forget to call setPositions?")
        mf, mt = self._fresh_outputs()
        self._bind_stream(mf, mt)
        up, un = self._ptr(mf)
        wp, wn = self._ptr(mt)
        self._check(self._lib.lmg_sqrt_mdot_w(self._h, up, un, wp, wn, float(prefactor)))
        return mf, mt

    def sqrtMdotW_noise(self, dW, prefactor=1.0):
        """prefactor * M^{1/2} dW for a given Gaussian vector dW ([dW_F; dW_T]),
        returning (linear, angular, iterations, residual)."""
        if self.getNumberParticles() <= 0:
            raise RuntimeError("[libMobility] The number of particles is not set. Did you "
                               "forget to call setPositions?")
        z = _Arr(dW, self.precision)
        mf, mt = self._fresh_outputs()
        self._bind_stream(mf, mt)
        up, un = self._ptr(mf)
        wp, wn = self._ptr(mt)
        it = ctypes.c_int()
        res = ctypes.c_double()
        self._check(self._lib.lmg_sqrt_mdot_w_noise(
            self._h, ctypes.c_void_p(z.ptr), z.size, up, un, wp, wn, float(prefactor),
            ctypes.byref(it), ctypes.byref(res)))
        return mf, mt, it.value, res.value

    def LangevinVelocities(self, dt, kbt, forces=None, torques=None):
        """pythonify.h:273-294 / MobilityInterface.h:191-206"""
        f, t, mf, mt = self._setup_arrays(forces, torques)
        if f is None:
            mf = self._zeros(self._last_shape, self._last_framework, self._last_device)
        if self._include_angular and t is None:
            mt = self._zeros(self._last_shape, self._last_framework, self._last_device)
        if self.getNumberParticles() <= 0:
            raise RuntimeError("[libMobility] The number of particles is not set. Did you "
                               "forget to call setPositions?")
        self._bind_stream(f, t, mf, mt)
        up, un = self._ptr(mf)
        wp, wn = self._ptr(mt)
        self._check(self._lib.lmg_langevin_velocities(
            self._h, float(dt), float(kbt), ctypes.c_void_p(f.ptr) if f else None,
            f.size if f else 0, ctypes.c_void_p(t.ptr) if t else None, t.size if t else 0,
            up, un, wp, wn))
        return mf, mt

    def divM(self, prefactor=1.0):
        """pythonify.h:329-345: thermal drift, zero for open boundaries."""
        if self.getNumberParticles() <= 0:
            raise RuntimeError("[libMobility] The number of particles is not set. Did you "
                               "forget to call setPositions?")
        mf, mt = self._fresh_outputs()
        self._bind_stream(mf, mt)
        up, un = self._ptr(mf)
        wp, wn = self._ptr(mt)
        self._check(self._lib.lmg_div_m(self._h, up, un, wp, wn, float(prefactor)))
        return mf, mt

    def clean(self):
        """Frees the solver's Lanczos storage and scratch."""
        self._check(self._lib.lmg_clean(self._h))


class SelfMobility(NBody):
    """libMobility's SelfMobility (solvers/SelfMobility/mobility.h): no
    hydrodynamic interactions, mobility 1/(6 pi eta a) I (and 1/(8 pi eta a^3) I
    for rotations), computed on the host through the same C ABI."""

    _create = "lmg_create_self_mobility"

    def setParameters(self, parameter=None):
        """Accepted and ignored, as in the reference (mobility.h:52-54)."""
        return None

