"""Ensembles of independent NBody systems (no counterpart in the reference).

An ``Ensemble`` holds many systems of uneven size, each open or above its own
bottom wall, sharing one viscosity and hydrodynamic radius (forces only, no
torques).  Every system behaves as its own ``NBody`` solver; the work of all
systems runs together on the GPU (C ABI: ``lmg_ensemble_*`` in
include/libmobility_gb300.h).

    from libmobility_gb300.ensemble import Ensemble
    e = Ensemble(precision="float")
    e.setSystems(sizes, geometry, wallHeights)   # geometry: "open"/"single_wall" or 0/1
    e.initialize(viscosity=1.0, hydrodynamicRadius=1.0, tolerance=1e-6)
    e.setPositions(pos)                  # all systems concatenated, (sum N, 3)
    U = e.Mdot(F)                        # M F per system
    U, its, errs, ms = e.sqrtMdotW(dW)   # M^{1/2} dW per system, Lanczos per system
"""
import ctypes
import json

import numpy as np

from . import _capi
from .nbody import _PRECISIONS, _NP, _Arr, _is_torch, _torch, _default_precision

_GEOM = {"open": 0, "single_wall": 1, 0: 0, 1: 1}


class Ensemble:
    precision = _default_precision()

    def __init__(self, precision=None):
        lib = _capi.load()
        p = precision or type(self).precision
        if p not in _PRECISIONS:
            raise RuntimeError("precision must be 'float' or 'double'")
        self.precision = p
        self._h = None
        h = ctypes.c_void_p()
        _capi.check(lib.lmg_ensemble_create(_PRECISIONS[p], ctypes.byref(h)))
        self._lib = lib
        self._h = h
        self._sizes = None

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.lmg_ensemble_destroy(self._h)
            self._h = None

    def _check(self, st):
        _capi.check(st, self._h, ensemble=True)

    def _bind_stream(self, *objs):
        """Work goes on the caller's current torch stream when CUDA tensors
        are involved, else on the handle's own stream."""
        for x in objs:
            if x is None:
                continue
            cuda = x.is_cuda if isinstance(x, _Arr) else (_is_torch(x) and x.is_cuda)
            if cuda:
                stream = _torch().cuda.current_stream(x.device).cuda_stream
                self._check(self._lib.lmg_ensemble_set_stream(self._h, ctypes.c_void_p(stream)))
                return
        self._check(self._lib.lmg_ensemble_set_stream(self._h, _capi.LMG_OWN_STREAM))

    @property
    def numberParticles(self):
        return int(np.sum(self._sizes)) if self._sizes is not None else 0

    def setSystems(self, sizes, geometry, wallHeights=None):
        sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        try:
            geom = np.ascontiguousarray([_GEOM[g] for g in geometry], dtype=np.int32)
        except KeyError as exc:
            raise RuntimeError("geometry entries must be 'open' or 'single_wall'") from exc
        if geom.size != sizes.size:
            raise RuntimeError("sizes and geometry must have one entry per system")
        hp = None
        if wallHeights is not None:
            wh = np.ascontiguousarray(wallHeights, dtype=np.float64)
            if wh.size != sizes.size:
                raise RuntimeError("wallHeights must have one entry per system")
            self._wh = wh
            hp = ctypes.c_void_p(wh.ctypes.data)
        self._check(self._lib.lmg_ensemble_set_systems(
            self._h, int(sizes.size), ctypes.c_void_p(sizes.ctypes.data),
            ctypes.c_void_p(geom.ctypes.data), hp))
        self._sizes = sizes

    def initialize(self, viscosity, hydrodynamicRadius, tolerance=1e-4, seed=0, autotune=True):
        self._check(self._lib.lmg_ensemble_initialize(
            self._h, float(viscosity), float(hydrodynamicRadius), float(tolerance),
            int(seed), 1 if autotune else 0))

    def setPositions(self, positions):
        a = _Arr(positions, self.precision)
        self._bind_stream(a)
        self._check(self._lib.lmg_ensemble_set_positions(
            self._h, ctypes.c_void_p(a.ptr) if a.ptr else None, a.size))

    def _out(self, like):
        n = 3 * self.numberParticles
        shape = like.shape if (like is not None and like.size == n) else (n // 3, 3)
        if like is not None and like.framework == "torch":
            torch = _torch()
            dt = torch.float32 if self.precision == "float" else torch.float64
            return torch.zeros(shape, dtype=dt, device=like.device)
        return np.zeros(shape, dtype=_NP[self.precision])

    @staticmethod
    def _ptr(x):
        if _is_torch(x):
            return ctypes.c_void_p(x.data_ptr()), x.numel()
        return ctypes.c_void_p(x.ctypes.data), x.size

    def Mdot(self, forces):
        """U = M F for every system (forces of all systems concatenated)."""
        F = _Arr(forces, self.precision)
        U = self._out(F)
        self._bind_stream(F, U)
        up, un = self._ptr(U)
        self._check(self._lib.lmg_ensemble_mdot(
            self._h, ctypes.c_void_p(F.ptr) if F.ptr else None, F.size, up, un))
        return U

    def sqrtMdotW(self, dW=None, prefactor=1.0, out=None):
        """Returns (U, iterations, errors, completion_ms): U = prefactor *
        M^{1/2} dW per system (added to `out` when given; dW None draws the
        noise from the seed), and per system the Lanczos iterations, the last
        successive-iterate error and the host time in ms from the start of the
        call until its result was known."""
        W = _Arr(dW, self.precision) if dW is not None else None
        if out is None:
            out = self._out(W)
        self._bind_stream(W, out)
        op, on = self._ptr(out)
        nsys = self._sizes.size
        its = np.zeros(nsys, dtype=np.int32)
        errs = np.zeros(nsys, dtype=np.float64)
        ms = np.zeros(nsys, dtype=np.float64)
        self._check(self._lib.lmg_ensemble_sqrt_mdot_w(
            self._h, ctypes.c_void_p(W.ptr) if W is not None else None,
            W.size if W is not None else 0, op, on, float(prefactor),
            ctypes.c_void_p(its.ctypes.data), ctypes.c_void_p(errs.ctypes.data),
            ctypes.c_void_p(ms.ctypes.data)))
        return out, its, errs, ms

    def describe(self):
        """Groups of systems, their launch plans and autotuning timings."""
        buf = ctypes.create_string_buffer(1 << 20)
        self._check(self._lib.lmg_ensemble_describe(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())
