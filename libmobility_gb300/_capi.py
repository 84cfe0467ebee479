"""ctypes binding of the C ABI declared in include/libmobility_gb300.h.

This is the reference-side stub a Python caller uses in place of libMobility's
nanobind module (include/MobilityInterface/pythonify.h); the library itself is
``liblmg_gb300.so`` built in-tree by ``libmobility_gb300._build``.  Loading
fails loudly when the library is missing: there is no fallback path.
"""
import ctypes
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("LIBMOBILITY_GB300_LIB", _PKG / "liblmg_gb300.so"))

LMG_OK = 0
LMG_OWN_STREAM = ctypes.c_void_p(2**64 - 1)
STATUS_NAMES = {
    0: "LMG_OK", 1: "LMG_ERR_INVALID_ARGUMENT", 2: "LMG_ERR_NOT_INITIALIZED",
    3: "LMG_ERR_NO_POSITIONS", 4: "LMG_ERR_BELOW_WALL", 5: "LMG_ERR_NO_CONVERGENCE",
    6: "LMG_ERR_NAN", 7: "LMG_ERR_TIMEOUT", 8: "LMG_ERR_CUDA", 9: "LMG_ERR_NO_DEVICE",
    10: "LMG_ERR_INTERNAL",
}

LANCZOS_CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_double, ctypes.c_void_p)

# name -> (restype, argtypes), exactly the declarations of the public header
_VP, _SZ, _D, _I = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int
SIGNATURES = {
    "lmg_version": (ctypes.c_char_p, []),
    "lmg_last_error": (ctypes.c_char_p, [_VP]),
    "lmg_create": (_I, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _I,
                        ctypes.POINTER(_VP)]),
    "lmg_create_error": (ctypes.c_char_p, []),
    "lmg_create_self_mobility": (_I, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _I,
                                      ctypes.POINTER(_VP)]),
    "lmg_destroy": (_I, [_VP]),
    "lmg_set_stream": (_I, [_VP, _VP]),
    "lmg_set_lanczos_iteration_limit": (_I, [_VP, _I]),
    "lmg_set_parameters_nbody": (_I, [_VP, ctypes.c_char_p, _I, _I, _I, _D, _D]),
    "lmg_initialize": (_I, [_VP, _D, _D, _I, _D, ctypes.c_uint64, LANCZOS_CALLBACK, _VP]),
    "lmg_set_positions": (_I, [_VP, _VP, _SZ]),
    "lmg_get_number_particles": (_I, [_VP, ctypes.POINTER(ctypes.c_int64)]),
    "lmg_get_include_angular": (_I, [_VP, ctypes.POINTER(_I)]),
    "lmg_mdot": (_I, [_VP, _VP, _SZ, _VP, _SZ, _VP, _SZ, _VP, _SZ]),
    "lmg_mdot_rows": (_I, [_VP, ctypes.c_int64, ctypes.c_int64, _VP, _SZ, _VP, _SZ, _VP, _SZ,
                           _VP, _SZ]),
    "lmg_sqrt_mdot_w": (_I, [_VP, _VP, _SZ, _VP, _SZ, _D]),
    "lmg_sqrt_mdot_w_noise": (_I, [_VP, _VP, _SZ, _VP, _SZ, _VP, _SZ, _D,
                                   ctypes.POINTER(_I), ctypes.POINTER(_D)]),
    "lmg_langevin_velocities": (_I, [_VP, _D, _D, _VP, _SZ, _VP, _SZ, _VP, _SZ, _VP, _SZ]),
    "lmg_div_m": (_I, [_VP, _VP, _SZ, _VP, _SZ, _D]),
    "lmg_clean": (_I, [_VP]),
    "lmg_synchronize": (_I, [_VP]),
    "lmg_precision_name": (ctypes.c_char_p, [_VP]),
    "lmg_set_preconditioner": (_I, [_VP, ctypes.c_char_p, _VP, _SZ]),
    "lmg_get_preconditioner_solve_iterations": (_I, [_VP, ctypes.POINTER(_I)]),
    "lmg_mdot_noalloc_f32": (_I, [_VP, _VP, _VP, _VP, _VP, ctypes.c_int64, ctypes.c_int64, _I,
                                 _D, _D, _I, _VP, ctypes.c_char_p, _SZ]),
    "lmg_ensemble_create": (_I, [_I, ctypes.POINTER(_VP)]),
    "lmg_ensemble_destroy": (_I, [_VP]),
    "lmg_ensemble_last_error": (ctypes.c_char_p, [_VP]),
    "lmg_ensemble_set_stream": (_I, [_VP, _VP]),
    "lmg_ensemble_set_systems": (_I, [_VP, _I, _VP, _VP, _VP]),
    "lmg_ensemble_initialize": (_I, [_VP, _D, _D, _D, ctypes.c_uint64, _I]),
    "lmg_ensemble_set_positions": (_I, [_VP, _VP, _SZ]),
    "lmg_ensemble_mdot": (_I, [_VP, _VP, _SZ, _VP, _SZ]),
    "lmg_ensemble_sqrt_mdot_w": (_I, [_VP, _VP, _SZ, _VP, _SZ, _D, _VP, _VP, _VP]),
    "lmg_ensemble_describe": (_I, [_VP, ctypes.c_char_p, _SZ]),
}

_lib = None


def load():
    """Load liblmg_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"libmobility_gb300: native library {LIB_PATH} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python -m libmobility_gb300._build`")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    lib.lmg_internal_tridiag_sqrt_e1.restype = _I
    lib.lmg_internal_tridiag_sqrt_e1.argtypes = [_VP, _VP, _I, _VP]
    lib.lmg_internal_tridiag_sqrt_e1_quad.restype = _I
    lib.lmg_internal_tridiag_sqrt_e1_quad.argtypes = [_VP, _VP, _I, _VP]
    lib.lmg_internal_launch_count.restype = ctypes.c_ulonglong
    lib.lmg_internal_launch_count.argtypes = []
    lib.lmg_internal_mdot_plan_override.restype = _I
    lib.lmg_internal_mdot_plan_override.argtypes = [_I, _I]
    lib.lmg_internal_fma_probe.restype = _I
    lib.lmg_internal_fma_probe.argtypes = [_I, _I, _I, _VP, _VP]
    lib.lmg_internal_fma2_probe.restype = _I
    lib.lmg_internal_fma2_probe.argtypes = [_I, _I, _I, _VP, _VP]
    lib.lmg_internal_bounds_status.restype = ctypes.c_ulonglong
    lib.lmg_internal_bounds_status.argtypes = [_I, _I]
    lib.lmg_internal_bounds_probe.restype = _I
    lib.lmg_internal_bounds_probe.argtypes = []
    lib.lmg_internal_dfma_probe.restype = _I
    lib.lmg_internal_dfma_probe.argtypes = [_I, _I, _I, _VP, _VP]
    lib.lmg_internal_sym_plan.restype = _I
    lib.lmg_internal_sym_plan.argtypes = [_I, _I, ctypes.c_longlong, _I, _VP, _VP, _VP, _VP, _VP]
    _F = ctypes.c_float
    internal = {
        "lmg_internal_gemm": [_I, _I, _I, _I, _I, _VP, _I, _VP, _I, _VP, _I, _VP, _I, _F, _VP],
        "lmg_internal_tanh_backward": [_SZ, _VP, _VP, _VP],
        "lmg_internal_tc_gemm": [_I, _I, _I, _VP, _I, _VP, _I, _VP, _I, _VP, _I, _VP],
        "lmg_internal_tc_status": [_I],
        "lmg_internal_precond_tc": [_I],
        "lmg_internal_mse_grad": [_SZ, _VP, _VP, _VP, _F, _VP, _VP],
        "lmg_internal_colsum": [_I, _I, _VP, _VP, _VP],
        "lmg_internal_adam": [_SZ, _VP, _VP, _VP, _VP, _F, _F, _F, _F, _I, _VP],
        "lmg_internal_knn": [_VP, _I, _I, _VP, _VP],
        "lmg_internal_precond_build": [_VP, _VP, _I, _VP, _F, _F, _VP, _VP],
        "lmg_internal_precond_apply": [_VP, _VP, _I, _VP, _VP, _I, _VP],
        "lmg_internal_knn_k": [_I, _VP, _I, _I, _VP, _VP],
        "lmg_internal_precond_build_kh": [_I, _I, _VP, _VP, _I, _VP, _F, _F, _VP, _VP],
        "lmg_internal_precond_build_wall": [_I, _I, _VP, _VP, _I, _VP, _F, _F, _VP, _VP],
        "lmg_internal_precond_apply_k": [_I, _VP, _VP, _I, _VP, _VP, _I, _VP],
        "lmg_internal_precond_apply_kh": [_I, _VP, _I, _VP, _I, _VP, _VP, _I, _VP, _VP],
        "lmg_internal_lanczos_phase_timing": [_VP, _I],
        "lmg_internal_lanczos_phase_times": [_VP, _VP],
        "lmg_internal_barrier_timeout_probe": [_VP],
        "lmg_internal_sym_override": [_I, _I],
        "lmg_internal_sym_trace": [_VP],
        "lmg_internal_lanczos_step_mode": [_I],
        "lmg_internal_lanczos_step_shape": [_I, _I],
        "lmg_internal_classify_pointer": [_I, _I, _I],
        "lmg_internal_lanczos_device_sqrt": [_I],
        "lmg_internal_lanczos_lookahead": [_I],
        "lmg_internal_lanczos_check_wait": [_I],
    }
    for name, args in internal.items():
        fn = getattr(lib, name)
        fn.restype = _I
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, handle=None, ensemble=False):
    """Raise RuntimeError with the library's message for a failed call (the
    reference's exceptions surface as RuntimeError through nanobind)."""
    if status == LMG_OK:
        return
    lib = load()
    if handle is not None:
        get = lib.lmg_ensemble_last_error if ensemble else lib.lmg_last_error
        msg = get(handle).decode()
    else:
        msg = lib.lmg_create_error().decode()
    err = RuntimeError(msg or STATUS_NAMES.get(status, str(status)))
    err.status = status
    raise err
