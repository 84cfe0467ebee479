"""libmobility_gb300: GB300-native (sm_103a) NBody Rotne-Prager-Yamakawa
mobility solver with the interface of libMobility's NBody.

    from libmobility_gb300 import NBody
    s = NBody("open", "open", "single_wall")
    s.setParameters(wallHeight=0.0)
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, includeAngular=True)
    s.setPositions(pos)                 # (N, 3) or (3N,), numpy or torch
    U, W = s.Mdot(forces, torques)      # M.[F;T]
    dU, dW = s.sqrtMdotW(prefactor=1)   # M^{1/2} dW by Lanczos

The numeric work runs in the in-tree native library liblmg_gb300.so (C ABI in
include/libmobility_gb300.h); importing NBody fails if it is not built.
"""
from .nbody import NBody, SelfMobility

__all__ = ["NBody", "SelfMobility"]
__version__ = "1.1"
