"""The bounds-checked build (liblmg_gb300_checked.so, -DLMG_BOUNDS_CHECK).

In it every index of the all-pairs kernels (tiled and symmetric) is checked
before its global access; a failed check records (code << 48) | index in a
device status word and skips the access, so an indexing fault would show up as
a status instead of a GPU fault.  This test builds that variant, runs in a
subprocess (which loads it instead of the normal library) the shapes that
stress the index arithmetic -- single particles, ragged tiles, batches, source
splits, the symmetric kernel cut over many warps, FP32 and FP64, open and wall,
Mdot and sqrtMdotW -- checks every result against the FP64 oracle and requires
every status word to be clear; a probe kernel whose check fails on purpose
(it accesses nothing) shows that a failure is recorded.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent

SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from libmobility_gb300 import NBody, _capi
from oracle import oracle as orc
lib = _capi.load()
assert "checked" in str(_capi.LIB_PATH)
for w in range(3):
    lib.lmg_internal_bounds_status(w, 1)
worst = 0.0
rng = np.random.default_rng(8)
for prec in ("float", "double"):
    for wall in (0, 1):
        for ang in (0, 1):
            for N, nper in ((1, 1), (3, 3), (129, 129), (300, 100), (1000, 250), (2048, 2048)):
                p = rng.uniform(0, (N * 4 * np.pi / 3 / 0.1) ** (1 / 3), (N, 3))
                if wall:
                    p[:, 2] = rng.uniform(0.5, 10, N)
                F = rng.normal(size=(N, 3))
                T = rng.normal(size=(N, 3)) if ang else None
                s = NBody("open", "open", "single_wall" if wall else "open", precision=prec)
                nb = N // nper
                if wall:
                    s.setParameters("advise", nb, nper, wallHeight=0.0)
                else:
                    s.setParameters("advise", nb, nper)
                s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, includeAngular=bool(ang),
                             tolerance=1e-6)
                s.setPositions(p)
                U, W = s.Mdot(F, T)
                Uo, Wo = orc.mdot(p, F, T, a=1.0, viscosity=1.0, wall=wall, include_angular=ang,
                                  nper_batch=nper)
                worst = max(worst, float(np.abs(U - Uo).max() / max(np.abs(Uo).max(), 1e-300)))
                if N >= 129 and nper == N:
                    s.sqrtMdotW_noise(rng.normal(size=(6 if ang else 3) * N))
for warps in (1, 7, 200):
    lib.lmg_internal_sym_override(0, warps)
    p = rng.uniform(0, 30, (1537, 3))
    F = rng.normal(size=(1537, 3))
    s = NBody("open", "open", "open", precision="float")
    s.setParameters()
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
    s.setPositions(p)
    U, _ = s.Mdot(F)
    Uo, _ = orc.mdot(p, F, None, a=1.0, viscosity=1.0, wall=0, include_angular=0)
    worst = max(worst, float(np.abs(U - Uo).max() / np.abs(Uo).max()))
lib.lmg_internal_sym_override(0, 0)
status = [int(lib.lmg_internal_bounds_status(w, 0)) for w in range(3)]
assert lib.lmg_internal_bounds_probe() == 0
probe = int(lib.lmg_internal_bounds_status(3, 1))
print(json.dumps({"worst": worst, "status": status, "probe": probe}))
"""


def test_checked_build_runs_clean(cuda, oracle):
    from libmobility_gb300 import _build
    lib = _build.build(checked=True)
    env = dict(os.environ, LIBMOBILITY_GB300_LIB=str(lib))
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT)], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["status"] == [0, 0, 0], out
    assert out["probe"] >> 48 == 99 and (out["probe"] & 0xffffffffffff) >= 1000, out
    assert out["worst"] <= 1e-5, out
