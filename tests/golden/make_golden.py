"""Writes the golden fixtures of this directory from libMobility's OWN code.

The reference's pair physics (solvers/NBody/extra/hydrodynamicKernels.cuh) and
its Lanczos solver (include/lanczos/LanczosAlgorithm.{h,cu}) are compiled for
this CPU by oracle/build.py from the reference checkout (no source is copied),
run on seeded inputs, and their outputs are stored here so that tests can use
them on machines without the reference checkout (the GPU machine):

  ref_mdot_cases.npz     M.[F;T] of the reference pair code, float and double
                         builds, for open / wall geometries, every block
                         combination, batches, overlaps, coincident particles
                         and particles closer to the wall than one radius.
  ref_lanczos_cases.npz  sqrt(M) z of the reference lanczos::Solver (float and
                         double builds) for given z on dense M of small
                         systems, three calls in a row per solver so that the
                         adaptive convergence-check schedule is exercised,
                         with the iteration index each call returned.

Run:  python tests/golden/make_golden.py   (needs the reference checkout)
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import build as ob  # noqa: E402
from oracle import oracle as orc  # noqa: E402


def positions(rng, N, wall, box=8.0):
    p = rng.uniform(0, box, (N, 3))
    if wall:
        p[:, 2] = rng.uniform(0.2, 6.0, N)
    if N >= 6:
        p[5] = p[4]                    # coincident particles
        p[3] = p[2] + [0.7, 0.3, 0.1]  # overlapping pair (r < 2a)
        if wall:
            p[1, 2] = 0.5              # below one radius: damped, clamped
    return p


def mdot_cases():
    rng = np.random.default_rng(20240601)
    cases = []
    k = 0
    for wall in (0, 1):
        for ang, hasF, hasT in ((0, 1, 0), (1, 1, 0), (1, 0, 1), (1, 1, 1)):
            for N, nper in ((1, 1), (7, 7), (40, 20), (64, 64)):
                a = float(rng.uniform(0.8, 1.3))
                eta = float(rng.uniform(0.5, 1.5))
                wh = float(rng.choice([0.0, 2.5])) if wall else 0.0
                p = positions(rng, N, wall)
                p_user = p.copy()
                p_user[:, 2] += wh
                F = rng.normal(size=(N, 3)) if hasF else None
                T = rng.normal(size=(N, 3)) if hasT else None
                out = {}
                for dt, tag in ((np.float64, "d"), (np.float32, "f")):
                    # the reference shifts in `real` before the kernel
                    pw = (p_user.astype(dt).copy())
                    if wall:
                        pw[:, 2] = pw[:, 2] - dt(wh)
                    U, W = orc.ref_pair_mdot(pw, F, T, a=a, viscosity=eta, wall=wall,
                                             include_angular=ang, nper_batch=nper, dtype=dt)
                    out[f"U_{tag}"] = U
                    out[f"W_{tag}"] = W if ang else np.zeros((N, 3), dt)
                cases.append(dict(
                    meta=dict(wall=wall, ang=ang, hasF=hasF, hasT=hasT, N=N, nper=nper, a=a,
                              eta=eta, wall_height=wh),
                    pos=p_user, F=F if hasF else np.zeros((N, 3)),
                    T=T if hasT else np.zeros((N, 3)), **out))
                k += 1
    arrays = {}
    metas = []
    for i, c in enumerate(cases):
        metas.append(c["meta"])
        for key in ("pos", "F", "T", "U_d", "W_d", "U_f", "W_f"):
            arrays[f"c{i}_{key}"] = c[key]
    arrays["meta"] = np.array(json.dumps(metas))
    np.savez_compressed(HERE / "ref_mdot_cases.npz", **arrays)
    return len(cases)


def lanczos_cases():
    rng = np.random.default_rng(777)
    systems = [
        dict(wall=0, ang=1, N=16, a=1.0, eta=1 / (6 * np.pi)),
        dict(wall=1, ang=1, N=16, a=1.0, eta=1 / (6 * np.pi)),
        dict(wall=0, ang=0, N=30, a=0.9, eta=0.8),
    ]
    arrays = {}
    metas = []
    for si, s in enumerate(systems):
        p = rng.uniform(0, 10, (s["N"], 3))
        if s["wall"]:
            p[:, 2] = rng.uniform(1.5, 6.0, s["N"])
        M = orc.dense(p, a=s["a"], viscosity=s["eta"], wall=s["wall"],
                      include_angular=s["ang"])
        n = M.shape[0]
        arrays[f"s{si}_pos"] = p
        runs = []
        for dt, tol in ((np.float64, 1e-6), (np.float64, 1e-10), (np.float32, 1e-4)):
            ref = orc.RefLanczos(dt)
            zs, ys, its = [], [], []
            for call in range(3):
                z = rng.normal(size=n)
                y, it, _ = ref.run(M, z, tol)
                zs.append(z)
                ys.append(y.astype(np.float64))
                its.append(it)
            tag = f"s{si}_{np.dtype(dt).name}_{tol:g}"
            arrays[tag + "_z"] = np.array(zs)
            arrays[tag + "_y"] = np.array(ys)
            arrays[tag + "_it"] = np.array(its)
            runs.append(dict(tag=tag, dtype=np.dtype(dt).name, tol=tol))
        metas.append(dict(s, runs=runs))
    arrays["meta"] = np.array(json.dumps(metas))
    np.savez_compressed(HERE / "ref_lanczos_cases.npz", **arrays)
    return len(systems)


if __name__ == "__main__":
    if not ob.reference_available():
        raise SystemExit("reference checkout not found: cannot regenerate golden fixtures")
    ob.build_all()
    print("mdot cases:", mdot_cases())
    print("lanczos systems:", lanczos_cases())
