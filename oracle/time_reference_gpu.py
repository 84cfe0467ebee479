"""Times libMobility's own NBody CUDA kernel next to libmobility_gb300 on the
same GPU (test infrastructure: it launches the reference cubin made by
oracle/build.py through oracle/ref_gpu_launcher.cpp).

For each workload it prints one JSON line with pair interactions per second of
the reference "fast" kernel (computeRPYBatchedFastGPU with the launch shape of
its launcher, NbodyRPY.cu:99-116) and of this library's Mdot, both on device
buffers, CUDA events around 20 back-to-back launches after 3 warm-ups, and the
FP32 FMA throughput of plain and packed (f32x2) FMA chains.

    python oracle/time_reference_gpu.py
"""
import ctypes
import json
import math
import sys
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from oracle import build as ob  # noqa: E402


def workloads():
    rng = np.random.default_rng(1234)
    N = 4096
    L = (N * 4 * math.pi / 3 / 0.05) ** (1 / 3)
    yield dict(name="open UF, N=4096, phi=0.05", wall=0, ang=0, torques=False,
               pos=rng.uniform(0, L, (N, 3)), flops=36)
    N = 16384
    yield dict(name="wall 6x6, N=16384", wall=1, ang=1, torques=True,
               pos=np.column_stack([rng.uniform(0, 128, N), rng.uniform(0, 128, N),
                                    rng.uniform(1.5, 20, N)]), flops=380)
    N = 65536
    L = (N * 4 * math.pi / 3 / 0.2) ** (1 / 3)
    yield dict(name="open UF, N=65536, phi=0.2", wall=0, ang=0, torques=False,
               pos=rng.uniform(0, L, (N, 3)), flops=36)


def time_launches(fn, reps=20, warm=3):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3 / reps


def main():
    ob.build_oracle()
    lib = ctypes.CDLL(str(HERE / "_build" / "libref_gpu_launcher.so"))
    lib.ref_gpu_last_error.restype = ctypes.c_char_p
    for dbl, tag in ((0, "f"), (1, "d")):
        rc = lib.ref_gpu_load(dbl, str(HERE / "_ref" / f"ref_nbody_{tag}.cubin").encode())
        if rc:
            raise SystemExit(lib.ref_gpu_last_error().decode())
    from libmobility_gb300 import NBody, _capi
    mylib = _capi.load()
    a, eta = 1.0, 1 / (6 * math.pi)
    t0, rt0, r0 = 1 / (6 * math.pi * eta * a), 1 / (8 * math.pi * eta * a * a), \
        1 / (8 * math.pi * eta * a ** 3)
    for w in workloads():
        N = w["pos"].shape[0]
        rng = np.random.default_rng(7)
        F = rng.normal(size=(N, 3))
        T = rng.normal(size=(N, 3)) if w["torques"] else None
        out = {"workload": w["name"], "pairs": N * N, "flops_per_pair": w["flops"]}
        for prec, dt in (("float", torch.float32), ("double", torch.float64)):
            if prec == "double" and N > 16384:
                continue
            dp = torch.tensor(w["pos"], dtype=dt, device="cuda")
            dF = torch.tensor(F, dtype=dt, device="cuda")
            dT = torch.tensor(T, dtype=dt, device="cuda") if T is not None else None
            U = torch.zeros((N, 3), dtype=dt, device="cuda")
            W = torch.zeros((N, 3), dtype=dt, device="cuda")
            st = torch.cuda.current_stream().cuda_stream

            def ref():
                rc = lib.ref_gpu_mdot(ctypes.c_int(prec == "double"), ctypes.c_int(w["wall"]),
                                      ctypes.c_void_p(dp.data_ptr()),
                                      ctypes.c_void_p(dF.data_ptr()),
                                      ctypes.c_void_p(dT.data_ptr() if dT is not None else None),
                                      ctypes.c_void_p(U.data_ptr()),
                                      ctypes.c_void_p(W.data_ptr()), ctypes.c_int(1),
                                      ctypes.c_int(N), ctypes.c_double(t0), ctypes.c_double(r0),
                                      ctypes.c_double(rt0), ctypes.c_double(a),
                                      ctypes.c_int(w["ang"]), ctypes.c_void_p(st))
                assert rc == 0

            t_ref = time_launches(ref)
            s = NBody("open", "open", "single_wall" if w["wall"] else "open", precision=prec)
            s.setParameters(**({"wallHeight": 0.0} if w["wall"] else {}))
            s.initialize(viscosity=eta, hydrodynamicRadius=a, includeAngular=bool(w["ang"]))
            s.setPositions(dp)
            t_me = time_launches(lambda: s.Mdot(dF, dT))
            out[prec] = {"reference_pairs_per_s": N * N / t_ref,
                         "gb300_pairs_per_s": N * N / t_me,
                         "speedup": t_ref / t_me,
                         "reference_ms": t_ref * 1e3, "gb300_ms": t_me * 1e3}
        print(json.dumps(out), flush=True)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    sink = torch.zeros(256, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    for name, fn in (("ffma", mylib.lmg_internal_fma_probe),
                     ("ffma2", mylib.lmg_internal_fma2_probe)):
        blocks, threads, iters = sms * 8, 256, 4096
        t = time_launches(lambda: fn(blocks, threads, iters, sink.data_ptr(), st), reps=5)
        print(json.dumps({"probe": name, "tflops": blocks * threads * iters * 128 / t / 1e12}))


if __name__ == "__main__":
    main()
