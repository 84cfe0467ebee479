#!/usr/bin/env python
"""Benchmark of the NBody hot path on GB300.

Workload (default): single-wall Rotne-Prager-Blake mobility, N = 16384,
a = 1, viscosity 1/(6 pi), x, y ~ U[0, 128), z ~ U[1.5, 20], forces, torques
and dW ~ N(0, 1) (seeded), FP32 pair kernel with FP64 Krylov scalars.  One
step = one Mdot M.[F;T] plus one sqrtMdotW (plain Lanczos to the reference
criterion |y_i - y_{i-1}|/|y_{i-1}| <= 1e-6) with the step's dW.

value = pair interactions evaluated per second over whole steps (Mdot and
every Lanczos matvec; the Lanczos vector work, eigen-solves and checks are in
the time but earn nothing); the unit is pair-interactions/s.  Inputs are
resident in HBM; the 129 MB L2 is flushed between timed steps (inputs are
smaller than L2).  e2e is the same metric through the public API with host
(numpy) buffers, host<->device copies included.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload wall16k|open4k]

With --gpus N > 1 (under torchrun) every rank runs its own replica of the
workload on its own GPU; there is no collective on the data path.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("sqrtMdotW solves/s at 1e-6 residual (learned-precond vs plain); "
          "Mdot pair-interactions/s")
# algorithmic flops per pair interaction (FMA = 2, add/mul = 1,
# rsqrt/rcp/div/sqrt = 1): open UF 36, open 6x6 89, wall UF 160, wall 6x6 380
FLOPS_PER_PAIR = {("open", False): 36, ("open", True): 89, ("wall", False): 160,
                  ("wall", True): 380}
WORKLOADS = {
    "wall16k": dict(N=16384, wall=True, ang=True, tol=1e-6,
                    desc="single-wall RPY, N=16384, forces+torques, includeAngular, "
                         "Mdot + Lanczos sqrtMdotW to 1e-6"),
    "open4k": dict(N=4096, wall=False, ang=False, tol=1e-6,
                   desc="open-boundary RPY, N=4096, forces only, phi=0.05, "
                        "Mdot + Lanczos sqrtMdotW to 1e-6"),
    "open16k": dict(N=16384, wall=False, ang=False, tol=1e-6,
                    desc="open-boundary RPY, N=16384, forces only, phi=0.05, "
                         "Mdot + Lanczos sqrtMdotW to 1e-6"),
}

# dram__bytes_read.sum + dram__bytes_write.sum per launch of the Mdot kernel
# from one ncu capture of each workload (profiles/mdot_kernel_*.md); the
# kernel reads its inputs once (positions, forces, torques) and writes the
# split partials, which stay in L2
MDOT_TRAFFIC = {"wall16k": 633.3e3, "open16k": 417.8e3}


def make_inputs(w, seed):
    rng = np.random.default_rng(seed)
    N = w["N"]
    if w["wall"]:
        pos = np.column_stack([rng.uniform(0, 128, N), rng.uniform(0, 128, N),
                               rng.uniform(1.5, 20, N)])
    else:
        L = (N * 4 * math.pi / 3 / 0.05) ** (1 / 3)
        pos = rng.uniform(0, L, (N, 3))
    F = rng.normal(size=(N, 3))
    T = rng.normal(size=(N, 3)) if w["ang"] else None
    dW = rng.normal(size=(6 if w["ang"] else 3) * N)
    return pos, F, T, dW


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, seconds, ws):
    """Whole-job rate of a replicated run: every rank processed
    `units_per_rank` in its own time; the job rate is all ranks' units over
    the slowest rank's time (max over ranks)."""
    return units_per_rank * ws / max_over_ranks(seconds, ws)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        load = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2(buf):
    buf.zero_()  # 256 MB write, larger than the 129 MB L2


def fp32_peak_tflops(lib, torch):
    """FP32 FMA throughput of this GPU, measured now (8 independent chains per
    thread, enough CTAs to fill every SM)."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4096
    sink = torch.zeros(threads, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        lib.lmg_internal_fma_probe(blocks, threads, iters, sink.data_ptr(), st)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lib.lmg_internal_fma_probe(blocks, threads, iters, sink.data_ptr(), st)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        best = max(best, blocks * threads * iters * 64 * 2 / t / 1e12)
    return best


def fp64_peak_tflops(lib, torch):
    """FP64 FMA throughput of this GPU, measured now (same structure as the
    FP32 probe; GB300's FP64 units are narrow, so fewer rounds)."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 128
    sink = torch.zeros(threads, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    lib.lmg_internal_dfma_probe(blocks, threads, iters, sink.data_ptr(), st)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lib.lmg_internal_dfma_probe(blocks, threads, iters, sink.data_ptr(), st)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        best = max(best, blocks * threads * iters * 64 * 2 / t / 1e12)
    return best


def graph_time(torch, fn, reps=20):
    """Average device time of `fn` (one kernel launch, or a few) captured
    `reps` times in a CUDA graph and replayed between CUDA events, so the host
    cost of the Python call does not starve the GPU at small sizes; without
    graph capture, back-to-back calls are timed."""
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    try:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="relaxed"):
            for _ in range(reps):
                fn()
        g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / reps, "cuda-graph replay of %d launches" % reps
    except Exception as exc:  # pragma: no cover - depends on the driver
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / reps, f"back-to-back calls ({exc.__class__.__name__})"


def flushed_time(torch, fn, flush, reps=20):
    """Median device time of one call of `fn` right after the L2 is flushed
    (its inputs then come from HBM), CUDA events around the call."""
    ts = []
    for _ in range(reps):
        flush_l2(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    return statistics.median(ts)


def open4k_inputs(seed=1234):
    """N = 4096 uniform in the cube of volume fraction 0.05 (a = 1), forces
    N(0, 1)."""
    rng = np.random.default_rng(seed)
    N = 4096
    L = (N * 4 * math.pi / 3 / 0.05) ** (1 / 3)
    return rng.uniform(0, L, (N, 3)), rng.normal(size=(N, 3))


def open4k_mdot(torch, lib, peak32, peak64, flush):
    """Open-boundary translational Mdot, N = 4096, a = 1,
    viscosity 1/(6 pi), in FP32 and FP64 on device-resident inputs.  The FP32
    handle takes the symmetric kernel; the tiled kernel's time on the same
    handle is given beside it.  Returns the sub-object and the results (for
    the error against the FP64 oracle, filled in by the caller)."""
    from libmobility_gb300 import NBody
    pos, F = open4k_inputs()
    N = pos.shape[0]
    pairs = float(N) * N
    out = {"workload": "open RPY (UF), N=4096, cube at phi=0.05, a=1, viscosity 1/(6 pi), "
                       "F ~ N(0,1), seed 1234",
           "pairs": pairs, "flops_per_pair": FLOPS_PER_PAIR[("open", False)]}
    results = {}
    for prec, dt, peak in (("float", torch.float32, peak32), ("double", torch.float64, peak64)):
        s = NBody("open", "open", "open", precision=prec)
        s.setParameters()
        s.initialize(viscosity=1 / (6 * math.pi), hydrodynamicRadius=1.0)
        dpos = torch.tensor(pos, dtype=dt, device="cuda")
        dF = torch.tensor(F, dtype=dt, device="cuda")
        s.setPositions(dpos)
        t, how = graph_time(torch, lambda: s.Mdot(dF, None), reps=50)
        t_cold = flushed_time(torch, lambda: s.Mdot(dF, None), flush)
        U, _ = s.Mdot(dF, None)
        torch.cuda.synchronize()
        results[prec] = U.double().cpu().numpy()
        ach = pairs * out["flops_per_pair"] / t / 1e12
        e = {"ms": t * 1e3, "pair_interactions_per_s": pairs / t, "achieved_tflops": ach,
             "peak_tflops": peak, "frac": ach / peak,
             "peak_source": ("FP32" if prec == "float" else "FP64") + " FMA-chain probe "
                            "measured in this run",
             "kernel_timing": how + " (inputs in L2)",
             "ms_after_l2_flush": t_cold * 1e3}
        if prec == "float":
            e["kernel"] = "mdot_sym_kernel (symmetric, each unordered pair once)"
            assert lib.lmg_internal_sym_override(1, 0) == 0
            try:
                t_tiled, _ = graph_time(torch, lambda: s.Mdot(dF, None), reps=50)
            finally:
                lib.lmg_internal_sym_override(0, 0)
            e["tiled_kernel_ms"] = t_tiled * 1e3
            e["speedup_vs_tiled_kernel"] = t_tiled / t
        else:
            e["kernel"] = "mdot_kernel<double>"
        out[prec] = e
    return out, pos, F, results


def open4k_sqrt(torch, lib, solves=20):
    """Square root of the open N = 4096 system: open boundary, FP32,
    tolerance 1e-6, sqrtMdotW solves per second (host wall clock around each
    call, device-resident dW) with T^{1/2} e1 of the convergence checks by
    quadrature on the host (the default), by the exact QL on the host and by
    quadrature on the device, on fresh handles after 3 warm-up solves each."""
    from libmobility_gb300 import NBody
    pos, _ = open4k_inputs()
    N = pos.shape[0]
    dpos = torch.tensor(pos, dtype=torch.float32, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(17)
    dWs = [torch.randn(3 * N, generator=g, device="cuda") for _ in range(solves + 3)]
    out = {"workload": "open RPY, N=4096, cube at phi=0.05, FP32, tolerance 1e-6"}
    try:
        for name, mode in (("host_quadrature", 2), ("host_ql", 0), ("device_quadrature", 1)):
            assert lib.lmg_internal_lanczos_device_sqrt(mode) == 0
            s = NBody("open", "open", "open", precision="float")
            s.setParameters()
            s.initialize(viscosity=1 / (6 * math.pi), hydrodynamicRadius=1.0, tolerance=1e-6,
                         seed=9)
            s.setPositions(dpos)
            its, ts = [], []
            for k, dW in enumerate(dWs):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                _, _, it, _ = s.sqrtMdotW_noise(dW)
                torch.cuda.synchronize()
                if k >= 3:
                    ts.append(time.perf_counter() - t0)
                    its.append(it)
            t = sum(ts) / len(ts)
            out[name] = {"solves_per_s": 1.0 / t, "ms_per_solve": t * 1e3,
                         "lanczos_iterations": sum(its) / len(its)}
    finally:
        lib.lmg_internal_lanczos_device_sqrt(2)
    out["default"] = "host_quadrature"
    out["speedup_host_quadrature_vs_host_ql"] = (out["host_quadrature"]["solves_per_s"]
                                                 / out["host_ql"]["solves_per_s"])
    return out


def reference_gpu_mdot(torch, wall16k_inputs):
    """libMobility's own NBody CUDA kernel (computeRPYBatchedFastGPU, launch
    shape of its launcher, NbodyRPY.cu:99-116), compiled for sm_103a from the
    reference sources into oracle/_ref, next to this library's Mdot on the
    same GPU and inputs: open UF, N = 4096, and single wall, all blocks,
    N = 16384, FP32 and FP64, both timed as CUDA
    graph replays of 20 launches on device buffers."""
    import ctypes
    from oracle import build as ob
    from libmobility_gb300 import NBody
    ob.build_oracle()
    here = ROOT / "oracle"
    cubins = [here / "_ref" / f"ref_nbody_{t}.cubin" for t in ("f", "d")]
    if not all(c.exists() for c in cubins):
        return {"unavailable": "reference cubin not built (oracle/_ref is made where the "
                               "reference sources are)"}
    rl = ctypes.CDLL(str(here / "_build" / "libref_gpu_launcher.so"))
    rl.ref_gpu_last_error.restype = ctypes.c_char_p
    for dbl, c in enumerate(cubins):
        if rl.ref_gpu_load(dbl, str(c).encode()):
            return {"unavailable": rl.ref_gpu_last_error().decode()}
    a, eta = 1.0, 1 / (6 * math.pi)
    t0, r0, rt0 = 1 / (6 * math.pi * eta * a), 1 / (8 * math.pi * eta * a ** 3), \
        1 / (8 * math.pi * eta * a * a)
    pos1, F1 = open4k_inputs()
    pos2, F2, T2, _ = wall16k_inputs
    out = {"kernel": "computeRPYBatchedFastGPU (libMobility NbodyRPY.cu:26-97), sm_103a cubin"}
    for name, wall, ang, pos, F, T, fpp in (
            ("open4k_uf", 0, 0, pos1, F1, None, FLOPS_PER_PAIR[("open", False)]),
            ("wall16k_6x6", 1, 1, pos2, F2, T2, FLOPS_PER_PAIR[("wall", True)])):
        N = pos.shape[0]
        ent = {}
        for prec, dt in (("float", torch.float32), ("double", torch.float64)):
            dp = torch.tensor(pos, dtype=dt, device="cuda")
            dF = torch.tensor(F, dtype=dt, device="cuda")
            dT = torch.tensor(T, dtype=dt, device="cuda") if T is not None else None
            U = torch.zeros((N, 3), dtype=dt, device="cuda")
            W = torch.zeros((N, 3), dtype=dt, device="cuda")

            def ref():
                st = torch.cuda.current_stream().cuda_stream
                rc = rl.ref_gpu_mdot(ctypes.c_int(prec == "double"), ctypes.c_int(wall),
                                     ctypes.c_void_p(dp.data_ptr()),
                                     ctypes.c_void_p(dF.data_ptr()),
                                     ctypes.c_void_p(dT.data_ptr() if dT is not None else None),
                                     ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(W.data_ptr()),
                                     ctypes.c_int(1), ctypes.c_int(N), ctypes.c_double(t0),
                                     ctypes.c_double(r0), ctypes.c_double(rt0), ctypes.c_double(a),
                                     ctypes.c_int(ang), ctypes.c_void_p(st))
                if rc:
                    raise RuntimeError(rl.ref_gpu_last_error().decode())

            t_ref, _ = graph_time(torch, ref)
            s = NBody("open", "open", "single_wall" if wall else "open", precision=prec)
            s.setParameters(**({"wallHeight": 0.0} if wall else {}))
            s.initialize(viscosity=eta, hydrodynamicRadius=a, includeAngular=bool(ang))
            s.setPositions(dp)
            t_me, _ = graph_time(torch, lambda: s.Mdot(dF, dT))
            pairs = float(N) * N
            ent[prec] = {"reference_ms": t_ref * 1e3, "ours_ms": t_me * 1e3,
                         "reference_pair_interactions_per_s": pairs / t_ref,
                         "ours_pair_interactions_per_s": pairs / t_me,
                         "reference_tflops": pairs * fpp / t_ref / 1e12,
                         "speedup": t_ref / t_me}
        out[name] = ent
    out["timing"] = "cuda-graph replay of 20 launches each, device buffers, inputs in L2"
    return out


def mdot_kernel_time(torch, s, dF, dT, reps=20):
    """Average time of one Mdot launch on the device.  The launches are
    captured in a CUDA graph and replayed between CUDA events on the same
    stream, so the host-side cost of the Python call does not starve the GPU
    at small N; if capture is not possible, back-to-back calls are timed."""
    for _ in range(3):
        s.Mdot(dF, dT)
    torch.cuda.synchronize()
    try:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="relaxed"):
            for _ in range(reps):
                s.Mdot(dF, dT)
        g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / reps, "cuda-graph replay of %d Mdot launches" % reps
    except Exception as exc:  # pragma: no cover - depends on the driver
        torch.cuda.synchronize()
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            s.Mdot(dF, dT)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / reps, f"back-to-back calls ({exc.__class__.__name__})"


def sqrtmdotw_comparison(torch, steps, warmup, rank, N=65536):
    """Plain vs learned-preconditioned sqrtMdotW on the clustered workload:
    N = 65536 particles in 512 Gaussian clusters (sigma = 4a, hard-sphere
    rejection at 2a), volume fraction 0.2, open boundary, tolerance 1e-6.
    Positions are set again before every solve, so the preconditioner (kNN +
    network) is rebuilt each time, as in a time-stepping run."""
    from libmobility_gb300 import NBody
    from libmobility_gb300.precond import random_system
    rng = np.random.default_rng(2025 + rank)
    t0 = time.perf_counter()
    pos = random_system(rng, N, 0.2, True)
    gen_s = time.perf_counter() - t0
    dpos = torch.tensor(pos, dtype=torch.float32, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(77 + rank)
    dWs = [torch.randn(3 * N, generator=g, device="cuda") for _ in range(steps + warmup)]
    out = {"workload": "open RPY, N=65536, 512 Gaussian clusters sigma=4a, hard-sphere "
                       "rejection at 2a, phi=0.2, tolerance 1e-6",
           "generation_s": gen_s}
    for kind in ("none", "mlp"):
        s = NBody("open", "open", "open", precision="float")
        s.setParameters()
        s.initialize(viscosity=1 / (6 * math.pi), hydrodynamicRadius=1.0, tolerance=1e-6,
                     seed=3 + rank)
        s.setPreconditioner(kind)
        its, inner, times = [], [], []
        for k, dW in enumerate(dWs):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.setPositions(dpos)
            _, _, it, _ = s.sqrtMdotW_noise(dW)
            torch.cuda.synchronize()
            if k >= warmup:
                times.append(time.perf_counter() - t0)
                its.append(it)
                inner.append(s.lastPreconditionerSolveIterations() if kind == "mlp" else 0)
        t = sum(times) / len(times)
        out[kind] = {"solves_per_s": 1.0 / t, "ms_per_solve": t * 1e3,
                     "lanczos_iterations": sum(its) / len(its),
                     "iterations_min_max": [min(its), max(its)], "solves": len(its)}
        if kind == "mlp":
            out[kind]["p_solve_iterations"] = sum(inner) / len(inner)
        # where the time goes: device spans of two more solves, outside the
        # timed ones (the events add a synchronisation at the end of a solve)
        s._lanczos_phase_timing(True)
        for dW in dWs[warmup:warmup + 2]:
            s.setPositions(dpos)
            s.sqrtMdotW_noise(dW)
        torch.cuda.synchronize()
        ph = s._lanczos_phase_times()
        s._lanczos_phase_timing(False)
        nit = ph["iterations"]
        out[kind]["per_iteration_us"] = {
            "operator": 1e3 * ph["operator_ms"] / nit, "vector_update": 1e3 * ph["vector_ms"] / nit}
        out[kind]["per_solve_ms"] = {"preconditioner_build": ph["build_ms"] / ph["solves"],
                                     "p_solve": ph["psolve_ms"] / ph["solves"]}
    out["speedup_learned_vs_plain"] = out["mlp"]["solves_per_s"] / out["none"]["solves_per_s"]
    return out


def precond_network_gemms(torch, lib, M=65536):
    """The preconditioner network's three layers (the shipped open network:
    48 neighbours, 512-512 hidden units, 438 outputs) as GEMMs over M = 65536
    particles, on the tensor cores (tcgen05 kind::tf32, TMA-fed, accumulator
    in tensor memory) and on the CUDA cores (FP32, the build's default),
    CUDA-event timed on device buffers; then the whole build both ways.  The
    tensor-core figures are against the bf16 cuBLAS peak halved (TF32 runs at
    half the bf16 rate)."""
    from libmobility_gb300 import precond as pc
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def ev(fn, reps=10):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps * 1e-3

    st = lambda: ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)  # noqa: E731
    peak = None
    try:
        with open(Path(__file__).resolve().parent / "MEASURED_PEAKS.json") as f:
            peak = json.load(f)["bf16_tflops"] / 2
    except Exception:
        pass
    out = {"M": M, "tf32_peak_tflops": peak,
           "peak_source": "MEASURED_PEAKS.json bf16_tflops / 2 (TF32 rate)"}
    g = torch.Generator(device="cuda").manual_seed(5)
    layers = []
    for (N, K) in ((512, 144), (512, 512), (438, 512)):
        A = torch.randn(M, K, generator=g, device="cuda")
        Bt = torch.randn(N, K, generator=g, device="cuda") / math.sqrt(K)
        B = Bt.t().contiguous()
        bias = torch.randn(N, generator=g, device="cuda")
        C1 = torch.empty(M, N, device="cuda")
        C2 = torch.empty(M, N, device="cuda")
        t_tc = ev(lambda: lib.lmg_internal_tc_gemm(M, N, K, p(A), K, p(Bt), K, p(C1), N, p(bias),
                                                   1, st()))
        t_cc = ev(lambda: lib.lmg_internal_gemm(0, 0, M, N, K, p(A), K, p(B), N, p(C2), N,
                                                p(bias), 1, ctypes.c_float(0.0), st()))
        fl = 2.0 * M * N * K
        ach = fl / t_tc / 1e12
        layers.append({"N": N, "K": K, "tensor_core_us": t_tc * 1e6, "cuda_core_us": t_cc * 1e6,
                       "tensor_core_tflops": ach, "cuda_core_tflops": fl / t_cc / 1e12,
                       "frac_of_tf32_peak": ach / peak if peak else None,
                       "max_abs_diff": float((C1 - C2).abs().max())})
    out["layers"] = layers
    out["tc_status"] = lib.lmg_internal_tc_status(1)
    params = pc.load_weights(pc.default_weights(False))
    k, h = pc.shape_of_params(len(params))
    rng = np.random.default_rng(3)
    L = (M * 4 * math.pi / 3 / 0.2) ** (1 / 3)
    pos = torch.tensor(rng.uniform(0, L, (M, 3)), dtype=torch.float32, device="cuda")
    dparams = torch.tensor(params, device="cuda")
    nb = torch.empty((k + 1, M), dtype=torch.int32, device="cuda")
    lib.lmg_internal_knn_k(k, p(pos), M, M, p(nb), None)
    blk = torch.empty((k + 1, 9, M), device="cuda")
    try:
        for name, tc in (("build_cuda_core_ms", 0), ("build_tensor_core_ms", 1)):
            assert lib.lmg_internal_precond_tc(tc) == 0
            out[name] = 1e3 * ev(lambda: lib.lmg_internal_precond_build_kh(
                k, h, p(pos), p(nb), M, p(dparams), 1.0, 1.0, p(blk), st()), reps=5)
    finally:
        lib.lmg_internal_precond_tc(0)
    out["default"] = "cuda_core (the TF32 network adds about 3 Lanczos iterations per solve)"
    return out


def ensemble_systems(rng, nsys=256):
    """256 systems, N ~ U[200, 4000], half open and half single wall,
    volume fraction ~ U[0.02, 0.25] each (a = 1): open systems uniform in a
    cube, wall systems with x, y uniform in a square and z ~ U[1.5, 20]
    (the slab holds the volume fraction)."""
    sizes = rng.integers(200, 4001, nsys)
    geoms = np.arange(nsys) % 2
    rng.shuffle(geoms)
    phis = rng.uniform(0.02, 0.25, nsys)
    pos = []
    for n, g, phi in zip(sizes, geoms, phis):
        vol = n * 4 * math.pi / 3 / phi
        if g:
            L = math.sqrt(vol / 18.5)
            pos.append(np.column_stack([rng.uniform(0, L, n), rng.uniform(0, L, n),
                                        rng.uniform(1.5, 20, n)]))
        else:
            pos.append(rng.uniform(0, vol ** (1 / 3), (n, 3)))
    return sizes, geoms, np.concatenate(pos)


def ensemble_comparison(torch, steps, warmup, rank, nsys=256, sequential=True, peak=None):
    """Batched ensemble of 256 uneven systems (open and wall mixed) in one
    handle, FP32, tolerance 1e-6: Mdot and sqrtMdotW for all systems per call,
    against one NBody solver per system run one after the other."""
    from libmobility_gb300 import NBody
    from libmobility_gb300.ensemble import Ensemble
    rng = np.random.default_rng(4242 + rank)
    sizes, geoms, pos = ensemble_systems(rng, nsys)
    ntot = int(sizes.sum())
    eta = 1 / (6 * math.pi)
    f32 = dict(dtype=torch.float32, device="cuda")
    dpos = torch.tensor(pos, **f32)
    g = torch.Generator(device="cuda").manual_seed(99 + rank)
    dF = torch.randn(ntot, 3, generator=g, **f32)
    dWs = [torch.randn(ntot, 3, generator=g, **f32) for _ in range(steps + warmup)]
    e = Ensemble(precision="float")
    e.setSystems(sizes, geoms, np.zeros(len(sizes)))
    t0 = time.perf_counter()
    e.initialize(viscosity=eta, hydrodynamicRadius=1.0, tolerance=1e-6, seed=5 + rank)
    e.setPositions(dpos)
    e.Mdot(dF)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    pairs = float(np.sum(sizes.astype(np.float64) ** 2))
    for _ in range(3):
        e.Mdot(dF)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    reps = 10
    for _ in range(reps):
        e.Mdot(dF)
    e1.record()
    e1.synchronize()
    t_mdot = e0.elapsed_time(e1) * 1e-3 / reps
    # credited flops of one product of all systems: open UF 36, wall UF 160 per pair
    flops = float(sum(float(n) ** 2 * FLOPS_PER_PAIR[("wall" if gm else "open", False)]
                      for n, gm in zip(sizes, geoms)))
    times, lat, its_all = [], [], []
    for k, dW in enumerate(dWs):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, its, _, ms = e.sqrtMdotW(dW)
        torch.cuda.synchronize()
        if k >= warmup:
            times.append(time.perf_counter() - t0)
            lat.extend(ms.tolist())
            its_all.append(its)
    t_sqrt = sum(times) / len(times)
    its_m = np.mean(its_all, axis=0)
    sqrt_pairs = float(np.sum(sizes.astype(np.float64) ** 2 * (its_m + 1)))
    # the same systems and noise, one NBody solver per system, one after another
    seq = []
    off = 0
    dW0 = dWs[warmup]
    for n, gm in zip(sizes, geoms) if sequential else ():
        s = NBody("open", "open", "single_wall" if gm else "open", precision="float")
        s.setParameters(**({"wallHeight": 0.0} if gm else {}))
        s.initialize(viscosity=eta, hydrodynamicRadius=1.0, tolerance=1e-6, seed=5)
        s.setPositions(dpos[off:off + n])
        s.sqrtMdotW_noise(dW0[off:off + n])  # first call allocates
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.sqrtMdotW_noise(dW0[off:off + n])
        torch.cuda.synchronize()
        seq.append(time.perf_counter() - t0)
        off += n
    t_seq = sum(seq) if seq else None
    return {
        "workload": "%d systems, N ~ U[200, 4000] (total %d), half open / half single wall "
                    "(z ~ U[1.5, 20]), phi ~ U[0.02, 0.25], FP32, tolerance 1e-6" % (nsys, ntot),
        "groups": len(e.describe()["groups"]),
        "setup_and_autotune_s": setup_s,
        "mdot_ms": t_mdot * 1e3,
        "mdot_pair_interactions_per_s": pairs / t_mdot,
        "mdot_achieved_tflops": flops / t_mdot / 1e12,
        "mdot_frac_of_fp32_peak": flops / t_mdot / 1e12 / peak if peak else None,
        "flops_note": "open UF 36 and wall UF 160 credited flops per pair; padding dummies "
                      "earn nothing",
        "sqrtMdotW_ms_per_call": t_sqrt * 1e3,
        "system_solves_per_s": len(sizes) / t_sqrt,
        "sqrtMdotW_pair_interactions_per_s": sqrt_pairs / t_sqrt,
        "lanczos_iterations": {"min": float(np.min(its_all)), "median": float(np.median(its_all)),
                               "max": float(np.max(its_all))},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "what": "host time from the start of the batched call until each "
                               "system's result was known"},
        "sequential_single_solvers_ms": t_seq * 1e3 if t_seq else None,
        "speedup_batched_vs_sequential": t_seq / t_sqrt if t_seq else None,
    }


def large_wall_mdot(torch, rank, reps=3):
    """Matrix-vector product of the large wall system: single wall, N = 262144,
    x, y ~ U[0, 1024), z ~ U[1.5, 40], forces and torques, includeAngular,
    FP32; CUDA events around `reps` launches on device-resident inputs (its
    FP64 check on 4096 rows is tests/test_large_gpu.py)."""
    from libmobility_gb300 import NBody
    N = 262144
    rng = np.random.default_rng(31 + rank)
    pos = np.column_stack([rng.uniform(0, 1024, N), rng.uniform(0, 1024, N),
                           rng.uniform(1.5, 40, N)])
    f32 = dict(dtype=torch.float32, device="cuda")
    dpos = torch.tensor(pos, **f32)
    dF = torch.tensor(rng.normal(size=(N, 3)), **f32)
    dT = torch.tensor(rng.normal(size=(N, 3)), **f32)
    s = NBody("open", "open", "single_wall", precision="float")
    s.setParameters(wallHeight=0.0)
    s.initialize(viscosity=1 / (6 * math.pi), hydrodynamicRadius=1.0, includeAngular=True)
    s.setPositions(dpos)
    s.Mdot(dF, dT)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        s.Mdot(dF, dT)
    e1.record()
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3 / reps
    pairs = float(N) * N
    return {"workload": "single wall, N=262144, x,y ~ U[0,1024), z ~ U[1.5,40], forces + "
                        "torques, includeAngular, FP32",
            "mdot_ms": t * 1e3, "mdot_pair_interactions_per_s": pairs / t,
            "achieved_tflops": pairs * FLOPS_PER_PAIR[("wall", True)] / t / 1e12}


def large_wall_sqrt(torch, rank):
    """Square root of the large wall system: single wall, N = 262144, x, y ~ U[0,
    1024), z ~ U[1.5, 40], includeAngular, FP32, tolerance 1e-6: one
    sqrtMdotW of plain Lanczos and one with the learned wall preconditioner
    (rebuilt for the solve), same dW, wall time and iterations."""
    from libmobility_gb300 import NBody
    N = 262144
    rng = np.random.default_rng(31 + rank)
    pos = np.column_stack([rng.uniform(0, 1024, N), rng.uniform(0, 1024, N),
                           rng.uniform(1.5, 40, N)])
    dpos = torch.tensor(pos, dtype=torch.float32, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(13 + rank)
    dW = torch.randn(6 * N, generator=g, device="cuda")
    out = {"workload": "single wall, N=262144, x,y ~ U[0,1024), z ~ U[1.5,40], includeAngular, "
                       "FP32, tolerance 1e-6, one solve per arm (same dW)"}
    for kind in ("none", "mlp"):
        s = NBody("open", "open", "single_wall", precision="float")
        s.setParameters(wallHeight=0.0)
        s.initialize(viscosity=1 / (6 * math.pi), hydrodynamicRadius=1.0, includeAngular=True,
                     tolerance=1e-6, seed=3 + rank)
        s.setPreconditioner(kind)
        s.setPositions(dpos)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.setPositions(dpos)
        _, _, it, res = s.sqrtMdotW_noise(dW)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        out[kind] = {"ms_per_solve": t * 1e3, "lanczos_iterations": it, "residual": res}
        if kind == "mlp":
            out[kind]["network"] = "wall, 48 neighbours, 512-512 hidden"
            out[kind]["p_solve_iterations"] = s.lastPreconditionerSolveIterations()
    out["speedup_learned_vs_plain"] = out["none"]["ms_per_solve"] / out["mlp"]["ms_per_solve"]
    return out


def hbm_peak_gbs():
    """The measured copy bandwidth (GB/s), None when the file is absent."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)),
                               "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def krylov_phases(torch, s, ddW, t_mdot, solves=3):
    """Device time of the Lanczos work outside the matvec on the main
    workload: the vector updates after each matvec (alpha, beta, next basis
    vector: 4 n s algorithmic bytes per iteration) and the convergence checks
    (y = |z| V c over m basis vectors, (m + 1) n s, plus 2 n s for the error
    norm), against the measured HBM copy bandwidth.  The vectors are n = 6N
    FP32 (393 KB at N = 16384): they live in L2 and each update is a few
    launches of a grid reduction, so these phases are latency-bound."""
    torch.cuda.synchronize()
    s._lanczos_phase_timing(True)
    for _ in range(solves):
        s.sqrtMdotW_noise(ddW)
    torch.cuda.synchronize()
    t = s._lanczos_phase_times()
    s._lanczos_phase_timing(False)
    its = t["iterations"] / t["solves"]
    peak = hbm_peak_gbs()
    vec_gbs = t["vector_bytes"] / (t["vector_ms"] * 1e-3) / 1e9
    chk_gbs = t["check_bytes"] / (t["check_ms"] * 1e-3) / 1e9
    return {
        "solves": int(t["solves"]),
        "iterations_issued_per_solve": its,
        "checks_per_solve": t["checks"] / t["solves"],
        "vector_update_us_per_iteration": 1e3 * t["vector_ms"] / t["iterations"],
        "vector_update_bytes_per_iteration": t["vector_bytes"] / t["iterations"],
        "vector_update_gbs": vec_gbs,
        "check_us_per_check": 1e3 * t["check_ms"] / max(1, t["checks"]),
        "check_gbs": chk_gbs,
        "hbm_peak_gbs": peak, "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy)",
        "vector_update_frac": vec_gbs / peak if peak else None,
        "check_frac": chk_gbs / peak if peak else None,
        "matvec_us": t_mdot * 1e6,
        "vector_share_of_iteration": (t["vector_ms"] / t["iterations"])
        / (t["vector_ms"] / t["iterations"] + t_mdot * 1e3),
        "note": "checks run on a high-priority side stream, overlapping the next matvec",
    }


def cpu_baseline(w, pos, F, T, seconds=8.0):
    """FP64 C oracle (all host threads) on a bounded sample of the workload:
    the first R target rows against every source."""
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle as orc
    cores = os.cpu_count() or 1
    N = w["N"]
    rows = max(cores, 8)
    while True:
        t0 = time.perf_counter()
        orc.mdot(pos, F, T, a=1.0, viscosity=1 / (6 * math.pi), wall=w["wall"],
                 include_angular=w["ang"], rows=(0, rows), nthreads=cores)
        dt = time.perf_counter() - t0
        if dt > seconds / 4 or rows >= N:
            break
        rows = min(N, int(rows * max(2.0, seconds / 4 / max(dt, 1e-3))))
    reps = max(1, int(seconds / max(dt, 1e-3)))
    t0 = time.perf_counter()
    for _ in range(reps):
        orc.mdot(pos, F, T, a=1.0, viscosity=1 / (6 * math.pi), wall=w["wall"],
                 include_angular=w["ang"], rows=(0, rows), nthreads=cores)
    dt = (time.perf_counter() - t0) / reps
    return {"value": rows * N / dt, "unit": "pair-interactions/s", "cores": cores,
            "kind": "port",
            "sample": f"FP64 C oracle, Mdot rows 0..{rows - 1} x {N} sources, {reps} reps"}


def oracle_error_open4k(pos, F, results):
    """Max |U - U_oracle| / max |U_oracle| of the open N = 4096 products
    against the FP64 C oracle (all host threads), every row."""
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle as orc
    Uo, _ = orc.mdot(pos, F, None, a=1.0, viscosity=1 / (6 * math.pi), wall=0,
                     include_angular=0, nthreads=os.cpu_count() or 1)
    Uo = np.asarray(Uo, np.float64).reshape(-1)
    scale = np.abs(Uo).max()
    return {p: float(np.abs(u.reshape(-1) - Uo).max() / scale) for p, u in results.items()}


def line_config(w, ws):
    """The config object both arms print: the workload, its size and
    tolerance, how caches are kept out of the timing, and the rank layout."""
    return {"workload": w["desc"], "N": w["N"], "tolerance": w["tol"],
            "l2": "GPU arm: L2 flushed between timed steps (inputs smaller than L2); "
                  "CPU arm: no GPU, host caches as they are",
            "parallelism": f"replicas x{ws}"}


def run_reference(args, w, ws, rank):
    if rank != 0:
        return
    pos, F, T, _ = make_inputs(w, 1234)
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(w, pos, F, T, seconds=1.0)
    for _ in range(args.steps):
        vals.append(cpu_baseline(w, pos, F, T, seconds=4.0))
    v = statistics.median(x["value"] for x in vals)
    base = dict(vals[0], value=v)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "pair-interactions/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": line_config(w, ws),
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": "pair-interactions/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args, w, ws, rank, local):
    import torch
    from libmobility_gb300 import NBody, _capi
    lib = _capi.load()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pos, F, T, dW = make_inputs(w, 1234 + rank)
    N = w["N"]
    eta = 1 / (6 * math.pi)
    s = NBody("open", "open", "single_wall" if w["wall"] else "open", precision="float")
    s.setParameters(**({"wallHeight": 0.0} if w["wall"] else {}))
    s.initialize(viscosity=eta, hydrodynamicRadius=1.0, includeAngular=w["ang"],
                 tolerance=w["tol"], seed=7 + rank)
    f32 = dict(dtype=torch.float32, device=dev)
    dpos = torch.tensor(pos, **f32)
    dF = torch.tensor(F, **f32)
    dT = torch.tensor(T, **f32) if T is not None else None
    ddW = torch.tensor(dW, **f32)
    s.setPositions(dpos)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    iters = []

    def step():
        s.Mdot(dF, dT)
        _, _, it, _ = s.sqrtMdotW_noise(ddW)
        iters.append(it)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    iters.clear()
    n0 = lib.lmg_internal_launch_count()
    times = []
    with ClockSampler(local) as clk:
        barrier(ws)
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush_l2(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            step()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
        torch.cuda.synchronize()
        barrier(ws)
    launches = lib.lmg_internal_launch_count() - n0
    clocks = clk.summary()
    pairs = N * N
    it_mean = sum(iters) / len(iters)
    pairs_per_step = pairs * (1 + (it_mean + 1))  # Mdot + (iterations+1) matvecs
    t_local = sum(times) / len(times)
    value = aggregate_rate(pairs_per_step, t_local, ws)
    t_step = max_over_ranks(t_local, ws)

    # --- kernel-level figures: Mdot alone ---
    t_mdot, kernel_timing = mdot_kernel_time(torch, s, dF, dT)
    # sqrtMdotW alone
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        s.sqrtMdotW_noise(ddW)
    torch.cuda.synchronize()
    t_sqrt = (time.perf_counter() - t0) / 3
    krylov = krylov_phases(torch, s, ddW, t_mdot)
    peak = fp32_peak_tflops(lib, torch)
    peak64 = fp64_peak_tflops(lib, torch)
    open4k, pos1, F1, res1 = open4k_mdot(torch, lib, peak, peak64, flush)
    open4k_sq = open4k_sqrt(torch, lib)
    ref_gpu = None
    if not args.skip_reference_gpu:
        ref_gpu = reference_gpu_mdot(torch, (pos, F, T, dW))
    fpp = FLOPS_PER_PAIR[("wall" if w["wall"] else "open", w["ang"])]
    achieved = pairs * fpp / t_mdot / 1e12

    # --- e2e through the public API with host buffers ---
    pos32 = pos.astype(np.float32)
    F32 = F.astype(np.float32)
    T32 = T.astype(np.float32) if T is not None else None
    dW32 = dW.astype(np.float32)
    s2 = NBody("open", "open", "single_wall" if w["wall"] else "open", precision="float")
    s2.setParameters(**({"wallHeight": 0.0} if w["wall"] else {}))
    s2.initialize(viscosity=eta, hydrodynamicRadius=1.0, includeAngular=w["ang"],
                  tolerance=w["tol"], seed=7 + rank)
    e2e_iters = []

    def step_e2e():
        s2.setPositions(pos32)
        U, W = s2.Mdot(F32, T32)
        u, wv, it, _ = s2.sqrtMdotW_noise(dW32)
        e2e_iters.append(it)
        return U, W, u, wv

    for _ in range(2):
        step_e2e()
    e2e_iters.clear()
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    torch.cuda.synchronize()
    t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps, ws)
    it_e2e = sum(e2e_iters) / len(e2e_iters)
    h2d = pos32.nbytes + F32.nbytes + (T32.nbytes if T32 is not None else 0) + dW32.nbytes
    d2h = 2 * 4 * 3 * N * (2 if w["ang"] else 1)
    e2e_value = pairs * (1 + (it_e2e + 1)) * ws / t_e2e

    cmp = None
    if not args.skip_precond:
        # the preconditioned stopping step moves by +-4 from one dW to the next:
        # at least 12 solves per arm
        cmp = sqrtmdotw_comparison(torch, max(12, args.steps), 2, rank)
        cmp["network_gemm"] = precond_network_gemms(torch, lib)
    ens = None
    if not args.skip_ensemble:
        ens = ensemble_comparison(torch, max(2, args.steps), 2, rank, peak=peak)
    large = large_sqrt = None
    if not args.skip_large:
        large = large_wall_mdot(torch, rank)
        large["frac_of_fp32_peak"] = large["achieved_tflops"] / peak
        large_sqrt = large_wall_sqrt(torch, rank)

    if rank != 0:
        return
    cpu = cpu_baseline(w, pos, F, T)
    err1 = oracle_error_open4k(pos1, F1, res1)
    for prec, e in err1.items():
        open4k[prec]["max_rel_err_vs_fp64_oracle"] = e
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    datasheet = (sms * 256 * clocks["sm_mhz"] * 1e-6) if clocks else None
    line = {
        "metric": METRIC, "value": value, "unit": "pair-interactions/s", "n_gpus": ws,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": line_config(w, ws),
        "sqrtMdotW": {"solves_per_s": 1.0 / t_sqrt, "lanczos_iterations": it_mean,
                      "preconditioner": "none (plain Lanczos)"},
        "sqrtMdotW_learned_vs_plain": cmp,
        "ensemble_256": ens,
        "wall_262k_mdot": large,
        "wall_262k_sqrt": large_sqrt,
        "open4k_mdot": open4k,
        "open4k_sqrt": open4k_sq,
        "reference_gpu": ref_gpu,
        "krylov_phases": krylov,
        "mdot_pair_interactions_per_s": pairs / t_mdot,
        "e2e": {"value": e2e_value, "unit": "pair-interactions/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": t_e2e * 1e3},
        "roofline": {"bound": "fp32", "kernel": "mdot_kernel (pair interactions)",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": MDOT_TRAFFIC.get(args.workload),
                     "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "ncu capture of this kernel and workload",
                     "peak_source": "FP32 FMA-chain probe measured in this run",
                     "datasheet_fp32_tflops": datasheet,
                     "datasheet_note": "SMs x 128 FP32 FMA/clk x 2 flops x median SM clock "
                                       "under load",
                     "flops_per_pair": fpp, "kernel_ms": t_mdot * 1e3,
                     "kernel_timing": kernel_timing},
        "cpu_baseline": cpu,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="wall16k", choices=sorted(WORKLOADS))
    ap.add_argument("--skip-precond", action="store_true",
                    help="skip the plain vs learned-preconditioner sqrtMdotW comparison")
    ap.add_argument("--skip-ensemble", action="store_true",
                    help="skip the batched ensemble of 256 uneven systems")
    ap.add_argument("--skip-large", action="store_true",
                    help="skip the N = 262144 single-wall Mdot and square roots")
    ap.add_argument("--skip-reference-gpu", action="store_true",
                    help="skip the reference CUDA kernel timed beside this library's Mdot")
    ap.add_argument("--only", choices=["ensemble", "precond", "open4k", "large", "tcgemm"],
                    default=None,
                    help="run one sub-measurement alone and print it (for profiling)")
    ap.add_argument("--ensemble-systems", type=int, default=256)
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    ws, rank, local = dist_setup()
    if args.only == "ensemble":  # the ensemble measurement alone (profiling runs)
        import torch
        out = ensemble_comparison(torch, args.steps, args.warmup, rank, args.ensemble_systems,
                                  sequential=False)
        if rank == 0:
            print(json.dumps({"ensemble": out}))
        return
    if args.only == "precond":  # plain vs learned sqrtMdotW alone (profiling runs)
        import torch
        out = sqrtmdotw_comparison(torch, args.steps, args.warmup, rank)
        if rank == 0:
            print(json.dumps({"sqrtMdotW_learned_vs_plain": out}))
        return
    if args.only == "tcgemm":  # the preconditioner network's GEMMs alone (profiling runs)
        import torch
        from libmobility_gb300 import _capi
        out = precond_network_gemms(torch, _capi.load())
        if rank == 0:
            print(json.dumps({"precond_network_gemm": out}))
        return
    if args.only == "large":  # the N = 262144 wall square roots alone
        import torch
        out = large_wall_sqrt(torch, rank)
        if rank == 0:
            print(json.dumps({"wall_262k_sqrt": out}))
        return
    if args.only == "open4k":  # the open N = 4096 figures alone (profiling runs)
        import torch
        from libmobility_gb300 import _capi
        lib = _capi.load()
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
        out, _, _, _ = open4k_mdot(torch, lib, fp32_peak_tflops(lib, torch),
                                   fp64_peak_tflops(lib, torch), flush)
        sq = open4k_sqrt(torch, lib)
        if rank == 0:
            print(json.dumps({"open4k_mdot": out, "open4k_sqrt": sq}))
        return
    if args.impl == "reference":
        run_reference(args, w, ws, rank)
    else:
        run_ours(args, w, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
