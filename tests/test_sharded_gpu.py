"""Row-partitioned sqrtMdotW on the GPU (libmobility_gb300.sharded with the
lmg_mdot_rows product), against the single-GPU solver's sqrtMdotW for the
same Gaussian vector.

One rank without a process group, and two gloo ranks as two processes that
share the one GPU, each with its own NBody handle holding all positions (the
ranks exchange vectors on the host; their kernels never wait on one
another).  At tolerance 1e-3 (about a dozen iterations) the iteration counts
must equal the single-GPU solver's (FP32: within one).  The two solvers sum
in different orders (the row launch splits the sources differently, the
inner products are reduced differently), and Lanczos without
reorthogonalisation amplifies such rounding differences: measured 8e-9
relative in FP64 on open N = 3000.  The results must agree within 1e-6
relative in FP64 and within 5 x tol in FP32, well inside what the tolerance
allows either solve."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-3
AGREE = {"double": 1e-6, "float": 5 * TOL}
SLACK = {"double": 0, "float": 1}


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _system(N, wall, ang, seed=5):
    rng = np.random.default_rng(seed)
    if wall:
        L = (N * 4 * np.pi / 3 / 0.1) ** 0.5
        pos = np.column_stack([rng.uniform(0, L, N), rng.uniform(0, L, N),
                               rng.uniform(1.1, 6.0, N)])
    else:
        pos = rng.uniform(0, (N * 4 * np.pi / 3 / 0.1) ** (1 / 3), (N, 3))
    dW = rng.normal(size=(2 if ang else 1) * 3 * N)
    return pos, dW


def _handle(prec, wall, ang, pos):
    import torch
    from libmobility_gb300 import NBody
    s = NBody("open", "open", "single_wall" if wall else "open", precision=prec)
    if wall:
        s.setParameters("advise", wallHeight=0.0)
    else:
        s.setParameters("advise")
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, includeAngular=bool(ang),
                 tolerance=TOL, seed=1)
    dt = torch.float32 if prec == "float" else torch.float64
    s.setPositions(torch.tensor(pos, dtype=dt, device="cuda"))
    return s


def _sharded(prec, wall, ang, N):
    """prefactor-1 M^{1/2} dW rows of this rank (numpy) and the iteration."""
    import torch
    from libmobility_gb300.sharded import ShardedLanczos, sqrt_mdot_w_rows
    pos, dW = _system(N, wall, ang)
    s = _handle(prec, wall, ang, pos)
    dt = torch.float32 if prec == "float" else torch.float64
    lz = ShardedLanczos(N, include_angular=ang, dtype=dt, device="cuda")
    lin, angv, it = sqrt_mdot_w_rows(s, lz, lz.local_rows(torch.from_numpy(dW)), TOL)
    out = lin.reshape(-1).cpu().numpy().astype(np.float64)
    if ang:
        out = np.concatenate([out, angv.reshape(-1).cpu().numpy().astype(np.float64)])
    return lz.row_begin, lz.row_end, out, it


def _single(prec, wall, ang, N):
    pos, dW = _system(N, wall, ang)
    s = _handle(prec, wall, ang, pos)
    U, W, it, _ = s.sqrtMdotW_noise(dW)
    U = U.reshape(-1).cpu().numpy().astype(np.float64)
    if ang:
        return np.concatenate([U, W.reshape(-1).cpu().numpy().astype(np.float64)]), it
    return U, it


def _rel(x, ref):
    return np.abs(x - ref).max() / np.abs(ref).max()


CASES = [("double", 0, 0, 3000), ("double", 1, 1, 2000), ("float", 0, 0, 4096),
         ("float", 1, 1, 2500)]


@pytest.mark.parametrize("case", CASES)
def test_one_rank_matches_single_gpu_solver(cuda, case):
    prec, wall, ang, N = case
    y1, it1 = _single(prec, wall, ang, N)
    _, _, y, it = _sharded(prec, wall, ang, N)
    assert abs(it - it1) <= SLACK[prec]
    assert _rel(y, y1) <= AGREE[prec]


def _worker(rank, ws, port, case, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        q.put((rank,) + _sharded(*case))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case", [("double", 1, 1, 2000), ("float", 0, 0, 4096)])
def test_two_ranks_match_single_gpu_solver(cuda, case):
    import torch.multiprocessing as mp
    prec, wall, ang, N = case
    y1, it1 = _single(prec, wall, ang, N)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, case, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts = sorted(q.get(timeout=600) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    its = [p[4] for p in parts]
    assert its[0] == its[1] and abs(its[0] - it1) <= SLACK[prec]
    lin, angv = [], []
    for _, b, e, y, _ in parts:
        n = 3 * (e - b)
        lin.append(y[:n])
        angv.append(y[n:])
    y = np.concatenate(lin + (angv if ang else []))
    assert _rel(y, y1) <= AGREE[prec]
