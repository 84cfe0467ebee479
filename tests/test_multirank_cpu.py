"""bench.py's multi-rank path on CPU: two gloo ranks run as replicas, the
barrier holds, timing is the maximum over ranks and the whole-job rate counts
every rank's work over the slowest rank's time."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    bench.barrier(ws)
    t = 1.0 + rank  # rank 1 is the slow one
    m = bench.max_over_ranks(t, ws)
    rate = bench.aggregate_rate(100.0, t, ws)
    bench.barrier(ws)
    dist.destroy_process_group()
    q.put((rank, m, rate))


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, rate in res:
        assert m == 2.0            # max over ranks
        assert rate == 100.0       # 2 ranks x 100 units / 2 s
