"""bench.py's multi-rank host logic as world_size-2 gloo ranks on the CPU:
per-rank timings max-reduced, whole-job throughput = units of all ranks /
slowest rank (weak scaling, no collective on the data path)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    assert bench.dist_env() == (ws, rank, rank)
    slowest = bench.reduce_max(1.0 + rank, ws, device="cpu")  # rank 1 is slower
    q.put((rank, slowest, bench.job_rate(100.0, slowest, ws)))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 2.0, 100.0), (1, 2.0, 100.0)]


def test_single_rank_is_identity():
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
    assert bench.job_rate(10.0, 2.0, 1) == pytest.approx(5.0)
