"""The bench's multi-rank timing on CPU ranks (gloo, world size 2): each
rank times its own replica and the job reports the slowest rank."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = 10.0 * (rank + 1)
        dist.barrier()
        q.put((rank, bench.max_over_ranks(ms, world, "cpu")))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_is_the_job_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 20.0, 1: 20.0}


def test_single_rank_passes_through():
    import bench
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
