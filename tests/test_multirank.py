"""The benchmark's multi-rank aggregation on two gloo ranks (CPU): every rank
gets the slowest rank's time, and the whole-job rate counts all ranks' work."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = 10.0 + 5.0 * rank
    got = bench.max_over_ranks(ms, dist, device="cpu")
    rate = bench.whole_job_rate(64, world, got / 1e3)
    q.put((rank, got, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_max_and_weak_scaling_rate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, rate in out:
        assert got == 15.0
        assert abs(rate - 2 * 64 / 0.015) < 1e-6
