"""bench.py under torch.distributed with two ranks (gloo, CPU): the replica barrier, the
max-over-ranks time and the whole-job rate (units of all ranks over the slowest rank's time)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        r, w, _ = bench.env_rank()
        bench.barrier(w)
        m = bench.allreduce_max(10.0 + rank, w)
        value, ms = bench.replica_rate(1000 * 50, 20.0 + 5.0 * rank, w)
        q.put((rank, r, w, m, value, ms))
    finally:
        dist.destroy_process_group()


def test_replica_rate_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r, w, m, value, ms in out:
        assert (r, w) == (rank, 2)
        assert m == 11.0                      # max over ranks
        assert ms == 25.0                     # the slowest rank's time
        assert value == 2 * 1000 * 50 / 0.025  # units of both ranks over it


def test_replica_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    value, ms = bench.replica_rate(1000, 500.0, 1)
    assert (value, ms) == (2000.0, 500.0)
