"""Scene split over devices (woodem_gb300.shard), tested on the CPU: the footprint placement, and
the two-rank distributed batch and job stream under torch.distributed with the gloo backend, with
a stand-in runner in place of the GPU Batch (each "scene" is a seeded random walk whose result
depends on the scene alone). Checked: every scene runs on exactly one rank, the gathered results
are in scene order and equal to one rank running everything, the loads are balanced."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from woodem_gb300 import shard  # noqa: E402
from woodem_gb300.serve import Job  # noqa: E402


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_assign_balances_and_is_deterministic():
    rng = np.random.default_rng(0)
    fp = np.exp(rng.uniform(np.log(1e3), np.log(5e4), 256)) * 3000
    for nd in (1, 2, 3, 8):
        a = shard.assign(fp, nd)
        assert np.array_equal(a, shard.assign(fp, nd))
        assert set(a.tolist()) == set(range(nd))
        load = np.bincount(a, weights=fp, minlength=nd)
        # largest-first greedy: no device exceeds the average by more than the largest item
        assert load.max() - load.mean() <= fp.max()
    with pytest.raises(MemoryError):
        shard.assign([5.0, 5.0, 5.0], 2, capacity=8.0)


def test_assign_stream_is_a_function_of_the_stream():
    rng = np.random.default_rng(1)
    jobs = [Job(i, None, int(rng.integers(2000, 300000)), int(rng.integers(5000, 50000)), float(t))
            for i, t in enumerate(np.cumsum(rng.exponential(0.05, 200)))]
    a = shard.assign_stream(jobs, 4)
    b = shard.assign_stream(list(reversed(jobs)), 4)  # the same stream listed in another order
    assert np.array_equal(a, b[::-1])
    work = np.bincount(a, weights=[j.n * j.steps for j in jobs], minlength=4)
    assert work.max() - work.mean() <= max(j.n * j.steps for j in jobs)


class _Walk:
    """Stand-in scene: a seeded random walk of n particles."""

    def __init__(self, k, n):
        self.k, self.n = k, n


def _walk_runner(scenes, steps, device):
    out = []
    for s in scenes:
        rng = np.random.default_rng(s.k)
        x = np.zeros((s.n, 3))
        for _ in range(steps):
            x += rng.standard_normal((s.n, 3))
        out.append({"pos": x, "device": device, "step": steps})
    return out


def _scenes():
    rng = np.random.default_rng(7)
    return [_Walk(k, int(rng.integers(5, 60))) for k in range(23)]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from woodem_gb300 import shard as sh
        from woodem_gb300.serve import Job as J
        sc = _scenes()
        res, dev = sh.run_distributed(sc, 7, rank, world, runner=_walk_runner, footprints=[s.n * 3000 for s in sc])
        jobs = [J(i, None, 1000 + 100 * i, 5000, 0.1 * i) for i in range(17)]

        def serve_fn(mine):
            for j in mine:
                j.start, j.end = j.arrival, j.arrival + 1.0 + rank
            return mine

        recs, jdev = sh.serve_distributed(jobs, rank, world, serve_fn)
        q.put((rank, [r["pos"] for r in res], [r["device"] for r in res], dev.tolist(), recs, jdev.tolist()))
    finally:
        dist.destroy_process_group()


def test_distributed_batch_and_stream_two_gloo_ranks():
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
    sc = _scenes()
    alone = _walk_runner(sc, 7, 0)
    (r0, pos0, d0, dev0, recs0, jd0), (r1, pos1, d1, dev1, recs1, jd1) = out
    assert dev0 == dev1 and jd0 == jd1          # both ranks computed the same placement
    assert set(dev0) == {0, 1}
    assert d0 == dev0 and d1 == dev1            # each scene ran on the rank it was placed on
    for k in range(len(sc)):
        assert np.array_equal(pos0[k], alone[k]["pos"]) and np.array_equal(pos1[k], alone[k]["pos"])
    assert recs0 == recs1 and [r[0] for r in recs0] == list(range(17))  # every job once, gathered on both ranks
    for r in recs0:
        assert r[3] - r[1] == pytest.approx(1.0 + jd0[r[0]])  # the record came from the rank that served the job
