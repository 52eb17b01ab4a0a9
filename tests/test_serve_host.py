"""Serving loop host logic on the CPU, with a stand-in for the device slot pool: admission by
arrival (first come), the smallest free slot that holds the job, slots reloaded as jobs end, runs
to the next tick or to the earliest job end, and the latency statistics."""
import numpy as np
import pytest

from woodem_gb300 import serve


class FakePool:
    """The SlotPool interface: slots of fixed capacity that advance their job by `run(n)`."""

    def __init__(self, caps):
        self.cap = np.asarray(caps, dtype=np.int64)
        self.K = len(caps)
        self.start = np.concatenate([[0], np.cumsum(self.cap)])
        self.job = [None] * self.K
        self.done = [0] * self.K
        self.loads = []      # (slot, job id, tick of the load)
        self.runs = []       # steps of each run call
        self.ticks = 0

    def load(self, k, A, n_steps, job=None):
        assert self.job[k] is None and A.n <= self.cap[k]
        self.job[k], self.done[k] = job, 0
        self.loads.append((k, job.id, self.ticks))

    def clear(self, k):
        self.job[k] = None

    def status(self, k):
        j = self.job[k]
        return (self.done[k], j.steps if j else 0)

    def run(self, n):
        self.runs.append(n)
        self.ticks += 1
        for k in range(self.K):
            if self.job[k] is not None:
                self.done[k] = min(self.job[k].steps, self.done[k] + n)

    def nodes(self, k, n):
        return {"pos": np.zeros((n, 3))}


class Desc:
    def __init__(self, n):
        self.n = n
        self.n_nodes = n


@pytest.fixture(autouse=True)
def no_compile(monkeypatch):
    # the stand-in scenes are their own compiled description
    monkeypatch.setattr(serve._plan, "compile_scene", lambda S: S)


def _jobs(specs):
    return [serve.Job(i, (lambda n=n: Desc(n)), n, steps, t) for i, (n, steps, t) in enumerate(specs)]


def test_admission_and_slot_reuse():
    pool = FakePool([100, 400, 400])
    # (size, steps, arrival tick)
    jobs = _jobs([(90, 1000, 0), (300, 250, 0), (350, 600, 0), (380, 100, 1), (50, 300, 2)])
    srv = serve.Server(pool, tick=500, keep_results=True, clock="ticks")
    done = srv.run(jobs)
    assert sorted(j.id for j in done) == [0, 1, 2, 3, 4]
    first = {jid: (k, t) for k, jid, t in pool.loads}
    # the small job takes the small slot, the two large ones the large slots, all at once
    assert first[0][0] == 0 and {first[1][0], first[2][0]} == {1, 2}
    # job 3 (380) waits for a large slot: it is loaded when job 1 (250 steps) has ended
    assert first[3][1] > 0 and first[3][0] == first[1][0]
    for j in done:
        assert j.start >= j.arrival and j.end >= j.start
        assert j.result is not None
    # a run never goes past the earliest end of a running job, nor past a tick
    assert max(pool.runs) <= 500
    assert srv.particle_steps == sum(j.n * j.steps for j in jobs)


def test_job_larger_than_every_slot_waits_forever_and_horizon_stops():
    pool = FakePool([100])
    jobs = _jobs([(50, 200, 0), (500, 100, 0)])
    srv = serve.Server(pool, tick=100, clock="ticks")
    done = srv.run(jobs, horizon=50)
    assert [j.id for j in done] == [0]


def test_latency_stats_and_poisson_stream():
    class J:
        def __init__(self, a, e):
            self.arrival, self.end = a, e
    st = serve.latency_stats([J(0.0, 1.0), J(1.0, 3.0), J(2.0, 2.5)])
    assert st["n"] == 3 and st["p50"] == pytest.approx(1.0)
    assert serve.latency_stats([])["n"] == 0
    a = serve.poisson_jobs(5.0, 10.0, 3, lambda n, s: None, lambda n, s: None, 2000, 30000, 2000, 5000)
    b = serve.poisson_jobs(5.0, 10.0, 3, lambda n, s: None, lambda n, s: None, 2000, 30000, 2000, 5000)
    assert [(j.n, j.steps, j.arrival, j.periodic) for j in a] == [(j.n, j.steps, j.arrival, j.periodic) for j in b]
    assert all(0 <= j.arrival < 10.0 for j in a) and all(2000 <= j.steps <= 5000 for j in a)
    assert all(2000 <= j.n <= 30000 + 6 for j in a)


def test_failed_periodic_job_stops_the_server():
    """A periodic job whose scene cannot be built (its build raises in the worker thread) stops
    the serving loop with an error instead of leaving the job unfinished and its HBM reserved."""
    def bad_build():
        raise RuntimeError("no room for the spheres")
    jobs = [serve.Job(0, (lambda: Desc(100)), 100, 10, 0.0),
            serve.Job(1, bad_build, 1000, 10, 0.0, periodic=True)]
    srv = serve.Server(FakePool([200, 200]), tick=5, clock="ticks")
    with pytest.raises(RuntimeError, match="periodic job failed"):
        srv.run(jobs)
