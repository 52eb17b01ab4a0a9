"""Serving loop: scene jobs admitted as they arrive, continuously batched on one GPU.

Aperiodic jobs (box settles of spheres and walls) run in the slots of one device simulation (a
SlotPool): a slot holds one job at a time and is reloaded in place when its job ends, while the
other slots keep running with their state and contacts on the device, so jobs that arrive while
others are on the GPU join them at the next tick. Periodic jobs (one periodic cell per
simulation) run as their own simulations on their own CUDA streams, driven by worker threads, so
their work overlaps the slots' on the device. Admission is against an HBM budget (device bytes per
particle of a slot or a job) and the slots' capacities.

A job's result does not depend on what runs beside it: a slot integrates its job with the same
operations, in the same order, as the job alone (see woodem_gb300.batch).
"""
import ctypes as C
import math
import threading
import time

import numpy as np

from . import _native, _plan

# device bytes per particle held by the GPU path (state, mirrors, contacts with ~6 potential
# contacts per sphere, incidence, collider scratch); used for admission
BYTES_PER_PARTICLE = 3000


class SlotPool:
    """A device simulation whose scenes are ``len(capacities)`` slots of the given particle
    capacities (all empty at first)."""

    def __init__(self, capacities, precision="fp64", mats_per_slot=2, device=0, template=None):
        self.cap = np.asarray(capacities, dtype=np.int64)
        K = len(self.cap)
        self.K = K
        self.start = np.concatenate([[0], np.cumsum(self.cap)]).astype(np.int64)
        n = int(self.start[-1])
        self.mats_per_slot = mats_per_slot
        self.H = _native.Handle(device)
        L, h = self.H.L, self.H.h
        cfg = dict(template.config) if template is not None else None
        if cfg is None:
            raise ValueError("SlotPool needs a template job (its configuration sets precision and masks)")
        cfg["precision"] = {"fp64": 0, "fp32": 1}[precision]
        cfgs = (_native.wg_config * K)(*[_native.make_config(_native.wg_config, cfg) for _ in range(K)])
        pstart = np.ascontiguousarray(self.start)
        self.H.check(L.wg_set_scenes(h, K, C.cast(cfgs, C.c_void_p), pstart.ctypes.data_as(C.POINTER(C.c_int64))), "set_scenes")
        m = K * mats_per_slot
        one = np.ones(m)
        self.H.check(L.wg_set_materials(h, m, _native.ptr(one * 1000), _native.ptr(one * 1e7), _native.ptr(one * .5),
                                        _native.ptr(one * .2)), "set_materials")
        z3 = np.zeros((n, 3))
        ori = np.tile([1.0, 0, 0, 0], (n, 1))
        self.H.check(L.wg_set_nodes(h, n, _native.ptr(z3), _native.ptr(ori), _native.ptr(z3), _native.ptr(z3), _native.ptr(z3),
                                    _native.ptr(z3), _native.ptr(np.ones(n)), _native.ptr(np.ones((n, 3))),
                                    _native.ptr(np.full(n, 63, np.uint32), _native.P_U32)), "set_nodes")
        nodes = np.full((n, 3), -1, np.int32)
        nodes[:, 0] = np.arange(n, dtype=np.int32)
        mat = np.repeat(np.arange(K, dtype=np.int32) * mats_per_slot, self.cap)
        self.H.check(L.wg_set_particles(h, n, _native.ptr(np.zeros(n, np.int32), _native.P_I32), _native.ptr(nodes, _native.P_I32),
                                        _native.ptr(np.full(n, 1e-3)), _native.ptr(np.zeros(n, np.int32), _native.P_I32),
                                        _native.ptr(np.zeros(n, np.int32), _native.P_I32), _native.ptr(np.zeros(n)),
                                        _native.ptr(np.zeros((n, 3))), _native.ptr(mat, _native.P_I32),
                                        _native.ptr(np.zeros(n, np.uint32), _native.P_U32)), "set_particles")
        for k in range(K):
            self.H.check(L.wg_slot_clear(h, k), "slot_clear")
        self.job = [None] * K

    def load(self, k, A, n_steps, job=None):
        """Put the compiled scene ``A`` (woodem_gb300._plan.compile_scene) into slot k for n_steps."""
        L, h = self.H.L, self.H.h
        nd, pa, mt = A.nodes, A.particles, A.materials
        if np.any(pa["nodes"][:, 0] != np.arange(A.n_particles)) or A.n_nodes != A.n_particles:
            raise ValueError("slot jobs have one node per particle, in particle order")
        if A.config.get("track_energy"):
            raise NotImplementedError("energy tracking is not supported in serving slots")
        p = _native.ptr
        cfg = _native.make_config(_native.wg_config, A.config)
        self.H.check(L.wg_slot_load(h, k, C.cast(C.byref(cfg), C.c_void_p), A.n_particles, p(nd["pos"]), p(nd["ori"]), p(nd["vel"]),
                                    p(nd["angVel"]), p(nd["mass"]), p(nd["inertia"]), p(nd["flags"], _native.P_U32),
                                    p(np.ascontiguousarray(pa["shape"], np.int32), _native.P_I32), p(pa["radius"]),
                                    p(np.ascontiguousarray(pa["axis"], np.int32), _native.P_I32),
                                    p(np.ascontiguousarray(pa["sense"], np.int32), _native.P_I32),
                                    p(np.ascontiguousarray(pa["mat"], np.int32), _native.P_I32), p(pa["mask"], _native.P_U32),
                                    len(mt["density"]), p(mt["density"]), p(mt["young"]), p(mt["tanPhi"]), p(mt["ktDivKn"]),
                                    int(n_steps)), "slot_load")
        self.job[k] = job

    def clear(self, k):
        self.H.check(self.H.L.wg_slot_clear(self.H.h, k), "slot_clear")
        self.job[k] = None

    def status(self, k):
        d, e = C.c_int64(), C.c_int64()
        self.H.check(self.H.L.wg_slot_status(self.H.h, k, C.byref(d), C.byref(e)), "slot_status")
        return d.value, e.value

    def nodes(self, k, n):
        out = {key: np.empty((n, w)) for key, w in (("pos", 3), ("ori", 4), ("vel", 3), ("angVel", 3), ("force", 3), ("torque", 3))}
        self.H.check(self.H.L.wg_get_slot_nodes(self.H.h, k, n, *[_native.ptr(out[key]) for key in
                                                                  ("pos", "ori", "vel", "angVel", "force", "torque")]),
                     "get_slot_nodes")
        return out

    def run(self, n):
        self.H.check(self.H.L.wg_run(self.H.h, int(n)), "run")

    def close(self):
        if self.H is not None:
            self.H.close()
            self.H = None


class Job:
    """A scene job: ``build()`` returns the Scene (built when the job is admitted), ``steps`` the
    number of steps to run; ``n`` its particle count (for admission). A periodic job may give
    ``phases``: a list of (fraction of its steps, Cell.nextGradV) run in turn (e.g. an isotropic
    compression, then the shear); the steps of the phases add up to ``steps``."""

    def __init__(self, jid, build, n, steps, arrival, periodic=False, phases=None):
        self.id, self.build, self.n, self.steps, self.arrival, self.periodic = jid, build, n, steps, arrival, periodic
        self.phases = phases
        self.start = self.end = None
        self.result = None
        self.done_steps = 0

    def phase_steps(self):
        """(steps, nextGradV or None) of each phase."""
        if not self.phases:
            return [(self.steps, None)]
        out, left = [], self.steps
        for k, (frac, g) in enumerate(self.phases):
            n = left if k == len(self.phases) - 1 else min(left, int(round(frac * self.steps)))
            out.append((n, g))
            left -= n
        return out


class Server:
    """Continuous batching of jobs: aperiodic jobs in the slots of a SlotPool (reloaded in place as
    jobs end), periodic jobs as their own simulations in worker threads. ``clock`` is "wall" (job
    arrivals and latencies in seconds of wall time) or "ticks" (arrivals in ticks, deterministic)."""

    def __init__(self, pool, hbm_budget=150e9, tick=500, max_periodic=4, keep_results=False, clock="wall", periodic_chunk=2000):
        self.pool = pool
        self.budget = hbm_budget
        self.tick = tick
        self.max_periodic = max_periodic
        self.keep = keep_results
        self.clock = clock
        self.periodic_chunk = periodic_chunk
        self.done = []
        self.steps_done = 0
        self.particle_steps = 0.0
        self.partial_particle_steps = 0.0   # steps done by jobs still unfinished when the run stopped
        self.pool_bytes = float(pool.start[-1]) * BYTES_PER_PARTICLE

    def _now(self, t0, ticks):
        return time.perf_counter() - t0 if self.clock == "wall" else float(ticks)

    def run(self, jobs, horizon=None):
        """Serve ``jobs`` (sorted by arrival); returns the finished jobs. Stops when all jobs are
        done, or at ``horizon`` (seconds or ticks) with the unfinished ones left out (the steps
        they did are counted in ``partial_particle_steps``)."""
        pending = list(jobs)
        queue = []
        periodic_running = []
        lock = threading.Lock()
        stop = threading.Event()
        t0 = time.perf_counter()
        ticks = 0
        used_periodic_bytes = [0.0]

        errors = []

        def run_periodic(job):
            try:
                run_periodic_job(job)
            except BaseException as e:  # re-raised by the serving loop
                with lock:
                    errors.append(e)
                    used_periodic_bytes[0] -= job.n * BYTES_PER_PARTICLE
                stop.set()

        def run_periodic_job(job):
            job.start = self._now(t0, ticks)
            S = job.build()
            for n, g in job.phase_steps():
                if g is not None:
                    S.cell.nextGradV = np.asarray(g, dtype=float)
                while n > 0 and not stop.is_set():
                    k = min(n, self.periodic_chunk)
                    S.run(k)
                    n -= k
                    job.done_steps += k
            finished = job.done_steps >= job.steps
            if finished:
                S.sync()
                if self.keep:
                    job.result = {k: S.dem._nodes.soa.col(k).copy() for k in ("pos", "vel", "angVel", "force", "torque")}
            S.close()
            with lock:
                used_periodic_bytes[0] -= job.n * BYTES_PER_PARTICLE
                if finished:
                    job.end = self._now(t0, ticks)
                    self.done.append(job)
                    self.particle_steps += job.n * job.steps
                else:
                    self.partial_particle_steps += job.n * job.done_steps

        while True:
            if errors:
                break
            now = self._now(t0, ticks)
            while pending and pending[0].arrival <= now:
                queue.append(pending.pop(0))
            # admission: periodic jobs to threads, the others to free slots that fit (first come)
            still = []
            for job in queue:
                if job.periodic:
                    busy = sum(1 for th in periodic_running if th.is_alive())
                    need = job.n * BYTES_PER_PARTICLE
                    if busy < self.max_periodic and self.pool_bytes + used_periodic_bytes[0] + need <= self.budget:
                        used_periodic_bytes[0] += need
                        th = threading.Thread(target=run_periodic, args=(job,), daemon=True)
                        th.start()
                        periodic_running.append(th)
                        continue
                    still.append(job)
                    continue
                free = [k for k in range(self.pool.K) if self.pool.job[k] is None and self.pool.cap[k] >= job.n]
                if free:
                    k = min(free, key=lambda q: self.pool.cap[q])
                    S = job.build()
                    A = _plan.compile_scene(S)
                    self.pool.load(k, A, job.steps, job=job)
                    job.start = now
                    job.A = A
                    continue
                still.append(job)
            queue = still
            periodic_running = [th for th in periodic_running if th.is_alive()]
            active = [k for k in range(self.pool.K) if self.pool.job[k] is not None]
            if not active and not queue and not pending and not periodic_running:
                break
            if horizon is not None and now >= horizon:
                for k in active:
                    self.partial_particle_steps += self.pool.job[k].n * min(self.pool.status(k)[0], self.pool.job[k].steps)
                stop.set()
                break
            if active:
                # run to the next tick, or to the end of the earliest job if sooner
                left = min(self.pool.job[k].steps - self.pool.status(k)[0] for k in active)
                n = max(1, min(self.tick, left))
                self.pool.run(n)
                self.steps_done += n
                ticks += 1
                for k in active:
                    d, e = self.pool.status(k)
                    job = self.pool.job[k]
                    if d >= job.steps:
                        if self.keep:
                            job.result = self.pool.nodes(k, job.A.n_nodes)
                        job.end = self._now(t0, ticks)
                        self.particle_steps += job.n * job.steps
                        self.done.append(job)
                        self.pool.clear(k)
            else:
                if self.clock == "wall":
                    time.sleep(0.002)
                ticks += 1
        for th in periodic_running:
            th.join()
        if errors:
            raise RuntimeError("a periodic job failed: %r" % (errors[0],)) from errors[0]
        self.elapsed = time.perf_counter() - t0
        return self.done


def poisson_jobs(rate, horizon, seed, make_box, make_peri, nmin, nmax, smin, smax, p_periodic=0.5, peri_phases=None):
    """Seeded Poisson stream of jobs over [0, horizon): sizes log-uniform in [nmin, nmax], step counts
    uniform in [smin, smax], periodic with probability p_periodic; ``make_box(n, seed)`` and
    ``make_peri(n, seed)`` build the scenes; ``peri_phases(n, steps, seed)`` gives the phases of a
    periodic job (or None)."""
    rng = np.random.default_rng(seed)
    t, jobs, jid = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= horizon:
            break
        n = int(math.exp(rng.uniform(math.log(nmin), math.log(nmax))))
        steps = int(rng.integers(smin, smax + 1))
        peri = bool(rng.random() < p_periodic)
        s = int(rng.integers(0, 2 ** 31))
        build = (lambda n=n, s=s: make_peri(n, s)) if peri else (lambda n=n, s=s: make_box(n, s))
        phases = peri_phases(n, steps, s) if (peri and peri_phases) else None
        jobs.append(Job(jid, build, n + (0 if peri else 6), steps, t, periodic=peri, phases=phases))
        jid += 1
    return jobs


def latency_stats(jobs):
    lat = np.array([j.end - j.arrival for j in jobs if j.end is not None])
    if len(lat) == 0:
        return {"p50": None, "p99": None, "n": 0}
    return {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)), "mean": float(lat.mean()), "n": int(len(lat))}
