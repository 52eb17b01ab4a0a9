"""Independent scenes spread over several GPUs: batches and job streams split by scene.

The reference runs a parametric study as one process per table line (``woo-batch``,
core/main/wooMain.py:753-852): lines never exchange data, so they scale by placing them on
separate workers. Here the worker is a GPU: every scene (or job) goes to one device, chosen by its
device-memory footprint so that the devices carry similar loads, and the scenes of one device run
together in one Batch (or one serving pool). No data moves between devices while the scenes run;
the results are gathered on the host at the end.

Two ways to drive it:
* one process, several devices: ``ShardedBatch(scenes, devices=[0, 1, ...])`` builds one Batch per
  device and advances them from one host thread each;
* one process per device (torch.distributed, as launched by ``torch.distributed.run``):
  ``run_distributed(scenes, steps, rank, world)`` runs the scenes assigned to ``rank`` on its
  local GPU and gathers every scene's result on all ranks (``all_gather_object``: host data, no
  device collective on the data path); ``serve_distributed`` does the same for a job stream.
  Every rank builds the same scene list (or stream) from the same seeds and computes the same
  assignment, so the ranks agree on who runs what without exchanging it.

``assign`` is deterministic: the same footprints and device count give the same placement.
"""
import threading

import numpy as np

# device bytes per particle of the GPU path (state, mirrors, ~6 potential contacts per sphere,
# incidence, collider scratch), the unit of the footprint
BYTES_PER_PARTICLE = 3000


def footprint(S):
    """Device-memory footprint of a scene in bytes (its particle count times the per-particle figure)."""
    return float(len(S.dem.par)) * BYTES_PER_PARTICLE


def assign(footprints, n_devices, capacity=None):
    """Place items of the given footprints on n_devices devices: largest first, each on the device
    with the least load so far (ties to the lower device index). Returns the device of each item,
    in item order. With ``capacity`` (bytes per device) an item that fits on no device raises."""
    fp = np.asarray(footprints, dtype=float)
    if n_devices < 1:
        raise ValueError("n_devices must be at least 1")
    load = np.zeros(n_devices)
    out = np.zeros(len(fp), dtype=np.int64)
    for i in np.argsort(-fp, kind="stable"):
        d = int(np.argmin(load))
        if capacity is not None and load[d] + fp[i] > capacity:
            raise MemoryError("item %d (%.3g bytes) fits on no device (capacity %.3g bytes)" % (i, fp[i], capacity))
        out[i] = d
        load[d] += fp[i]
    return out


def assign_stream(jobs, n_devices):
    """Placement of a job stream, in arrival order: each job goes to the device with the least
    work (particles x steps) assigned so far. It depends on the stream alone, so every rank that
    generates the same stream computes the same placement without exchanging it."""
    work = np.zeros(n_devices)
    out = np.zeros(len(jobs), dtype=np.int64)
    for i, j in enumerate(sorted(range(len(jobs)), key=lambda q: (jobs[q].arrival, q))):
        d = int(np.argmin(work))
        out[j] = d
        work[d] += float(jobs[j].n) * float(jobs[j].steps)
    return out


def serve_distributed(jobs, rank, world, serve_fn):
    """Serve the jobs placed on this rank (``assign_stream``) with ``serve_fn(jobs) -> finished
    jobs`` (for example a Server on a SlotPool of this rank's GPU) and gather, on every rank, the
    (id, arrival, start, end, n, steps) record of every finished job of all ranks."""
    dev = assign_stream(jobs, world)
    mine = [j for j, d in zip(jobs, dev) if d == rank]
    done = serve_fn(mine) if mine else []
    local = [(j.id, j.arrival, j.start, j.end, j.n, j.steps) for j in done]
    if world == 1:
        parts = [local]
    else:
        import torch.distributed as dist
        parts = [None] * world
        dist.all_gather_object(parts, local)
    return sorted((r for part in parts for r in part), key=lambda r: r[0]), dev


def _default_runner(scenes, steps, device):
    """Run the scenes as one Batch on ``device`` for ``steps`` steps and return each scene's
    node state (pos, vel, angVel, force, torque) and Scene.step."""
    from .batch import Batch
    for S in scenes:
        S.gpu.device = device
    B = Batch(scenes, device=device)
    B.run(steps)
    B.close()
    out = []
    for S in scenes:
        nd = S.dem._nodes.soa
        out.append({"step": int(S.step), **{k: nd.col(k).copy() for k in ("pos", "vel", "angVel", "force", "torque")}})
    return out


def run_distributed(scenes, steps, rank, world, runner=None, footprints=None):
    """Run the scenes assigned to this rank (one Batch on this rank's GPU) for ``steps`` steps and
    return every scene's result, gathered from all ranks, in scene order. ``runner(scenes, steps,
    device)`` runs a list of scenes (the default builds a Batch on the GPU); ``footprints``
    overrides the per-scene footprint. Needs an initialised torch.distributed process group when
    world > 1 (any backend: the gather carries host objects)."""
    runner = runner or _default_runner
    fps = footprints if footprints is not None else [footprint(S) for S in scenes]
    dev = assign(fps, world)
    mine = [i for i in range(len(scenes)) if dev[i] == rank]
    res = runner([scenes[i] for i in mine], steps, rank) if mine else []
    local = list(zip(mine, res))
    if world == 1:
        gathered = [local]
    else:
        import torch.distributed as dist
        gathered = [None] * world
        dist.all_gather_object(gathered, local)
    out = [None] * len(scenes)
    for part in gathered:
        for i, r in part:
            out[i] = r
    if any(r is None for r in out):
        raise RuntimeError("a scene was run by no rank")
    return out, dev


class ShardedBatch:
    """The scenes split over several devices of one process, one Batch per device, advanced from
    one host thread per device (each device's steps run while the others' do)."""

    def __init__(self, scenes, devices, footprints=None):
        from .batch import Batch
        self.scenes = list(scenes)
        self.devices = list(devices)
        fps = footprints if footprints is not None else [footprint(S) for S in self.scenes]
        self.device_of = assign(fps, len(self.devices))
        self.batches = []
        for k, d in enumerate(self.devices):
            group = [S for S, g in zip(self.scenes, self.device_of) if g == k]
            if group:
                for S in group:
                    S.gpu.device = d
                self.batches.append(Batch(group, device=d))

    def run(self, n):
        errs = []

        def go(B):
            try:
                B.run(n)
            except BaseException as e:  # raised in the caller below
                errs.append(e)

        th = [threading.Thread(target=go, args=(B,)) for B in self.batches]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if errs:
            raise errs[0]

    def close(self):
        for B in self.batches:
            B.close()
        self.batches = []
