"""Autotuner of the launch shape of a device simulation.

The results of a simulation do not depend on the launch shape (threads per block of the contact
kernels, steps queued per host check of the collider request, CUDA-graph replay of such a chunk of
steps): every contact and every particle is updated by the same operations in the same order.
The tuner therefore measures candidate shapes on real steps of the simulation it tunes (the steps
count as part of the run) and keeps the fastest by the median over rounds, the default shape
unless another is faster by more than a margin.
"""
import ctypes as C

import numpy as np

DEFAULT_CANDIDATES = (
    # (contact threads per block, steps per chunk, CUDA graph, facet/wall contacts on a second
    # stream beside the sphere-sphere ones); block -256 selects the resident-grid FP32
    # sphere-sphere kernel whose threads prefetch their next contact
    (-256, 32, False, True),
    (-256, 32, False, False),
    (256, 32, False, True),
    (128, 32, False, True),
    (-256, 8, True, True),
    (-256, 32, True, True),
    (-256, 32, True, False),
    (-256, 64, True, True),
)


def _handle(sim):
    return sim.H.L, sim.H.h


def set_launch(sim, block=0, chunk=32, graph=False, concurrent=True):
    L, h = _handle(sim)
    flags = (1 if graph else 0) | (0 if concurrent else 2)
    sim.H.check(L.wg_set_launch(h, int(block), int(chunk), flags), "set_launch")


def _run_ms(sim, steps):
    sim.run(steps)
    L, h = _handle(sim)
    tot = C.c_double()
    ph = np.zeros(4)
    nl = C.c_int64()
    L.wg_get_timing(h, C.byref(tot), ph.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nl))
    return tot.value


def autotune(sim, trial_steps=64, candidates=DEFAULT_CANDIDATES, rounds=3, margin=0.02):
    """Time ``trial_steps`` steps of ``sim`` (a Simulation or a Batch) with each candidate launch
    shape, ``rounds`` times in turn (the median counts), set the fastest and return
    (best, {candidate: ms per step}). The first candidate is the default shape; another one is
    chosen only if it is faster than the default by more than ``margin`` (a fraction), so that
    timing noise does not pick a shape that is no better."""
    times = {c: [] for c in candidates}
    for _ in range(rounds):
        for c in candidates:
            set_launch(sim, *c)
            times[c].append(_run_ms(sim, trial_steps) / trial_steps)
    med = {c: float(np.median(v)) for c, v in times.items()}
    default = candidates[0]
    best = min(med, key=med.get)
    if med[best] > (1.0 - margin) * med[default]:
        best = default
    set_launch(sim, *best)
    return best, med
