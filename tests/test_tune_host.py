"""Autotuner selection logic (woodem_gb300/tune.py) on the CPU, with a stand-in simulation whose
step time depends on the launch shape: the median over rounds counts, the default shape (the
first candidate) is kept unless another is faster by more than the margin, and the chosen shape
is the one set at the end."""
import ctypes as C

import numpy as np

from woodem_gb300 import tune


class FakeLib:
    def __init__(self, ms_of):
        self.ms_of = ms_of      # launch shape -> ms per step (a list: one value per call in turn)
        self.shape = None
        self.calls = {}
        self.last_ms = 0.0
        self.history = []

    def wg_set_launch(self, h, block, chunk, flags):
        self.shape = (block, chunk, bool(flags & 1), not (flags & 2))
        self.history.append(self.shape)
        return 0

    def wg_get_timing(self, h, tot, ph, nl):
        C.cast(tot, C.POINTER(C.c_double))[0] = self.last_ms
        return 0


class FakeSim:
    def __init__(self, ms_of):
        class H:
            pass
        self.H = H()
        self.H.L = FakeLib(ms_of)
        self.H.h = None
        self.H.check = lambda r, what: None

    def run(self, steps):
        L = self.H.L
        k = L.calls.get(L.shape, 0)
        seq = L.ms_of[L.shape]
        L.last_ms = seq[k % len(seq)] * steps
        L.calls[L.shape] = k + 1


CANDS = ((-256, 32, False, True), (256, 32, False, True), (-256, 8, True, True))


def test_default_kept_within_margin():
    sim = FakeSim({CANDS[0]: [1.00], CANDS[1]: [0.99], CANDS[2]: [1.2]})
    best, med = tune.autotune(sim, trial_steps=10, candidates=CANDS, rounds=3, margin=0.02)
    assert best == CANDS[0] and sim.H.L.history[-1] == CANDS[0]
    assert np.isclose(med[CANDS[1]], 0.99)


def test_faster_shape_chosen():
    sim = FakeSim({CANDS[0]: [1.00], CANDS[1]: [1.1], CANDS[2]: [0.90]})
    best, _ = tune.autotune(sim, trial_steps=10, candidates=CANDS, rounds=3, margin=0.02)
    assert best == CANDS[2] and sim.H.L.history[-1] == CANDS[2]


def test_median_over_rounds():
    # one slow outlier round of the otherwise fastest shape does not disqualify it
    sim = FakeSim({CANDS[0]: [1.00], CANDS[1]: [0.80, 3.0, 0.80], CANDS[2]: [0.95]})
    best, med = tune.autotune(sim, trial_steps=10, candidates=CANDS, rounds=3, margin=0.02)
    assert best == CANDS[1] and np.isclose(med[CANDS[1]], 0.80)
