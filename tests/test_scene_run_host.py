"""Scene.run / one / stop / wait / running (core/Scene.cpp:33-96) on a stand-in for the device
simulation: a background run issues its steps in chunks from another thread, stop() ends it
after the chunk in progress, wait() joins it and raises the exception it ended with."""
import threading
import time

import pytest

import woodem_gb300 as woo
from woodem_gb300 import _plan
from woodem_gb300.core import Scene
from woodem_gb300.dem import DemField


class _FakeSim:
    """Advances Scene.step by n per run call, slowly; fails at a chosen step."""
    dirty_structure = False

    def __init__(self, S):
        self.S, self.calls, self.threads = S, [], set()
        self.fail_at = getattr(S, "_fail_at", None)

    def run(self, n):
        self.threads.add(threading.current_thread().name)
        self.calls.append(n)
        time.sleep(0.002)
        if self.fail_at is not None and self.S.step + n >= self.fail_at:
            raise RuntimeError("run: injected failure")
        self.S.step += n

    def pull(self):
        pass

    def close(self):
        pass


@pytest.fixture
def S(monkeypatch):
    monkeypatch.setattr(_plan, "Simulation", _FakeSim)
    monkeypatch.setattr(Scene, "_BG_CHUNK", 100)
    return Scene(fields=[DemField()])


def test_run_sets_stop_at_step(S):
    S.run(250)
    assert S.step == 250 and S.stopAtStep == 250 and S._sim.calls == [250]
    S.stopAtStep = 400
    S.run()
    assert S.step == 400
    with pytest.raises(ValueError):
        S.run()  # nothing to run to, and waiting would never end
    S.one()
    assert S.step == 401


def test_background_run_and_wait(S):
    S.run(1050, wait=False)
    assert S.running
    with pytest.raises(RuntimeError):
        S.run(10)
    with pytest.raises(RuntimeError):
        S.one()
    S.wait()
    assert not S.running and S.step == 1050 and S.stopAtStep == 1050
    assert S._sim.calls == [100] * 10 + [50] and S._sim.threads == {"woo-scene-run"}


def test_stop_unbounded_run(S):
    S.run(wait=False)  # no stopAtStep: runs until stop()
    while S.step < 300:
        time.sleep(0.001)
    S.stop()
    S.wait()
    assert not S.running and S.step % 100 == 0 and S.step >= 300


def test_wait_raises_the_run_exception(S):
    S._fail_at = 350
    S.run(1000, wait=False)
    with pytest.raises(RuntimeError, match="injected failure"):
        S.wait()
    assert S.step == 300 and not S.running
    S.wait()  # the exception is raised once


def test_sync_and_save_while_running(S, tmp_path, monkeypatch):
    from woodem_gb300 import checkpoint
    monkeypatch.setattr(checkpoint, "contact_snapshot", lambda S: None)
    S.run(2000, wait=False)
    S.sync()  # takes the scene's lock between chunks
    path = str(tmp_path / "s.bin")
    S.save(path)
    S.wait()
    S2 = Scene.load(path)
    assert 0 <= S2.step <= 2000 and S2.step % 100 == 0 and not S2.running
    S.close()
    assert S._sim is None


def test_batch_wait_runs_the_line_scene(S, monkeypatch):
    from woodem_gb300 import batch
    S.stopAtStep = 450
    batch.wait(S)  # outside a batch: nothing
    assert S.step == 0
    monkeypatch.setattr(batch.options, "batchTable", "t.txt")
    batch.wait(S)
    assert S.step == 450 and not S.running


def test_paused_holds_the_background_run(S):
    S.run(3000, wait=False)
    with S.paused():
        step = S.step
        time.sleep(0.05)
        assert S.step == step and step % 100 == 0
    S.wait()
    assert S.step == 3000
