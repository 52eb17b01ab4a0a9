"""DynDt on the CPU oracle and its host-side compilation (no GPU).

The reference has no test of DynDt; the oracle's restatement (pkg/dem/DynDt.cpp:17-113 with the
PeriodicEngine activation of core/Engine.cpp:169-194) is pinned here against the closed form of
a head-on contact of two equal spheres, against the activation rule restated step by step, and
against the dt update rule evaluated in Python with the same libm."""
import math

import pytest

from woodem_gb300 import _plan, scenes, utils
from woodem_gb300.dem import DynDt

from helpers import two_spheres


def _oracle(S, threads=2):
    from oracle.oracle import Oracle
    return Oracle(_plan.compile_scene(S), threads=threads, deterministic=True)


def _with_dyndt(S, **kw):
    S.engines = list(S.engines) + [DynDt(**kw)]
    return S


def test_two_spheres_closed_form(oracle_lib):
    """FrictPhys contact along y of two equal free spheres: ktrans = (kt, kn, kt), krot =
    lens^2 kt (1, 0, 1), so the critical dt is sqrt(2 m / kn) with kn = E pi r^2 / (2 lens)
    (FrictMat.cpp:20-44), lens = r + uN0/2 ~ r."""
    r, E, rho = 0.05, 1e8, 1e3
    S = _with_dyndt(two_spheres(gap=-1e-6, v0=1e-3, r=r, hertz=False), stepPeriod=1, maxRelInc=1e-4)
    dt0 = S.dt
    O = _oracle(S)
    O.run(3)
    st = O.dyndt()
    assert st.n_evals == 3 and st.n_done == 3 and st.step_last == 2 and st.step_prev == 1
    m = rho * 4 / 3 * math.pi * r ** 3
    kn = E * math.pi * r * r / (2 * r)
    assert st.crit_dt == pytest.approx(math.sqrt(2 * m / kn), rel=1e-4)
    # nextDt = min(crDt*dtSafety, dt*(1+maxRelInc)^(steps since the previous run)); crDt is far
    # above dt here, so dt grows by the factor at every step
    dt = dt0
    for n in (0, 1, 1):
        dt = min(st.crit_dt * 0.9, dt * math.pow(1 + 1e-4, n))
    assert st.dt == dt


def _activation(steps, start, dt, period=0, modulo=True, init_run=True, n_do=-1, virt=0.0):
    """The PeriodicEngine rule, step by step: returns (nDone, stepLast, stepPrev, steps run)."""
    n_done, last, prev, vlast, ran = 0, -1, -1, float("nan"), []
    t = 0.0
    for s in range(start, start + steps):
        init = last < 0
        if init:
            vlast, last = t, s
        due = (virt > 0 and t - vlast >= virt) or (period > 0 and ((s - last >= period) or (modulo and s % period == 0)))
        if (n_do < 0 or n_done < n_do) and due:
            vlast, prev, last = t, last, s
            if not (init and not init_run):
                n_done += 1
                ran.append(s)
        t += dt
    return n_done, last, prev, ran


@pytest.mark.parametrize("kw,start", [
    (dict(stepPeriod=10), 0),
    (dict(stepPeriod=10, initRun=False), 0),
    (dict(stepPeriod=10), 7),
    (dict(stepPeriod=10, stepModulo=False), 7),
    (dict(stepPeriod=6, nDo=3), 0),
    (dict(stepPeriod=0, virtPeriod=0), 0),
])
def test_activation_counters(kw, start, oracle_lib):
    """Dry-run DynDt (dt never changes) on a small box settle: the counters follow the rule."""
    S = scenes.box_settle_small(n=200, seed=3)
    S.step = start
    _with_dyndt(S, dryRun=True, **kw)
    if kw.get("stepPeriod") == 0:
        kw = dict(kw, virtPeriod=7.5 * S.dt)
        S.engines[-1].virtPeriod = kw["virtPeriod"]
    O = _oracle(S)
    O.run(40)
    st = O.dyndt()
    n_done, last, prev, ran = _activation(40, start, S.dt, period=kw.get("stepPeriod", 1), modulo=kw.get("stepModulo", True),
                                          init_run=kw.get("initRun", True), n_do=kw.get("nDo", -1), virt=kw.get("virtPeriod", 0.0))
    assert (st.n_done, st.step_last, st.step_prev) == (n_done, last, prev)
    assert st.n_evals == len(ran) and st.dt == S.dt


def _drum(**kw):
    return _with_dyndt(scenes.hertz_drum(n=800, seed=1, diameter=0.2, length=0.08, div=17, axDiv=4, fill_fraction=0.3), **kw)


def test_dry_run_and_dt_update(oracle_lib):
    """A drum (Hertz contacts from the first step): with dryRun only DynDt.dt moves; otherwise
    Scene.dt grows by (1+maxRelInc)^50 per run of DynDt until dtSafety times the critical dt caps it."""
    S = _drum(stepPeriod=50, maxRelInc=1e-2, dryRun=True)
    O = _oracle(S)
    O.run(301)
    st = O.dyndt()
    assert st.dt == S.dt and math.isfinite(st.crit_dt) and st.n_done == 7
    assert st.dyndt_dt == min(st.crit_dt * S.dtSafety, S.dt * math.pow(1.01, 50))
    S2 = _drum(stepPeriod=50, maxRelInc=1e-2)
    O2 = _oracle(S2)
    dt = S2.dt
    for k in range(6):
        O2.run(50 if k else 1)
        st2 = O2.dyndt()
        dt = min(st2.crit_dt * S2.dtSafety, dt * math.pow(1.01, 50 if k else 0))
        assert st2.dt == dt and math.isnan(st2.next_dt)
    assert st2.dt > S2.dt


def test_compile_refusals_and_automatic_dt():
    S = _with_dyndt(scenes.box_settle_small(n=50, seed=0, precision="fp32"), stepPeriod=10)
    assert _plan.compile_scene(S).config["dyndt"] == 1  # the FP32-force mode runs DynDt too
    S = _with_dyndt(scenes.box_settle_small(n=50, seed=0), stepPeriod=10, realPeriod=1.0)
    with pytest.raises(NotImplementedError, match="realPeriod"):
        _plan.compile_scene(S)
    S = _with_dyndt(scenes.box_settle_small(n=50, seed=0), stepPeriod=10, maxRelInc=1e-20)
    with pytest.raises(ValueError, match="maxRelInc"):
        _plan.compile_scene(S)
    S = scenes.hertz_drum(n=300, seed=1, diameter=0.2, length=0.08, div=17, axDiv=4, fill_fraction=0.3)
    fac = [p for p in S.dem.par if type(p.shape).__name__ == "Facet"][0]
    fac.shape.nodes[0].dem.blocked = ""
    _with_dyndt(S, stepPeriod=10)
    with pytest.raises(NotImplementedError, match="facet nodes"):
        _plan.compile_scene(S)
    from woodem_gb300.batch import Batch
    S = _with_dyndt(scenes.box_settle_small(n=50, seed=0), stepPeriod=10)
    S.trackEnergy = True  # DynDt runs in a Batch; energy tracking does not
    with pytest.raises(NotImplementedError, match="energy"):
        Batch([S])
    # Scene.dt unset: dtSafety * pWaveDt, as Scene::doOneStep does before the first step
    S = scenes.box_settle_small(n=50, seed=0)
    S.dt = float("nan")
    A = _plan.compile_scene(S)
    assert S.dt == S.dtSafety * utils.pWaveDt(S) and A.config["dt"] == S.dt
