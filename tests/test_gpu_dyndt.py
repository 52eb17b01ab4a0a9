"""DynDt on the GPU against the oracle, bitwise (FP64 plain mode).

DynDt runs after ContactLoop (pkg/dem/DynDt.cpp:93-113): the contact stiffnesses are summed on
the device per node in the order of Particle.contacts, the host applies the timestep rule, and
the new dt takes effect from the next step on. The run's chunks of queued steps end at the steps
where DynDt is due, so dt changes exactly where the reference changes it: positions,
velocities, forces, Scene.dt and the engine's counters must equal the oracle's bitwise."""
import math

import numpy as np
import pytest

from woodem_gb300 import _plan, scenes
from woodem_gb300.dem import DynDt

pytestmark = pytest.mark.gpu


def _oracle(S):
    from oracle.oracle import Oracle
    return Oracle(_plan.compile_scene(S), threads=4, deterministic=True)


def _with_dyndt(S, **kw):
    S.engines = list(S.engines) + [DynDt(**kw)]
    return S


def _compare(S, O, walls):
    S.sync()
    nd = S.dem._nodes.soa
    o = O.nodes()
    for k in ("pos", "vel", "angVel"):
        assert np.array_equal(nd.col(k), o[k]), "%s differs (max %g)" % (k, np.max(np.abs(nd.col(k) - o[k])))
    for k in ("force", "torque"):
        assert np.array_equal(nd.col(k), o[k]), "%s differs" % k
    g, od = S._sim.dyndt(), O.dyndt()
    assert g.dt == od.dt and S.dt == od.dt, "dt %r (GPU) vs %r (oracle)" % (g.dt, od.dt)
    assert (g.n_done, g.step_last, g.step_prev, g.n_evals) == (od.n_done, od.step_last, od.step_prev, od.n_evals)
    assert g.crit_dt == od.crit_dt or (math.isinf(g.crit_dt) and math.isinf(od.crit_dt))
    e = [x for x in S.engines if isinstance(x, DynDt)][0]
    assert (e.nDone, e.stepLast, e.stepPrev) == (od.n_done, od.step_last, od.step_prev)


def _run_pair(S, chunks, steps):
    A = _plan.compile_scene(S)
    walls = A.particles["nodes"][A.particles["shape"] == 1, 0]
    O = _oracle(S)
    dts = [S.dt]
    for _ in range(chunks):
        S.run(steps)
        O.run(steps)
        _compare(S, O, walls)
        dts.append(S.dt)
    return dts


def test_drum_hertz(gpu_lib):
    """Rotating drum, Hertz contacts from the first step, facets and walls: DynDt every 25 steps."""
    S = _with_dyndt(scenes.hertz_drum(n=3000, seed=2, diameter=0.3, length=0.12, div=31, axDiv=6, fill_fraction=0.3),
                    stepPeriod=25, maxRelInc=5e-3)
    dts = _run_pair(S, 6, 110)
    assert len(set(dts)) > 3  # dt changed several times


def test_box_idealelpl(gpu_lib):
    """Box settle (IdealElPl, walls): DynDt every 100 steps, contacts from about step 1500 on."""
    S = _with_dyndt(scenes.box_settle_small(n=1500, seed=0), stepPeriod=100, maxRelInc=1e-2)
    dts = _run_pair(S, 5, 500)
    assert len(set(dts)) > 2


def test_periodic_virt_period(gpu_lib):
    """Periodic cell compressed and sheared, DynDt by simulation time (virtPeriod)."""
    S = scenes.periodic_shear(n=600, seed=3, fill_fraction=0.4, shear_rate=0.0)
    g = -30.0 * np.eye(3)
    g[0, 2] = 40.0
    S.cell.nextGradV = g
    _with_dyndt(S, stepPeriod=0, virtPeriod=37.5 * S.dt, maxRelInc=1e-2)
    _run_pair(S, 4, 300)


def test_dry_run_and_granularity(gpu_lib):
    """Dry run leaves Scene.dt alone; one call of 400 steps, calls of 37 steps and single steps
    give the same state and dt."""
    S = _with_dyndt(scenes.hertz_drum(n=1500, seed=5, diameter=0.25, length=0.1, div=25, axDiv=5, fill_fraction=0.3),
                    stepPeriod=30, dryRun=True)
    dt0 = S.dt
    _run_pair(S, 2, 100)
    assert S.dt == dt0 and math.isfinite(S.engines[-1].dt)
    out = []
    for mode in range(3):
        S = _with_dyndt(scenes.hertz_drum(n=1500, seed=5, diameter=0.25, length=0.1, div=25, axDiv=5, fill_fraction=0.3),
                        stepPeriod=30, maxRelInc=1e-2)
        if mode == 0:
            S.run(400)
        elif mode == 1:
            for _ in range(10):
                S.run(37)
            S.run(30)
        else:
            for _ in range(400):
                S.run(1)
        S.sync()
        out.append((S.dt, {k: S.dem._nodes.soa.col(k).copy() for k in ("pos", "vel", "angVel")}))
        S.close()
    for q in (1, 2):
        assert out[q][0] == out[0][0]
        for k in out[0][1]:
            assert np.array_equal(out[q][1][k], out[0][1][k]), k


def test_dt_set_between_runs(gpu_lib):
    """Scene.dt and Scene.nextDt set between runs take effect (nextDt after the next step)."""
    S = scenes.box_settle_small(n=300, seed=1)
    dt0 = S.dt
    S.run(10)
    S.nextDt = 0.5 * dt0
    S.run(1)
    assert S.dt == 0.5 * dt0 and math.isnan(S.nextDt)
    t = S.time
    S.dt = 0.25 * dt0
    S.run(4)
    assert S.dt == 0.25 * dt0 and S.time == pytest.approx(t + 4 * 0.25 * dt0, rel=1e-12)


@pytest.mark.parametrize("build", ["drum", "box"])
def test_fp32_mode_against_fp64(build, gpu_lib):
    """DynDt in the FP32-force mode: the stiffnesses come from the FP32 contact state (kn, kt and
    the contact normal rounded to FP32; L6Geom.lens from the current overlap). From the same state
    both precisions run 300 steps with DynDt every 25 steps (the FP64 path is bitwise the
    oracle's, above). The first evaluation, on states that are still equal up to the FP32
    rounding of one step, gives the same critical timestep within 1e-3 relative (the rotational
    stiffness lens^2 kt takes the current overlap instead of the first step's: uN/2 against the
    radius, ~1e-4 in a settled bed); later evaluations follow trajectories that part: in the drum
    (a bed at rest) the critical timestep and Scene.dt agree within 5 %, in the settling box (the
    minimum over the nodes jumps to whichever particle holds the stiffest set of contacts at that
    step) within a factor 1.5; the activation counters agree exactly."""
    if build == "drum":
        mk = lambda prec: _with_dyndt(scenes.hertz_drum(n=3000, seed=2, diameter=0.3, length=0.12, div=31, axDiv=6,
                                                        fill_fraction=0.3, settle_steps=3000, precision=prec),
                                      stepPeriod=25, maxRelInc=5e-3)
    else:
        def mk(prec):
            S = scenes.box_settle_small(n=1500, seed=0, precision=prec)
            S.run(3000)
            S.close()
            return _with_dyndt(S, stepPeriod=25, maxRelInc=1e-2)
    S64, S32 = mk("fp64"), mk("fp32")
    crit = {}
    for S in (S64, S32):
        dts = []
        for _ in range(12):
            S.run(25)
            dts.append((S.dt, S._sim.dyndt().crit_dt))
        crit[S.gpu.precision] = dts
        e = [x for x in S.engines if isinstance(x, DynDt)][0]
        crit[S.gpu.precision + "_counters"] = (e.nDone, e.stepLast, e.stepPrev)
    a, b = np.array(crit["fp64"]), np.array(crit["fp32"])
    assert np.all(np.isfinite(a[:, 1])) and len(set(a[:, 0])) > 2
    assert b[0, 1] == pytest.approx(a[0, 1], rel=1e-3)
    if build == "drum":
        np.testing.assert_allclose(b[:, 1], a[:, 1], rtol=5e-2)
        np.testing.assert_allclose(b[:, 0], a[:, 0], rtol=5e-2)
    else:
        assert np.all(np.abs(np.log(b / a)) <= np.log(1.5))
    assert crit["fp64_counters"] == crit["fp32_counters"]
