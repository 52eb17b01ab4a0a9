"""Energy tracking (Scene.trackEnergy) on the CPU oracle (no GPU).

The reference has no energy test on this path; the oracle's restatement is pinned here by the
Leapfrog energy expressions (Leapfrog.cpp:52-97) evaluated step by step in Python for one
falling, damped sphere (same operations, same order: equal bit for bit), and by energy balances:
with all dissipation and work entries counted, the total of Scene.energy stays at the initial
kinetic energy (two spheres colliding elastically, with friction and with Hertz viscosity)."""
import math

import numpy as np
import pytest

import woodem_gb300 as woo
from woodem_gb300 import _plan, utils
from woodem_gb300.dem import DemField, FrictMat

from helpers import two_spheres


def _oracle(S):
    from oracle.oracle import Oracle
    return Oracle(_plan.compile_scene(S), threads=2, deterministic=True)


def test_falling_sphere_step_by_step(oracle_lib):
    """One free sphere under gravity with Leapfrog damping 0.2: grav, nonviscDamp and kinetic
    after every step equal the reference expressions evaluated in Python."""
    S = woo.core.Scene(fields=[DemField(gravity=(0, 0, -9.81))])
    m = FrictMat(density=2000, young=1e7)
    p = utils.sphere((0, 0, 1), 0.01, mat=m)
    S.dem.par.add([p])
    p.vel = (0.3, -0.1, 0.2)
    p.angVel = (1.0, 2.0, -3.0)
    S.engines = utils.defaultEngines(damping=0.2, dynDtPeriod=0)
    S.dt = 1e-4
    S.trackEnergy = True
    O = _oracle(S)
    mass, I = p.mass, p.inertia[0]
    g = np.array([0.0, 0.0, -9.81])
    v = np.array([0.3, -0.1, 0.2])
    w = np.array([1.0, 2.0, -3.0])
    dt, damping = S.dt, 0.2
    grav = damp = 0.0
    for step in range(50):
        # DemData.force: zero for a new particle, then m*g from Leapfrog's reset of the step before
        f = mass * g if step else np.zeros(3)
        t = np.zeros(3)
        # doDampingDissipation and doGravityWork with the velocities before the update
        a = (abs(v[0]) * abs(f[0]) + abs(v[1]) * abs(f[1])) + abs(v[2]) * abs(f[2])
        b = (abs(w[0]) * abs(t[0]) + abs(w[1]) * abs(t[1])) + abs(w[2]) * abs(t[2])
        damp = damp + (((a * damping) * dt) + ((b * damping) * dt))
        grav = grav + ((-((g[0] * v[0] + g[1] * v[1]) + g[2] * v[2])) * mass) * dt
        la = f / mass
        for k in range(3):
            s = f[k] * (v[k] + (0.5 * dt) * la[k])
            la[k] = la[k] * (1 - damping * (-1 if s < 0 else (1 if s > 0 else 0)))
        pv = v.copy()
        v = v + dt * la
        aa = np.zeros(3)
        w = w + dt * aa
        cv = pv + (0.5 * dt) * la
        et = (0.5 * mass) * ((cv[0] * cv[0] + cv[1] * cv[1]) + cv[2] * cv[2])
        er = 0.5 * ((w[0] * (I * w[0]) + w[1] * (I * w[1])) + w[2] * (I * w[2]))
        O.run(1)
        e = O.energy()
        assert e["grav"] == grav and e.get("nonviscDamp", 0.0) == damp and e["kinetic"] == et + er, step
        assert ("nonviscDamp" in e) == (damp != 0)  # created by the first non-zero addition
    assert sorted(e) == ["grav", "kinetic", "nonviscDamp"]


def _total_drift(S, steps, chunk):
    O = _oracle(S)
    O.run(1)
    e0 = O.energy()
    t0 = sum(e0.values())
    worst = 0.0
    for _ in range(steps // chunk):
        O.run(chunk)
        e = O.energy()
        worst = max(worst, abs(sum(e.values()) - t0) / t0)
    return worst, e


# Leapfrog takes the kinetic energy at the start of the step and the contact loop the elastic
# energy of the positions after it, so during a contact their sum is off by about omega*dt of
# the contact's energy (as in the reference, where the engines run in the same order): the
# balances below use dt = pWaveDt/100 and a 2 % bound.
def _fine(S):
    S.dt = 0.01 * utils.pWaveDt(S)
    S.trackEnergy = True
    return S


def test_elastic_collision_balance(oracle_lib):
    """Head-on FrictPhys collision without friction: kinetic + elast is conserved, and the
    spheres separate with their initial kinetic energy."""
    mat = FrictMat(density=1e3, young=1e8, ktDivKn=.2, tanPhi=0.0)
    S = _fine(two_spheres(gap=1e-6, v0=1.0, r=0.05, hertz=False, mat=mat))
    worst, e = _total_drift(S, 6000, 100)
    assert worst < 2e-2
    assert set(e) >= {"kinetic", "elast"} and "plast" not in e and e["elast"] == 0
    assert e["kinetic"] == pytest.approx(2 * 0.5 * S.dem.par[0].mass * 0.25, rel=1e-6)


def test_friction_and_hertz_dissipation(oracle_lib):
    """Oblique collisions: sliding (plast) with IdealElPl; viscous (viscN, viscT) and sliding
    dissipation with Hertz (en = 0.5). The sum of all entries stays at the initial energy."""
    mat = FrictMat(density=1e3, young=1e8, ktDivKn=.2, tanPhi=0.3)
    S = two_spheres(gap=1e-6, v0=1.0, r=0.05, hertz=False, mat=mat, offset=(0, 0, 0))
    S.dem.par[1].vel = (0.4, -0.5, 0.0)
    worst, e = _total_drift(_fine(S), 6000, 100)
    assert worst < 2e-2 and e["plast"] > 0
    S = two_spheres(gap=1e-6, v0=1.0, r=0.05, hertz=True, mat=FrictMat(density=1e3, young=1e8, ktDivKn=.2, tanPhi=0.3))
    S.engines[2].phyDisp[0].en = 0.5
    S.dem.par[1].vel = (0.2, -0.5, 0.0)
    S.engines[0].kinSplit = True
    worst, e = _total_drift(_fine(S), 9000, 100)
    assert worst < 2e-2 and e["viscN"] > 0 and "kinTrans" in e and "kinRot" in e and "kinetic" not in e


def test_periodic_gradv_work_balance(oracle_lib):
    """A periodic packing compressed and sheared by the cell, without Leapfrog damping: the work of
    the velocity gradient (ContactLoop.cpp:236-246, negative: energy put in) balances the kinetic,
    elastic and plastic entries to a few per cent once the packing is loaded."""
    from woodem_gb300 import scenes
    S = scenes.periodic_shear(n=600, seed=3, fill_fraction=0.4, shear_rate=0.0)
    g = -30.0 * np.eye(3)
    g[0, 2] = 40.0
    S.cell.nextGradV = g
    S.trackEnergy = True
    S.engines[0].damping = 0.0
    S.engines[2].evalStress = True
    O = _oracle(S)
    O.run(450)
    for _ in range(3):
        O.run(150)
        e = O.energy()
        assert e["gradV"] < 0 and abs(sum(e.values())) < 0.03 * sum(abs(v) for v in e.values())


def test_refusals():
    from woodem_gb300 import scenes
    S = scenes.box_settle_small(n=50, seed=0, precision="fp32")
    S.trackEnergy = True  # the FP32-force mode tracks energy too
    assert _plan.compile_scene(S).config["track_energy"] == 1
    from woodem_gb300.batch import Batch
    S = scenes.box_settle_small(n=50, seed=0)
    S.trackEnergy = True
    with pytest.raises(NotImplementedError, match="energy"):
        Batch([S])


def test_energy_tracker_api():
    E = woo.core.EnergyTracker()
    E["b"] = 2.0
    E.add(1.5, "a")
    E.add(0.5, "a")
    assert E.keys() == ["a", "b"] and E["a"] == 2.0 and "a" in E and len(E) == 2 and E.total() == 4.0
    assert list(E) == ["a", "b"] and E.items() == [("a", 2.0), ("b", 2.0)]
    with pytest.raises(KeyError):
        E["c"]
    E.clear()
    assert len(E) == 0 and E.relErr() == 0.0


def test_unbalanced_energy():
    S = woo.core.Scene(fields=[DemField()])
    with pytest.raises(RuntimeError):
        utils.unbalancedEnergy(S)
    S.trackEnergy = True
    assert math.isnan(utils.unbalancedEnergy(S))
    S.energy["kinetic"] = 2.0
    S.energy["elast"] = 4.0
    assert utils.unbalancedEnergy(S) == 0.5


def _sphere_on_wall():
    """py/tests/energy.py:71-76: a sphere resting deep in a wall, gravity, Leapfrog damping 0.4,
    DemField.minimalEngines (with DynDt), dt from dtSafety."""
    from woodem_gb300.core import Scene
    from woodem_gb300.dem import Wall, Sphere
    m = utils.defaultMaterial()
    return Scene(dtSafety=.9, trackEnergy=True, engines=DemField.minimalEngines(damping=.4),
                 fields=[DemField(gravity=(0, 0, -10), par=[Wall.make(0, axis=2, sense=1, mat=m),
                                                            Sphere.make((0, 0, .1), radius=.8, mat=m)])])


def test_reference_gravity_and_damping_skip(oracle_lib):
    """py/tests/energy.py:77-93 (TestLeapfrog): with DemData.gravitySkip on every node there is no
    grav entry and some nonviscDamp; with dampingSkip some grav and no nonviscDamp entry."""
    S = _sphere_on_wall()
    for n in S.dem.nodes:
        n.dem.gravitySkip = True
    S.dem.par[-1].vel = (0, 0, -1)
    O = _oracle(S)
    O.run(400)
    e = O.energy()
    assert "grav" not in e and e["nonviscDamp"] != 0.
    S = _sphere_on_wall()
    for n in S.dem.nodes:
        n.dem.dampingSkip = True
    O = _oracle(S)
    O.run(400)
    e = O.energy()
    assert e["grav"] != 0. and "nonviscDamp" not in e
