"""Energy tracking on the GPU against the oracle (FP64 plain mode).

Each step's contributions are summed on the device in a fixed order and the oracle sums them in
node and contact order, so the entries agree to a relative 1e-9 (accumulated over thousands of
steps), while the trajectory itself stays bitwise the oracle's: tracking energy changes no
state. The device sums are deterministic: the energies do not depend on how the steps are
split into calls."""
import numpy as np
import pytest

from woodem_gb300 import _plan, scenes, utils

from helpers import two_spheres

pytestmark = pytest.mark.gpu


def _oracle(S):
    from oracle.oracle import Oracle
    return Oracle(_plan.compile_scene(S), threads=4, deterministic=True)


def _cmp_energy(ge, oe, rtol=1e-9):
    assert set(ge) == set(oe), "entries %s (GPU) vs %s (oracle)" % (sorted(ge), sorted(oe))
    scale = max(abs(v) for v in oe.values()) if oe else 1.0
    for k in oe:
        assert ge[k] == pytest.approx(oe[k], rel=rtol, abs=1e-12 * scale), "%s: %r vs %r" % (k, ge[k], oe[k])


def _run_pair(S, chunks, steps):
    A = _plan.compile_scene(S)
    walls = A.particles["nodes"][A.particles["shape"] == 1, 0]
    O = _oracle(S)
    for _ in range(chunks):
        S.run(steps)
        O.run(steps)
        S.sync()
        nd = S.dem._nodes.soa
        o = O.nodes()
        for k in ("pos", "vel", "angVel"):
            assert np.array_equal(nd.col(k), o[k]), k
        _cmp_energy(dict(S.energy.items()), O.energy())
    return dict(S.energy.items())


def test_box_idealelpl_energies(gpu_lib):
    """Box settle (gravity, Leapfrog damping, walls, IdealElPl with friction)."""
    S = scenes.box_settle_small(n=1500, seed=0)
    S.trackEnergy = True
    e = _run_pair(S, 5, 500)
    assert {"kinetic", "grav", "nonviscDamp", "elast"} <= set(e)


def test_drum_hertz_energies_kin_split(gpu_lib):
    """Drum (Hertz with viscosity, facets, rotating caps), kinetic energy split."""
    S = scenes.hertz_drum(n=3000, seed=2, diameter=0.3, length=0.12, div=31, axDiv=6, fill_fraction=0.3)
    S.engines[0].kinSplit = True
    S.trackEnergy = True
    e = _run_pair(S, 4, 200)
    assert {"kinTrans", "kinRot", "grav", "elast", "viscN"} <= set(e) and "kinetic" not in e


@pytest.mark.parametrize("eval_stress", [False, True])
def test_periodic_energies(eval_stress, gpu_lib):
    """Periodic cell compressed and sheared (no Leapfrog energies in the first step: gradV is not
    the identity); with ContactLoop.evalStress, the work of the velocity gradient (gradV)."""
    S = scenes.periodic_shear(n=600, seed=3, fill_fraction=0.4, shear_rate=0.0)
    g = -30.0 * np.eye(3)
    g[0, 2] = 40.0
    S.cell.nextGradV = g
    S.trackEnergy = True
    S.engines[2].evalStress = eval_stress
    e = _run_pair(S, 3, 300)
    assert ("gradV" in e) == eval_stress


def test_broken_contacts_no_slip(gpu_lib):
    """IdealElPl with noSlip: the potential of a contact that breaks is booked as "broken"."""
    S = two_spheres(gap=-1e-4, v0=-0.5, r=0.05, hertz=False)
    S.engines = utils.defaultEngines(damping=0.0, dynDtPeriod=0, noSlip=True, verletDist=-0.05)
    S.dem.par[1].vel = (0.05, 0.25, 0.0)
    S.trackEnergy = True
    e = _run_pair(S, 4, 100)
    assert e["broken"] > 0


def test_granularity_and_clear(gpu_lib):
    """Energies of one call of 300 steps equal those of calls of 37 and of single steps, bitwise;
    Scene.energy.clear() restarts the accumulation."""
    out = []
    for mode in range(3):
        S = scenes.box_settle_small(n=800, seed=4)
        S.trackEnergy = True
        S.run(1400)  # contacts from about here on
        if mode == 0:
            S.run(300)
        elif mode == 1:
            for _ in range(8):
                S.run(37)
            S.run(4)
        else:
            for _ in range(300):
                S.run(1)
        out.append(dict(S.energy.items()))
        if mode == 0:
            grav = S.energy["grav"]
            S.energy.clear()
            S.run(10)
            assert abs(S.energy["grav"]) < abs(grav) and "nonviscDamp" in S.energy
        S.close()
    assert out[0] == out[1] == out[2]


@pytest.mark.parametrize("build", ["box", "drum"])
def test_fp32_mode_energies_against_fp64(build, gpu_lib):
    """Energy tracking in the FP32-force mode: the same terms, evaluated in FP64 from the FP32
    contact forces and accelerations. From the same settled state, both precisions run 300 steps
    (the FP64 path is bitwise the oracle's above); the same entries exist, and each agrees within
    1e-3 of the largest entry (the FP32 forces differ by ~1e-7 per step and the trajectories drift
    apart slowly); tracking energy changes no state of the FP32 run."""
    def mk(prec):
        if build == "box":
            S = scenes.box_settle_small(n=1500, seed=0, precision=prec)
            S.run(2500)
            S.close()
        else:
            S = scenes.hertz_drum(n=3000, seed=2, diameter=0.3, length=0.12, div=31, axDiv=6, fill_fraction=0.3, settle_steps=2000,
                                  precision=prec)
        return S

    out = {}
    for prec in ("fp64", "fp32"):
        S = mk(prec)
        S.trackEnergy = True
        S.run(300)
        out[prec] = dict(S.energy.items())
        S.sync()
        out[prec + "_pos"] = S.dem._nodes.soa.col("pos").copy()
        S.close()
    e64, e32 = out["fp64"], out["fp32"]
    assert set(e64) == set(e32) and {"kinetic", "grav", "elast"} <= set(e64)
    scale = max(abs(v) for v in e64.values())
    for k in e64:
        assert abs(e32[k] - e64[k]) <= 1e-3 * scale, "%s: %r (FP32) vs %r (FP64)" % (k, e32[k], e64[k])
    S = mk("fp32")
    S.run(300)
    S.sync()
    assert np.array_equal(S.dem._nodes.soa.col("pos"), out["fp32_pos"])  # tracking changed nothing
