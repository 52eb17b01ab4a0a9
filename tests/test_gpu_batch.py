"""Batches of independent scenes: each scene of a batch evolves exactly as it does alone.

The kernels update a scene's particles with the same operations, in the same order, whether the
scene runs alone or packed with others (the per-particle force sum follows the scene's own ids),
so positions, velocities, forces and torques are BITWISE equal in both precision modes, and so
are the real contacts with their forces. Exception, with its tolerance: the force and torque
reported on walls with more than 64 contacts (fixed tree sum over slots that include the zero
slots of non-real contacts): relative 1e-12. (Non-real potential contacts may differ: the collider
runs whenever any scene of the batch needs it, which changes which pairs are listed, not the
physics.)
"""
import numpy as np
import pytest

from woodem_gb300 import scenes, _plan
from woodem_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def _study(precision, seed=7):
    ss, tab = scenes.batch_study(n_scenes=5, seed=seed, nmin=300, nmax=1500, precision=precision)
    return ss


def _real(c):
    r = c["real"] != 0
    return {k: v[r] for k, v in c.items()}


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_equals_alone(precision, gpu_lib):
    mix = _study(precision)
    B = Batch(mix)
    for _ in range(3):
        B.run(2500)
    B.pull()
    cmix = [_real(B.contacts(k)) for k in range(len(mix))]
    B.close()
    alone = _study(precision)
    nreal = 0
    for k, S in enumerate(alone):
        S.run(7500)
        S.sync()
        ca = _real(S._sim.contacts())
        assert S.step == mix[k].step == 7500
        A = _plan.compile_scene(S)
        walls = A.particles["nodes"][A.particles["shape"] == 1, 0]
        other = np.ones(A.n_nodes, bool)
        other[walls] = False
        for key in ("pos", "vel", "angVel", "force", "torque"):
            a = S.dem._nodes.soa.col(key)
            b = mix[k].dem._nodes.soa.col(key)
            assert np.array_equal(a[other], b[other]), "scene %d %s differs alone vs batch (max %g)" % (k, key, np.max(np.abs(a - b)))
            # walls with many contacts are summed by a tree whose grouping depends on the (zero)
            # slots of non-real potential contacts, which the batch's collider schedule changes
            np.testing.assert_allclose(a[walls], b[walls], rtol=1e-12, atol=1e-12 * max(1e-30, np.abs(a[walls]).max()))
        for key in ("id_lo", "id_hi", "id_a", "fglob"):
            assert np.array_equal(ca[key], cmix[k][key]), "scene %d real contacts differ (%s)" % (k, key)
        nreal += len(ca["id_lo"])
        S.close()
    assert nreal > 100  # the scenes have reached their floors


def test_batch_scene_parameters_differ(gpu_lib):
    """Scenes of a batch keep their own dt, damping and materials (different settling)."""
    mix = _study("fp64", seed=3)
    dts = {S.dt for S in mix}
    assert len(dts) == len(mix)
    B = Batch(mix)
    B.run(100)
    B.pull()
    for S in mix:
        assert S.time == pytest.approx(100 * S.dt)
    B.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_with_dyndt_equals_alone(precision, gpu_lib):
    """The stock engine list with DynDt (utils.defaultEngines appends DynDt(stepPeriod=100)) in a
    batch: every scene keeps its own DynDt counters and Scene.dt, which change at the steps where
    they change with the scene alone; states, dt, time and counters equal the scene run alone
    (bitwise in both modes; walls with many contacts as in test_batch_equals_alone)."""
    from woodem_gb300.dem import DynDt

    def study():
        ss = _study(precision, seed=11)
        for q, S in enumerate(ss):
            S.engines = list(S.engines) + [DynDt(stepPeriod=(50, 100, 70, 100, 30)[q], maxRelInc=2e-2)]
        return ss

    mix = study()
    B = Batch(mix)
    for _ in range(3):
        B.run(1000)
    B.close()
    alone = study()
    changed = 0
    for k, S in enumerate(alone):
        S.run(3000)
        S.sync()
        assert S.step == mix[k].step == 3000
        assert S.dt == mix[k].dt and S.time == mix[k].time, "scene %d dt/time alone vs batch" % k
        ea, eb = S.engines[-1], mix[k].engines[-1]
        assert (ea.nDone, ea.stepLast, ea.stepPrev) == (eb.nDone, eb.stepLast, eb.stepPrev)
        changed += S.dt != study()[k].dt
        A = _plan.compile_scene(S)
        walls = A.particles["nodes"][A.particles["shape"] == 1, 0]
        other = np.ones(A.n_nodes, bool)
        other[walls] = False
        for key in ("pos", "vel", "angVel"):
            a, b = S.dem._nodes.soa.col(key), mix[k].dem._nodes.soa.col(key)
            assert np.array_equal(a[other], b[other]), "scene %d %s differs alone vs batch" % (k, key)
        S.close()
    assert changed >= 3  # DynDt changed dt in most scenes
