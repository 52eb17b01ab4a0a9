"""Serving: jobs admitted while others run give the same results as the jobs run alone.

Box-settle jobs of different sizes and step counts arrive at different ticks and are loaded into
the slots of one device simulation while other slots keep running (and are reloaded when their
jobs end); a periodic job runs beside them as its own simulation. Each job's final state is
compared with the same job run alone: BITWISE for positions, velocities, angular velocities and
the forces and torques of spheres; walls with more than 64 contacts report a tree sum whose
grouping depends on the zero slots of non-real contacts: relative 1e-12.
"""
import numpy as np
import pytest

from woodem_gb300 import scenes, _plan
from woodem_gb300.serve import SlotPool, Server, Job

pytestmark = pytest.mark.gpu


def _box(n, seed, precision):
    r = 3e-3 + 1e-3 * (seed % 3)
    return scenes.box_settle_scaled(n, r, seed=seed, young=1e7 * (1 + seed % 4), tanPhi=0.3 + 0.1 * (seed % 3),
                                    damping=0.1 * (seed % 4), precision=precision)


def _peri(n, seed, precision):
    S = scenes.periodic_shear(n=n, seed=seed, fill_fraction=0.4, shear_rate=0.0, precision=precision)
    g = -10.0 * np.eye(3)
    g[0, 2] = 20.0
    S.cell.nextGradV = g
    return S


def _alone(job_build, steps):
    S = job_build()
    S.run(steps)
    S.sync()
    out = {k: S.dem._nodes.soa.col(k).copy() for k in ("pos", "vel", "angVel", "force", "torque")}
    A = _plan.compile_scene(S)
    walls = A.particles["nodes"][A.particles["shape"] == 1, 0]
    S.close()
    return out, walls


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_jobs_same_alone_and_in_the_mix(precision, gpu_lib):
    specs = [(500, 11, 2000, 0), (1400, 12, 1500, 0), (800, 13, 2500, 1), (2200, 14, 1200, 3), (600, 15, 1800, 4)]
    jobs = []
    for jid, (n, seed, steps, tick) in enumerate(specs):
        jobs.append(Job(jid, (lambda n=n, seed=seed: _box(n, seed, precision)), n + 6, steps, tick))
    jobs.append(Job(len(jobs), (lambda: _peri(400, 21, precision)), 400, 300, 2, periodic=True))
    jobs.sort(key=lambda j: j.arrival)
    template = _plan.compile_scene(_box(500, 11, precision))
    pool = SlotPool([1600, 1600, 2400], precision=precision, template=template)
    srv = Server(pool, tick=500, keep_results=True, clock="ticks")
    done = srv.run(jobs)
    pool.close()
    assert len(done) == len(jobs)
    loaded_late = [j for j in done if not j.periodic and j.start > 0]
    assert loaded_late  # some jobs joined slots while others were running
    for j in done:
        if j.periodic:
            S = j.build()
            S.run(j.steps)
            S.sync()
            for k in ("pos", "vel", "angVel", "force", "torque"):
                assert np.array_equal(S.dem._nodes.soa.col(k), j.result[k])
            S.close()
            continue
        ref, walls = _alone(j.build, j.steps)
        other = np.ones(len(ref["pos"]), bool)
        other[walls] = False
        for k in ("pos", "vel", "angVel", "force", "torque"):
            a, b = ref[k], j.result[k]
            assert np.array_equal(a[other], b[other]), "job %d %s differs alone vs served (max %g)" % (j.id, k, np.max(np.abs(a - b)))
            np.testing.assert_allclose(a[walls], b[walls], rtol=1e-12, atol=1e-12 * max(1e-30, np.abs(a[walls]).max()))
