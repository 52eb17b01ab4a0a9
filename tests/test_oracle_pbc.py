"""Known-answer tests of the periodic cell, restated from the reference's py/tests/pbc.py against
the oracle (no GPU): cell kinematics under a velocity gradient (pbc.py:35-52) and the homothetic
corrections of particle velocity and position (pbc.py:70-87).

Setup of pbc.py:18-33: a 2.5 x 2.5 x 3 periodic cell, sphere 0 (r 0.5) at (1, 1, 1), sphere 1
(r 0.5) one unit along y and ten cells along z from it, moving with (0, 0, 5);
nextGradV = diag(0, 0, -1).
"""
import numpy as np
import pytest

import woodem_gb300 as woo
from woodem_gb300 import utils, _plan
from woodem_gb300.core import Cell
from woodem_gb300.dem import DemField, FrictMat

INIT_VEL = np.array([0, 0, 5.0])


def pbc_scene(homo, dt):
    S = woo.core.Scene(fields=[DemField(gravity=(0, 0, 0))])
    S.periodic = True
    S.cell.setBox(2.5, 2.5, 3)
    mat = FrictMat(density=1e3, young=1e7, ktDivKn=.2, tanPhi=.5)
    s0 = utils.sphere((1, 1, 1), .5, mat=mat)
    init_pos = np.array([1, 1 + 1.0, 1 + 10 * 3.0])
    s1 = utils.sphere(init_pos, .5, mat=mat)
    S.dem.par.add([s0, s1])
    s1.vel = tuple(INIT_VEL)
    S.engines = utils.defaultEngines(damping=0, dynDtPeriod=0, verletDist=-0.05)
    S.cell.nextGradV = np.diag([0, 0, -1.0])
    S.cell.homoDeform = homo
    S.dt = dt
    return S, init_pos


def oracle_of(S):
    from oracle.oracle import Oracle
    return Oracle(_plan.compile_scene(S))


def test_velgrad_integrates_cell(oracle_lib):
    """pbc.py:35-52 (HomoVel2): hSize and trsf follow hSize += dt*gradV*hSize, trsf += dt*gradV*trsf."""
    S, _ = pbc_scene(Cell.HomoVel2, 1e-3)
    O = oracle_of(S)
    hsize = np.diag([2.5, 2.5, 3.0])
    trsf = np.eye(3)
    gradv = np.zeros((3, 3))
    for _ in range(10):
        hsize = hsize + S.dt * gradv.dot(hsize)
        trsf = trsf + S.dt * gradv.dot(trsf)
        O.run(1)
        gradv = O.cell()[2]
    hs, tr, _ = O.cell()
    np.testing.assert_allclose(hs, hsize, atol=1e-7)
    np.testing.assert_allclose(tr, trsf, atol=1e-7)


def test_homothetic_resize_vel(oracle_lib):
    """pbc.py:70-81 (HomoVel): after one step vel_z = initVel_z + initPos_z * gradV_zz."""
    S, init_pos = pbc_scene(Cell.HomoVel, 1e-5)
    O = oracle_of(S)
    O.run(1)  # nextGradV becomes gradV at the end of this step
    O.run(1)
    v = O.nodes()["vel"][1]
    gzz = O.cell()[2][2, 2]
    assert gzz == -1.0
    # the second step applied the homothetic velocity correction once (positions moved by dt*vel)
    assert v[2] == pytest.approx(INIT_VEL[2] + init_pos[2] * gzz, abs=1e-3)


def test_homothetic_resize_pos(oracle_lib):
    """pbc.py:82-87 (HomoPos): velocity untouched, pos_z += pos_z * gradV_zz * dt."""
    S, init_pos = pbc_scene(Cell.HomoPos, 1e-5)
    O = oracle_of(S)
    O.run(1)
    p_before = O.nodes()["pos"][1].copy()
    O.run(1)
    n = O.nodes()
    assert n["vel"][1][2] == pytest.approx(INIT_VEL[2], rel=1e-12)
    expect = p_before[2] + p_before[2] * (-1.0) * S.dt + INIT_VEL[2] * S.dt
    assert n["pos"][1][2] == pytest.approx(expect, rel=1e-12)


def test_cross_cell_contact_exists(oracle_lib):
    """The pair of pbc.py (ten cells apart along z, touching through the periodic image) is a
    contact of the periodic collider, with cell distance 10 along z for the (0, 1) orientation."""
    S, _ = pbc_scene(Cell.HomoGradV2, 1e-10)
    O = oracle_of(S)
    O.run(1)
    c = O.contacts()
    assert len(c["id_lo"]) == 1
    assert tuple(c["cell_dist"][0]) == (0, 0, -10)


def _overlap_peri(mn, mx, a, b, size):
    """InsertionSortCollider::spatialOverlapPeri (pkg/dem/InsertionSortCollider.cpp:903-957)."""
    per = [0, 0, 0]
    for ax in range(3):
        dim = size[ax]
        m1, m2 = mn[a, ax], mn[b, ax]
        rel = lambda x, x0: ((x - x0) / dim - np.floor((x - x0) / dim)) * dim
        w = m2 if rel(m1, m2) < rel(m2, m1) else m1

        def wrap(x):
            xn = (x - w) / dim
            p = np.floor(xn)
            return w + (xn - p) * dim, int(p)
        (mn1, p1), (mx1, _) = wrap(mn[a, ax]), wrap(mx[a, ax])
        (mn2, p2), (mx2, _) = wrap(mn[b, ax]), wrap(mx[b, ax])
        per[ax] = p1 - p2
        if not (mn1 <= mx2 and mx1 >= mn2):
            return False, per
    return True, per


def fast_periodic_scene(seed=44, n=40, L=0.1, r=0.006, vmax=3.0):
    """n spheres of radius r at seeded random places in an L-cube periodic cell, moving with
    seeded random velocities of up to vmax per axis (a full collider run at every step)."""
    rng = np.random.default_rng(seed)
    S = woo.core.Scene(fields=[DemField(gravity=(0, 0, 0))])
    S.periodic = True
    S.cell.setBox(L, L, L)
    mat = FrictMat(density=1e3, young=1e5, ktDivKn=.2, tanPhi=.5)
    ps = [utils.sphere(tuple(p), r, mat=mat) for p in rng.uniform(0, L, (n, 3))]
    S.dem.par.add(ps)
    for p in ps:
        p.vel = tuple(rng.uniform(-vmax, vmax, 3))
    S.engines = utils.defaultEngines(damping=0, dynDtPeriod=0, verletDist=-0.05)
    S.dt = 1e-4
    return S


def test_periodic_insertion_sort_can_miss_an_overlap(oracle_lib):
    """The reference's periodic insertion sort (InsertionSortCollider.cpp:718-791, serial form)
    makes one pass over each circular bound list; a pass can leave an inversion next to the wrap
    point, and the overlap it hides is reported only at a later inversion of that pair. The oracle
    restates the pass; in this 40-sphere periodic cell (seeded fast random motion, a full run every
    step) the boxes of spheres 1 and 28 overlap across the z boundary after step 26 while the
    contact container does not hold the pair. The GPU broad phase computes the exact overlap set
    and holds it (its parity tests accept exactly such pairs)."""
    from oracle.oracle import Oracle
    S = fast_periodic_scene()
    A = _plan.compile_scene(S)
    O = Oracle(A, threads=1, deterministic=True)
    O.run(26)
    mn, mx = O.aabbs(A.n_particles)
    size = np.linalg.norm(O.cell()[0], axis=0)
    c = O.contacts()
    held = set(zip(c["id_lo"].tolist(), c["id_hi"].tolist()))
    assert O.stats().n_full_runs == 26
    ov, per = _overlap_peri(mn, mx, 1, 28, size)
    assert ov and per == [0, 0, 1] and (1, 28) not in held
    # every other overlap is held
    missing = [(a, b) for a in range(40) for b in range(a + 1, 40) if _overlap_peri(mn, mx, a, b, size)[0] and (a, b) not in held]
    assert missing == [(1, 28)]
    O.close()
