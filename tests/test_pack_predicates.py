"""Packing predicates, SpherePack.filtered and the regular packings of woo.pack
(py/_packPredicates.cpp:51-395, py/pack.py:323-391), checked against their defining inequalities."""
import itertools
import math

import numpy as np
import pytest

from woodem_gb300 import pack


def test_predicates_and_padding():
    box = pack.inAlignedBox((0, 0, 0), (1, 2, 3))
    assert box((0.5, 1, 1.5)) and box((0.5, 1, 1.5), 0.5) and not box((0.5, 1, 1.5), 0.6)
    assert np.allclose(box.center(), (0.5, 1, 1.5)) and np.allclose(box.dim(), (1, 2, 3))
    sph = pack.inSphere((0, 0, 0), 1.0)
    # the reference's test subtracts the padding on both sides: the centre decides
    assert sph((0.99, 0, 0), 0.5) and not sph((1.01, 0, 0))
    cyl = pack.inCylinder((0, 0, 0), (0, 0, 2), 0.5)
    assert cyl((0.3, 0, 1)) and not cyl((0.3, 0, 1), 0.25) and not cyl((0, 0, 0.1), 0.2) and cyl((0, 0, 0.3), 0.2)
    mn, mx = cyl.aabb()
    assert np.allclose(mn, (-0.5, -0.5, 0)) and np.allclose(mx, (0.5, 0.5, 2))
    tilted = pack.inCylinder((0, 0, 0), (1, 1, 0), 0.1)
    mn, mx = tilted.aabb()
    assert np.allclose(mn, (-0.1 / math.sqrt(2), -0.1 / math.sqrt(2), -0.1))
    hs = pack.inAlignedHalfspace(2, 1.0)
    assert hs((0, 0, 0.5), 0.4) and not hs((0, 0, 0.5), 0.5)
    assert not pack.inAlignedHalfspace(2, 1.0, lower=False)((0, 0, 1.5), 0.5)
    ar = pack.inAxisRange(0, (0, 1))
    assert ar((0.5, 9, 9), 0.5) and not ar((0.5, 9, 9), 0.51)
    with pytest.raises(RuntimeError):
        pack.inAxisRange(3, (0, 1))


def test_predicate_booleans():
    A = pack.inAlignedBox((0, 0, 0), (2, 2, 2))
    B = pack.inSphere((2, 1, 1), 1.0)
    for pt in itertools.product(np.linspace(-0.5, 3.5, 9), repeat=3):
        a, b = A(pt, 0.1), B(pt, 0.1)
        assert (A | B)(pt, 0.1) == (a or b)
        assert (A & B)(pt, 0.1) == (a and b)
        assert (A ^ B)(pt, 0.1) == (a != b)
        assert (A - B)(pt, 0.1) == (a and not B(pt, -0.1))
    mn, mx = (A & B).aabb()
    assert np.allclose(mn, (1, 0, 0)) and np.allclose(mx, (2, 2, 2))
    mn, mx = (A | B).aabb()
    assert np.allclose(mn, (0, 0, 0)) and np.allclose(mx, (3, 2, 2))


def test_filtered_recenter_and_clumps():
    sp = pack.SpherePack()
    for i in range(10):
        sp.add((i, 0, 0), 0.4)
    f = sp.filtered(pack.inAxisRange(0, (2.5, 6.5)))  # infinite predicate: no recentring
    assert sorted(c[0] for c, r in f) == [3, 4, 5, 6]
    f = sp.filtered(pack.inAlignedBox((100, -1, -1), (104, 1, 1)))  # moved onto the box centre
    assert sorted(c[0] for c, r in f) == [100.5, 101.5, 102.5, 103.5]
    f = sp.filtered(pack.inAlignedBox((0, -1, -1), (4, 1, 1)), recenter=False)  # centres in [0.4, 3.6]
    assert sorted(c[0] for c, r in f) == [1, 2, 3]
    cl = pack.SpherePack()
    cl.add((0, 0, 0), 0.4, 0)
    cl.add((1, 0, 0), 0.4, 0)
    cl.add((5, 0, 0), 0.4, 1)
    cl.add((6, 0, 0), 0.4, 1)
    f = cl.filtered(pack.inAxisRange(0, (-1, 5.5)))  # clump 1 loses a sphere: all of it goes
    assert [k for _, _, k in f.pack] == [0, 0]


@pytest.mark.parametrize("gap", [0.0, 0.01])
def test_regular_ortho_and_hexa(gap):
    r = 0.05
    pred = pack.inAlignedBox((0, 0, 0), (0.5, 0.4, 0.6)) - pack.inSphere((0.25, 0.2, 0.3), 0.1)
    ortho = pack.regularOrtho(pred, r, gap)
    hexa = pack.regularHexa(pred, r, gap)
    a = 2 * r + gap
    # the reference's odd layers sit (0, a·√3/4) off the even ones, a·√6/3 higher: some centres
    # of adjacent layers come to a·√(3/16+2/3) ≈ 0.924·a (a property of py/pack.py:334-351 kept here)
    for ss, expect in ((ortho, a), (hexa, a * math.sqrt(3 / 16. + 2 / 3.))):
        pos = np.array([s.pos for s in ss])
        assert len(pos) > 20
        assert all(pred(p, r) for p in pos)
        d = np.linalg.norm(pos[:, None, :] - pos[None, :, :], axis=-1) + np.eye(len(pos)) * 1e9
        assert d.min() == pytest.approx(expect, rel=1e-9)
        assert all(s.shape.radius == r for s in ss)
    # orthogonal grid: centres at min+r+k·a, below max-r (numpy.arange semantics)
    xx = np.arange(r, 0.5 - r, a)
    assert set(np.round(np.array([s.pos for s in ortho])[:, 0], 12)) <= set(np.round(xx, 12))
    # the hexagonal packing is denser than the orthogonal one in the same solid
    assert len(hexa) > len(ortho)
    with pytest.raises(ValueError):
        pack.regularOrtho(pack.inAlignedHalfspace(2, 0.0), r, gap)


def test_regular_packing_runs_as_scene():
    """Spheres of regularHexa go into a scene like those of utils.sphere."""
    import woodem_gb300 as woo
    from woodem_gb300.core import Scene
    from woodem_gb300.dem import DemField
    S = Scene(fields=[DemField(gravity=(0, 0, -9.81))])
    ids = S.dem.par.add(pack.regularHexa(pack.inCylinder((0, 0, 0), (0, 0, 0.2), 0.1), 0.01, 0.0))
    assert len(ids) == len(S.dem.par) > 50
    S.engines = woo.utils.defaultEngines(damping=0.3, dynDtPeriod=0)
    from woodem_gb300 import _plan
    A = _plan.compile_scene(S)
    assert len(A.particles["shape"]) == len(ids)


def test_from_simulation_round_trip():
    """SpherePack.toSimulation then fromSimulation gives the spheres and the periodic cell back;
    walls are left out and a sheared cell is refused."""
    from woodem_gb300 import utils
    from woodem_gb300.core import Scene
    from woodem_gb300.dem import DemField
    sp = pack.SpherePack()
    sp.makeCloud((0, 0, 0), (0.1, 0.1, 0.1), rMean=0.005, periodic=True, seed=3)
    S = Scene(fields=[DemField()])
    sp.toSimulation(S)
    S.dem.par.add(utils.wall(0.0, axis=2))
    back = pack.SpherePack().fromSimulation(S)
    assert len(back) == len(sp)
    c0, r0 = sp.toCcRr()
    c1, r1 = back.toCcRr()
    assert np.array_equal(c0, c1) and np.array_equal(r0, r1) and np.array_equal(back.cellSize, sp.cellSize)
    h = np.array(S.cell.hSize)
    h[0, 2] = 0.01
    S.cell.hSize = h
    with pytest.raises(RuntimeError):
        pack.SpherePack().fromSimulation(S)
