"""woo.pack.SpherePack counterpart (lib/sphere-pack/SpherePack.cpp, py/pack.py): makeCloud in its
radius modes (mean and fuzz, count and porosity, size distribution by number and by mass), the
non-overlap and containment of the packings (box and periodic), toSimulation, the text file
format, cellRepeat and psd."""
import math

import numpy as np
import pytest

import woodem_gb300 as woo
from woodem_gb300 import pack


def _no_overlap(sp, periodic=None):
    cc, rr = sp.toCcRr()
    from scipy.spatial import cKDTree
    L = periodic
    t = cKDTree(np.mod(cc, L) if L is not None else cc, boxsize=L)
    for i, j in t.query_pairs(2 * rr.max()):
        d = cc[i] - cc[j]
        if L is not None:
            d -= L * np.round(d / L)
        assert np.linalg.norm(d) >= rr[i] + rr[j] - 1e-15


def test_count_and_porosity(gpu_lib):
    sp = pack.SpherePack()
    n = sp.makeCloud((0, 0, 0), (1, 1, 1), rRelFuzz=0.3, num=500, porosity=0.8, seed=3)
    assert n == 500 == len(sp)
    cc, rr = sp.toCcRr()
    # the quantiles in decreasing order: rMean*(1 +- fuzz) for the porosity (SpherePack.cpp:152-155, 189-200)
    rMean = (1.0 * 0.2 / (math.pi * 4 / 3. * (1 + 0.09) * 500)) ** (1 / 3.)
    assert np.all(np.diff(rr) <= 0) and rr[0] == pytest.approx(rMean * (2 * ((500 + 0.5) / 501 - .5) * 0.3 + 1))
    assert np.all(cc - rr[:, None] >= 0) and np.all(cc + rr[:, None] <= 1)
    _no_overlap(sp)
    assert sp.sphereVol() == pytest.approx(0.2, rel=0.05)
    # a count that does not fit at porosity 0.5 is retried at higher porosities with smaller spheres
    sp = pack.SpherePack()
    assert sp.makeCloud((0, 0, 0), (1, 1, 1), rRelFuzz=0.3, num=500, seed=3) == 500
    assert sp.sphereVol() < 0.5
    _no_overlap(sp)


def test_mean_radius_fills_box(gpu_lib):
    sp = pack.SpherePack()
    n = sp.makeCloud((0, 0, 0), (0.2, 0.2, 0.2), rMean=0.01, rRelFuzz=0.2, seed=5)
    assert n > 200 and sp.sphereVol() / 0.008 > 0.15  # until the first sphere that finds no room (as the reference)
    _no_overlap(sp)


def test_psd_by_number_and_mass(gpu_lib):
    sizes, cumm = [0.01, 0.02, 0.04], [0.0, 0.5, 1.0]
    sp = pack.SpherePack()
    sp.makeCloud((0, 0, 0), (0.5, 0.5, 0.5), psdSizes=sizes, psdCumm=cumm, num=400, seed=2)
    d = 2 * sp.toCcRr()[1]
    assert len(sp) == 400 and d.min() >= 0.01 - 1e-12 and d.max() <= 0.04 + 1e-12
    assert np.mean(d <= 0.02) == pytest.approx(0.5, abs=0.01)
    sp2 = pack.SpherePack()
    sp2.makeCloud((0, 0, 0), (0.5, 0.5, 0.5), psdSizes=sizes, psdCumm=cumm, num=400, distributeMass=True, seed=2)
    edges, passing = sp2.psd(bins=30, mass=True)
    assert len(edges) == 31 and passing[0] == 0 and passing[-1] == pytest.approx(1.0)
    with pytest.raises(ValueError, match="same dimensions"):
        pack.SpherePack().makeCloud((0, 0, 0), (1, 1, 1), psdSizes=[1, 2], psdCumm=[0, .5, 1], num=10)
    with pytest.raises(ValueError, match="at least one"):
        pack.SpherePack().makeCloud((0, 0, 0), (1, 1, 1))


def test_periodic_and_to_simulation(gpu_lib, tmp_path):
    sp = pack.SpherePack()
    assert sp.makeCloud((0, 0, 0), (5, 5, 5), rMean=.5, rRelFuzz=.5, periodic=True, num=20, seed=1) == 20
    assert np.array_equal(sp.cellSize, [5, 5, 5])
    _no_overlap(sp, periodic=np.array([5.0, 5, 5]))
    S = woo.core.Scene(fields=[woo.dem.DemField()])
    ids = sp.toSimulation(S, rot=(math.cos(math.pi / 8), 0, 0, math.sin(math.pi / 8)), color=0)
    assert list(ids) == list(range(20)) and S.periodic
    # py/pack.py doctest: the cell rotated by 45 degrees about +z
    np.testing.assert_allclose(S.cell.hSize, [[3.5355339059327373, -3.5355339059327378, 0], [3.5355339059327378, 3.5355339059327373, 0],
                                              [0, 0, 5]], rtol=1e-14)
    f = str(tmp_path / "sp.txt")
    sp.userData = "study 1"
    sp.toFile(f)
    sp2 = pack.SpherePack()
    sp2.fromFile(f)
    assert np.array_equal(sp2.cellSize, sp.cellSize) and sp2.userData == "study 1"
    assert np.array_equal(sp2.toCcRr()[0], sp.toCcRr()[0]) and np.array_equal(sp2.toCcRr()[1], sp.toCcRr()[1])
    sp2.cellRepeat((2, 1, 3))
    assert len(sp2) == 120 and np.array_equal(sp2.cellSize, [10, 5, 15])
    _no_overlap(sp2, periodic=np.array([10.0, 5, 15]))
