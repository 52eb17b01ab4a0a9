"""Random sequential insertion on the device (wg_pack_rsa_device), the scene-generation step of
SpherePack::makeCloud (lib/sphere-pack/SpherePack.hpp:75) for the benchmark regions.

The device packer inserts spheres in rounds over a window of spheres, so its packing is not the
host packer's sphere for sphere; both must give valid packings with the same statistics:
* no two spheres overlap (minimum image in the periodic box), every sphere inside its region;
* every sphere placed where the host packer places every sphere (solid fraction 0.35 of
  radii uniform in [2, 4] mm in a periodic box, the periodic-shear configuration's insertion);
* the same seed gives the same packing, another seed another one;
* the centres are uniform: each octant of the box holds its share of the spheres within 5
  standard deviations, and the mean centre is the box centre within 1 % of the edge.
"""
import math
import time

import numpy as np
import pytest

from woodem_gb300 import scenes

pytestmark = pytest.mark.gpu


def _periodic_case(n, seed):
    rng = np.random.default_rng(seed)
    r = rng.uniform(2e-3, 4e-3, n)
    side = (float(np.sum(4 / 3.0 * math.pi * r ** 3)) / 0.35) ** (1 / 3.0)
    return r, side


def _no_overlap(c, r, boxsize=None):
    from scipy.spatial import cKDTree
    if boxsize is not None:
        c = np.mod(c, boxsize)
    t = cKDTree(c, boxsize=boxsize)
    pairs = t.query_pairs(2 * r.max(), output_type="ndarray")
    d = c[pairs[:, 0]] - c[pairs[:, 1]]
    if boxsize is not None:
        d -= boxsize * np.round(d / boxsize)
    dist = np.linalg.norm(d, axis=1)
    return bool(np.all(dist >= r[pairs[:, 0]] + r[pairs[:, 1]] - 1e-15))


def test_device_pack_periodic(gpu_lib):
    r, side = _periodic_case(20000, 3)
    c = scenes.pack_rsa(r, (0, 0, 0), (side, side, side), region=2, seed=5, device=True)
    assert c.shape == (20000, 3)
    assert np.all(c >= 0) and np.all(c < side)
    assert _no_overlap(c, r, boxsize=side)
    c2 = scenes.pack_rsa(r, (0, 0, 0), (side, side, side), region=2, seed=5, device=True)
    assert np.array_equal(c, c2)
    c3 = scenes.pack_rsa(r, (0, 0, 0), (side, side, side), region=2, seed=6, device=True)
    assert not np.array_equal(c, c3)
    # uniform centres
    oct_ = ((c > side / 2).astype(int) * [1, 2, 4]).sum(axis=1)
    cnt = np.bincount(oct_, minlength=8)
    assert np.all(np.abs(cnt - len(c) / 8) <= 5 * math.sqrt(len(c) / 8 * 7 / 8))
    assert np.all(np.abs(c.mean(axis=0) - side / 2) <= 0.01 * side)


def test_device_pack_box_and_cylinder(gpu_lib):
    r = scenes.lognormal_radii(5000, 0)
    c = scenes.pack_rsa(r, (0, 0, 0), (0.2, 0.2, 0.2), seed=1, device=True)
    assert _no_overlap(c, r)
    assert np.all(c - r[:, None] >= -1e-15) and np.all(c + r[:, None] <= 0.2 + 1e-15)
    # the lower part of an x-axis cylinder of radius 0.1 clipped at z <= 0
    Ri, zf = 0.1, 0.0
    r = scenes.lognormal_radii(3000, 1)
    c = scenes.pack_rsa(r, (0, -Ri, -Ri), (0.3, Ri, zf), region=1, params=(0.0, 0.0, Ri, zf), seed=2, device=True)
    assert _no_overlap(c, r)
    assert np.all(np.hypot(c[:, 1], c[:, 2]) <= Ri - r + 1e-15) and np.all(c[:, 2] + r <= zf + 1e-15)
    assert np.all(c[:, 0] - r >= -1e-15) and np.all(c[:, 0] + r <= 0.3 + 1e-15)


def test_device_pack_large(gpu_lib):
    """300 000 spheres, the largest periodic job of the serving stream: all placed, valid, and
    timed beside the host packer on the same input."""
    r, side = _periodic_case(300000, 4)
    t0 = time.perf_counter()
    c = scenes.pack_rsa(r, (0, 0, 0), (side, side, side), region=2, seed=7, device=True)
    t1 = time.perf_counter()
    h = scenes.pack_rsa(r, (0, 0, 0), (side, side, side), region=2, seed=7)
    t2 = time.perf_counter()
    print("300k periodic insertion: device %.3f s, host %.3f s" % (t1 - t0, t2 - t1))
    assert _no_overlap(c, r, boxsize=side) and len(c) == len(h) == 300000
