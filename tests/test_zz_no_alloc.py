"""GPU test of wg_broadphase_noalloc, the broad phase for callers that cannot allocate device
memory (a process whose device memory belongs to another runtime's pool, a loop that cannot take
the synchronisation of cudaMalloc/cudaFree).

It is checked against the regular entry point: the same sphere boxes give exactly the pair set
of wg_collide_only (integer ids, so the comparison is exact), on two calls in a row, then on a
smaller scene with another spread, since the calls share one static scratch array whose previous
contents must not leak into the next result. Degenerate inputs (boxes of zero extent, a far
outlier, a NaN coordinate, too small an output capacity) are checked against a brute-force
overlap test. This file is collected last so that a run stopping at the first failure has run
everything else.
"""
import ctypes

import numpy as np
import pytest

import woodem_gb300 as woo
from woodem_gb300 import utils, scenes, _plan, _native
from woodem_gb300.dem import DemField, FrictMat

pytestmark = pytest.mark.gpu


def _sphere_scene(n, seed):
    r = scenes.lognormal_radii(n, seed)
    c = scenes.pack_rsa(r, (0, 0, 0), (0.22, 0.22, 0.22), seed=seed + 1)
    S = woo.core.Scene(fields=[DemField()])
    S.dem.par.addSpheres(c, r, FrictMat(density=2500, young=1e8))
    # a generous verlet distance makes many box overlaps without touching spheres
    S.engines = utils.defaultEngines(dynDtPeriod=0, verletDist=-0.4)
    S.dt = 0.3 * utils.pWaveDt(S)
    return S


def _noalloc(L, mn, mx, mask, lone, cap):
    n = len(mn)
    mn = np.ascontiguousarray(mn, dtype=float)
    mx = np.ascontiguousarray(mx, dtype=float)
    mask = np.ascontiguousarray(mask, dtype=np.uint32)
    lo = np.full(max(cap, 1), -1, np.int32)
    hi = np.full(max(cap, 1), -1, np.int32)
    npairs = ctypes.c_int64(-1)
    rc = L.wg_broadphase_noalloc(n, _native.ptr(mn), _native.ptr(mx), _native.ptr(mask, _native.P_U32), lone, cap,
                                 _native.ptr(lo, _native.P_I32), _native.ptr(hi, _native.P_I32), ctypes.byref(npairs))
    k = npairs.value
    return rc, lo[:max(k, 0)], hi[:max(k, 0)], k


def _collider_pairs(L, S):
    """Pair set and boxes of the regular entry point (wg_collide_only) for a scene."""
    sim = _plan.Simulation(S)
    S._sim = sim
    sim.H.check(L.wg_collide_only(sim.H.h), "collide_only")
    ref = _plan.read_contacts(L, sim.H.h, "wg")
    n = sim.A.n_particles
    mn, mx = np.empty((n, 3)), np.empty((n, 3))
    sim.H.check(L.wg_get_aabbs(sim.H.h, _native.ptr(mn), _native.ptr(mx)), "get_aabbs")
    mask = np.ascontiguousarray(sim.A.particles["mask"], dtype=np.uint32)
    lone = int(sim.A.config["lone_mask"])
    sim.close()
    return ref, mn, mx, mask, lone


def _brute(mn, mx, mask, lone):
    """Closed 3-axis overlap and the mask test, every pair, sorted by (lo, hi)."""
    n = len(mn)
    i, j = np.triu_indices(n, 1)
    ov = np.all((mn[i] <= mx[j]) & (mx[i] >= mn[j]), axis=1)
    mm = mask[i] & mask[j]
    ok = ov & (mm != 0) & ((mm & lone) == 0)
    return i[ok].astype(np.int32), j[ok].astype(np.int32)


def test_noalloc_matches_collider():
    L = _native.lib()
    ref, mn, mx, mask, lone = _collider_pairs(L, _sphere_scene(6000, 11))
    n = len(mn)
    assert len(ref["id_lo"]) > 1000
    for call in range(2):
        rc, lo, hi, k = _noalloc(L, mn, mx, mask, lone, 8 * n)
        assert rc == 0, L.wg_broadphase_noalloc_error().decode()
        assert k == len(ref["id_lo"]), "call %d: %d pairs vs %d" % (call, k, len(ref["id_lo"]))
        assert np.array_equal(lo, ref["id_lo"]) and np.array_equal(hi, ref["id_hi"])
    # a smaller scene with another spread after the larger one: nothing of the previous call's
    # offsets, counter or pairs may show through
    ref2, mn2, mx2, mask2, lone2 = _collider_pairs(L, _sphere_scene(900, 5))
    rc, lo, hi, k = _noalloc(L, mn2 * 3.0, mx2 * 3.0, mask2, lone2, 8 * len(mn2))
    assert rc == 0, L.wg_broadphase_noalloc_error().decode()
    blo, bhi = _brute(mn2 * 3.0, mx2 * 3.0, mask2, lone2)
    assert np.array_equal(lo, blo) and np.array_equal(hi, bhi)
    rc, lo, hi, k = _noalloc(L, mn2, mx2, mask2, lone2, 8 * len(mn2))
    assert rc == 0 and np.array_equal(lo, ref2["id_lo"]) and np.array_equal(hi, ref2["id_hi"])
    # too small an output capacity: the capacity error, with the true count
    rc, _, _, k = _noalloc(L, mn2, mx2, mask2, lone2, 1)
    assert rc == -5 and k == len(ref2["id_lo"]) and b"capacity" in L.wg_broadphase_noalloc_error()


def test_noalloc_degenerate_boxes():
    L = _native.lib()
    rng = np.random.default_rng(3)
    # boxes of zero extent (points), some of them coinciding: pairs are the coinciding points
    pts = rng.integers(0, 12, size=(700, 3)).astype(float) * 1e-3
    m = np.ones(len(pts), np.uint32)
    rc, lo, hi, k = _noalloc(L, pts, pts, m, 0, 200000)
    assert rc == 0, L.wg_broadphase_noalloc_error().decode()
    blo, bhi = _brute(pts, pts, m, 0)
    assert k == len(blo) > 0 and np.array_equal(lo, blo) and np.array_equal(hi, bhi)
    # every box the same point
    one = np.zeros((50, 3))
    rc, lo, hi, k = _noalloc(L, one, one, np.ones(50, np.uint32), 0, 5000)
    assert rc == 0 and k == 50 * 49 // 2
    # a cluster of small boxes and one box far away (a spread of ~1e9 box sizes)
    c = rng.uniform(0, 0.05, size=(1500, 3))
    c[0] = (1e6, -1e6, 3e5)
    r = rng.uniform(1e-3, 3e-3, size=(1500, 1))
    mm = np.ones(1500, np.uint32)
    rc, lo, hi, k = _noalloc(L, c - r, c + r, mm, 0, 500000)
    assert rc == 0, L.wg_broadphase_noalloc_error().decode()
    blo, bhi = _brute(c - r, c + r, mm, 0)
    assert k == len(blo) > 0 and np.array_equal(lo, blo) and np.array_equal(hi, bhi)
    # a NaN coordinate is an argument error, not a silently dropped sphere
    bad = (c - r).copy()
    bad[7, 1] = np.nan
    rc, _, _, _ = _noalloc(L, bad, c + r, mm, 0, 500000)
    assert rc == -1 and b"finite" in L.wg_broadphase_noalloc_error()


def test_noalloc_rejects_oversize():
    L = _native.lib()
    n = 40000
    a = np.zeros((n, 3))
    m = np.ones(n, np.uint32)
    npairs = ctypes.c_int64(0)
    out = np.zeros(1, np.int32)
    rc = L.wg_broadphase_noalloc(n, _native.ptr(a), _native.ptr(a), _native.ptr(m, _native.P_U32), 0, 1,
                                 _native.ptr(out, _native.P_I32), _native.ptr(out, _native.P_I32), ctypes.byref(npairs))
    assert rc == -5 and b"32768" in L.wg_broadphase_noalloc_error()
