"""GPU test of wg_broadphase_noalloc, the broad phase for callers that cannot allocate device
memory (a runtime that owns the device memory pool, code running during CUDA graph capture).

It is checked against the regular entry point: the same sphere boxes give exactly the pair set
of wg_collide_only (integer ids, so the comparison is exact), on two calls in a row, since the
calls share one static scratch array whose previous contents must not leak into the next result.
This file is collected last so that a run stopping at the first failure has run everything else.
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


def test_noalloc_matches_collider():
    L = _native.lib()
    S = _sphere_scene(6000, 11)
    sim = _plan.Simulation(S)
    S._sim = sim
    sim.H.check(L.wg_collide_only(sim.H.h), "collide_only")
    ref = _plan.read_contacts(L, sim.H.h, "wg")
    n = sim.A.n_particles
    mn, mx = np.empty((n, 3)), np.empty((n, 3))
    sim.H.check(L.wg_get_aabbs(sim.H.h, _native.ptr(mn), _native.ptr(mx)), "get_aabbs")
    mask = np.ascontiguousarray(sim.A.particles["mask"], dtype=np.uint32)
    lone = int(sim.A.config["lone_mask"])
    assert len(ref["id_lo"]) > 1000
    for call in range(2):
        cap = 8 * n
        lo = np.full(cap, -1, np.int32)
        hi = np.full(cap, -1, np.int32)
        npairs = ctypes.c_int64(-1)
        rc = L.wg_broadphase_noalloc(n, _native.ptr(mn), _native.ptr(mx), _native.ptr(mask, _native.P_U32), lone, cap,
                                     _native.ptr(lo, _native.P_I32), _native.ptr(hi, _native.P_I32), ctypes.byref(npairs))
        assert rc == 0, L.wg_broadphase_noalloc_error().decode()
        k = npairs.value
        assert k == len(ref["id_lo"]), "call %d: %d pairs vs %d" % (call, k, len(ref["id_lo"]))
        assert np.array_equal(lo[:k], ref["id_lo"]) and np.array_equal(hi[:k], ref["id_hi"])
    sim.close()


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
