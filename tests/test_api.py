"""CPU tests of the host layer: Woo-style scripting API, plan validation, scene builders,
and the C ABI library (loads and exports every declared symbol; no GPU calls)."""
import math
import os
import re

import numpy as np
import pytest

import woodem_gb300 as woo
from woodem_gb300 import utils, triangulated, scenes, _plan, _native
from woodem_gb300.dem import (DemField, FrictMat, ContactLoop, InsertionSortCollider, Leapfrog, Cg2_Sphere_Sphere_L6Geom,
                              Cp2_FrictMat_FrictPhys, Law2_L6Geom_FrictPhys_IdealElPl, Bo1_Sphere_Aabb,
                              Cp2_FrictMat_HertzPhys, Law2_L6Geom_HertzPhys_DMT)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(gpu_lib):
    hdr = open(os.path.join(ROOT, "include", "woo_gpu.h")).read()
    names = set(re.findall(r"^\s*(?:int|void|const char\*|int64_t)\s+\**(wg_\w+)\s*\(", hdr, re.M))
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(gpu_lib, n), n


def test_oracle_library_loads(oracle_lib):
    assert hasattr(oracle_lib, "wo_run")


def test_default_engines_structure():
    ee = utils.defaultEngines(damping=.2, dynDtPeriod=0)
    assert [type(e).__name__ for e in ee] == ["Leapfrog", "InsertionSortCollider", "ContactLoop"]
    assert ee[0].reset is True and ee[0].damping == .2
    assert ee[1].verletDist == -.05
    assert isinstance(ee[2].lawDisp[0], Law2_L6Geom_FrictPhys_IdealElPl)
    ee = utils.defaultEngines()
    assert type(ee[-1]).__name__ == "DynDt"


def test_special_constructors():
    # ContactLoop([Cg2],[Cp2],[Law2]) (ContactLoop.cpp:52-66), InsertionSortCollider([Bo1]) (:983-991)
    cl = ContactLoop([Cg2_Sphere_Sphere_L6Geom()], [Cp2_FrictMat_FrictPhys()], [Law2_L6Geom_FrictPhys_IdealElPl()],
                     applyForces=True)
    assert len(cl.geoDisp) == 1 and cl.applyForces
    col = InsertionSortCollider([Bo1_Sphere_Aabb()], verletDist=0.01)
    assert col.verletDist == 0.01 and len(col.boundDispatcher) == 1
    with pytest.raises(AttributeError):
        Leapfrog(notAnAttribute=1)


def test_sphere_mass_inertia():
    m = FrictMat(density=2000, young=1e7)
    p = utils.sphere((1, 2, 3), 0.1, mat=m)
    mass = 4 / 3. * math.pi * 0.1 ** 3 * 2000
    assert p.mass == pytest.approx(mass, rel=1e-15)
    assert p.inertia[0] == pytest.approx(0.4 * mass * 0.01, rel=1e-15)
    w = utils.wall(0.5, axis=1, sense=-1)
    assert w.blocked == "xyzXYZ" and w.shape.axis == 1 and w.pos[1] == 0.5


def test_particle_views_and_containers():
    S = woo.core.Scene(fields=[DemField(gravity=(0, 0, -9.81))])
    ids = S.dem.par.add([utils.sphere((0, 0, 0), .1), utils.sphere((0, 0, .3), .1)])
    assert ids == [0, 1] and len(S.dem.par) == 2
    S.dem.par[1].vel = (1, 2, 3)
    assert list(S.dem.par[1].vel) == [1, 2, 3]
    rng = S.dem.par.addSpheres(np.zeros((5, 3)) + 2, 0.05, FrictMat())
    assert list(rng) == [2, 3, 4, 5, 6] and S.dem.par[4].shape.radius == 0.05


def test_plan_rejects_unsupported():
    S = scenes.box_settle_small(n=20, precision="fp32")
    S.engines = utils.defaultEngines(damping=.2)  # the stock engine list (DynDt) in the FP32-force mode
    assert _plan.compile_scene(S).config["dyndt"] == 1
    S.trackEnergy = True
    assert _plan.compile_scene(S).config["track_energy"] == 1
    S.engines[0].reset = False
    with pytest.raises(NotImplementedError):
        _plan.compile_scene(S)
    S = scenes.box_settle_small(n=20)
    S.engines = utils.defaultEngines(damping=.2)
    assert _plan.compile_scene(S).config["dyndt"] == 1 and S.engines[-1].stepPeriod == 100
    S.engines = utils.defaultEngines(dynDtPeriod=0, cp2=Cp2_FrictMat_HertzPhys(alpha=.5), law=Law2_L6Geom_HertzPhys_DMT())
    with pytest.raises(NotImplementedError):
        _plan.compile_scene(S)
    S.engines = utils.defaultEngines(dynDtPeriod=0)[::-1]
    with pytest.raises(NotImplementedError):
        _plan.compile_scene(S)
    S.engines = utils.defaultEngines(dynDtPeriod=0, lawKw=dict(iniEqlb=True))
    with pytest.raises(NotImplementedError):
        _plan.compile_scene(S)


def test_box_settle_config():
    S = scenes.box_settle(n=10000, seed=0)
    A = _plan.compile_scene(S)
    assert A.n_particles == 10006 and A.n_nodes == 10006
    assert A.config["dt"] == pytest.approx(0.3 * 0.005 / math.sqrt(1e7 / 3000), rel=1e-14)
    assert A.config["damping"] == .2 and A.config["verlet_dist"] == -.1 and A.config["law"] == 0
    pos = A.nodes["pos"][6:]
    assert pos[:, 2].min() > 0.011 - 1e-9 - 1e-3 and pos[:, 0].min() > 0.024 - 1.001e-3


def test_cylinder_mesh():
    ff = triangulated.cylinder((0, 0, 0), (0.6, 0, 0), 0.6, div=21, axDiv=5, capA=True, capB=True, wallCaps=True, angVel=1.0)
    caps, facets = ff[:2], ff[2:]
    assert len(facets) == 2 * 20 * 5
    assert caps[0].shape.sense == 1 and caps[1].shape.sense == -1 and caps[0].angVel[0] == 1.0
    for f in facets[:20]:
        n = f.shape.getNormal()
        c = np.mean([np.asarray(x.pos) for x in f.shape.nodes], axis=0)
        radial = np.array([0, c[1], c[2]])
        assert np.dot(n, radial) > 0  # outward
        # surface moves with omega x r (omega along +x)
        want = np.cross([1.0, 0, 0], radial)
        assert np.dot(f.shape.fakeVel, want) > 0


def test_pack_rsa_non_overlapping(gpu_lib):
    r = scenes.lognormal_radii(3000, 0)
    c = scenes.pack_rsa(r, (0, 0, 0), (0.2, 0.2, 0.2), seed=1)
    from scipy.spatial import cKDTree
    t = cKDTree(c)
    for i, j in t.query_pairs(2 * r.max()):
        assert np.linalg.norm(c[i] - c[j]) >= r[i] + r[j] - 1e-15
    assert np.all(c - r[:, None] >= -1e-15) and np.all(c + r[:, None] <= 0.2 + 1e-15)


def test_pack_rsa_device_rejects_arguments(gpu_lib):
    """wg_pack_rsa_device validates its arguments before any device call: -2 for a bad region
    kind, a non-positive radius, an empty box or a missing cylinder description."""
    from woodem_gb300 import _native
    r = np.full(10, 1e-3)
    out = np.zeros((10, 3))
    lo, hi = np.zeros(3), np.full(3, 0.1)
    P = _native.ptr

    def call(radii, lo_, hi_, kind, params):
        return gpu_lib.wg_pack_rsa_device(len(radii), P(radii), P(lo_), P(hi_), kind, params, 1, 100, P(out))
    assert call(r, lo, hi, 3, P(np.zeros(4))) == -2
    assert call(np.r_[r[:9], -1.0], lo, hi, 0, P(np.zeros(4))) == -2
    assert call(r, lo, lo, 0, P(np.zeros(4))) == -2
    assert call(r, lo, hi, 1, None) == -2
    assert gpu_lib.wg_pack_rsa_device(0, P(r), P(lo), P(hi), 0, P(np.zeros(4)), 1, 100, P(out)) == 0


def test_quadrilateral_mesh():
    """py/triangulated.py:70-83: 2*div0*div1 facets covering the quadrilateral, vertices shared."""
    ff = triangulated.quadrilateral((0, 0, 0), (2, 0, 0), (0, 3, 0), (2, 3, 0), div=(4, 3))
    assert len(ff) == 24
    area = sum(0.5 * np.linalg.norm(np.cross(np.asarray(f.shape.nodes[1].pos) - np.asarray(f.shape.nodes[0].pos),
                                             np.asarray(f.shape.nodes[2].pos) - np.asarray(f.shape.nodes[0].pos))) for f in ff)
    assert area == pytest.approx(6.0, rel=1e-12)
    assert len({id(n) for f in ff for n in f.shape.nodes}) == 5 * 4
    assert len(triangulated.quadrilateral((0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0))) == 8
    assert len(triangulated.quadrilateral((0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0), size=0.25)) == 32
    with pytest.raises(ValueError):
        triangulated.quadrilateral((0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0), size=0.5, div=(2, 2))
