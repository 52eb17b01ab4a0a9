"""Object construction rules of the scripting surface, restating py/tests/core.py
(testDispatcherCtor, testContactLoopCtor, testWrongFunctorType, testInvalidAttr, testShared,
testSharedAfterReload) for the classes of the path."""
import pytest

import woodem_gb300 as woo
from woodem_gb300 import utils
from woodem_gb300.core import Scene
from woodem_gb300.dem import (Bo1_Sphere_Aabb, CGeomDispatcher, Cg2_Facet_Sphere_L6Geom, Cg2_Sphere_Sphere_L6Geom,
                              ContactLoop, Cp2_FrictMat_FrictPhys, DemField, InsertionSortCollider, LawDispatcher,
                              Law2_L6Geom_FrictPhys_IdealElPl, Law2_L6Geom_HertzPhys_DMT, Sphere, BoundDispatcher)


def test_dispatcher_ctor():
    # functors of the same class collapse into one; different ones stay
    cld1 = LawDispatcher([Law2_L6Geom_FrictPhys_IdealElPl(), Law2_L6Geom_FrictPhys_IdealElPl()])
    assert len(cld1.functors) == 1
    cld2 = LawDispatcher([Law2_L6Geom_FrictPhys_IdealElPl(), Law2_L6Geom_HertzPhys_DMT()])
    assert len(cld2.functors) == 2


def test_contact_loop_ctor():
    cl = ContactLoop([Cg2_Facet_Sphere_L6Geom(), Cg2_Sphere_Sphere_L6Geom()], [Cp2_FrictMat_FrictPhys()],
                     [Law2_L6Geom_FrictPhys_IdealElPl()])
    assert len(cl.geoDisp.functors) == 2
    assert cl.geoDisp.__class__ == CGeomDispatcher
    assert cl.phyDisp.functors[0].__class__ == Cp2_FrictMat_FrictPhys
    assert cl.lawDisp.functors[0].__class__ == Law2_L6Geom_FrictPhys_IdealElPl
    # assigning a plain list gives the dispatcher of the attribute
    cl.lawDisp = [Law2_L6Geom_HertzPhys_DMT()]
    assert type(cl.lawDisp) == LawDispatcher and len(cl.lawDisp) == 1
    col = InsertionSortCollider([Bo1_Sphere_Aabb()])
    assert type(col.boundDispatcher) == BoundDispatcher and len(col.boundDispatcher.functors) == 1
    with pytest.raises(ValueError):
        ContactLoop([Cg2_Sphere_Sphere_L6Geom()])


def test_wrong_functor_type():
    with pytest.raises(TypeError):
        LawDispatcher([Bo1_Sphere_Aabb()])
    with pytest.raises(TypeError):
        ContactLoop([Law2_L6Geom_FrictPhys_IdealElPl()], [], [Cg2_Sphere_Sphere_L6Geom()])


def test_invalid_attr():
    with pytest.raises(AttributeError):
        Sphere(attributeThatDoesntExist=42)
    with pytest.raises(AttributeError):
        Sphere().attributeThatDoesntExist


def test_shared_material():
    m = utils.defaultMaterial()
    s1, s2 = utils.sphere((0, 0, 0), 1, mat=m), utils.sphere((0, 0, 0), 2, mat=m)
    s1.mat.young = 2342333
    assert s1.mat.young == s2.mat.young


def test_shared_after_reload():
    S = Scene(fields=[DemField()])
    m = utils.defaultMaterial()
    S.dem.par.add([utils.sphere((0, 0, 0), 1, mat=m), utils.sphere((0, 0, 0), 2, mat=m)])
    S.saveTmp()
    S = Scene.loadTmp()
    S.dem.par[0].mat.young = 9087438484
    assert S.dem.par[0].mat.young == S.dem.par[1].mat.young


def test_default_engines_dispatchers_round_trip():
    """The engines of utils.defaultEngines keep their dispatcher types through expr, json and pickle."""
    for e in utils.defaultEngines():
        for fmt in ("expr", "json", "pickle"):
            e2 = woo.core.Object.loads(e.dumps(format=fmt))
            for a in ("geoDisp", "phyDisp", "lawDisp", "boundDispatcher"):
                if hasattr(e, a):
                    assert type(getattr(e2, a)) == type(getattr(e, a))
                    assert [type(f) for f in getattr(e2, a)] == [type(f) for f in getattr(e, a)]
