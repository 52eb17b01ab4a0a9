"""``woo.utils`` counterparts used by scene scripts (py/utils.py:38-260)."""
import math
import random
import warnings

import numpy as np

from .dem import (DemField, Particle, Node, Sphere, Wall, Facet, FrictMat, Leapfrog, InsertionSortCollider,
                  ContactLoop, DynDt, Bo1_Sphere_Aabb, Bo1_Facet_Aabb, Bo1_Wall_Aabb, Cg2_Sphere_Sphere_L6Geom,
                  Cg2_Facet_Sphere_L6Geom, Cg2_Wall_Sphere_L6Geom, Cp2_FrictMat_FrictPhys,
                  Law2_L6Geom_FrictPhys_IdealElPl, SHAPE_SPHERE, DOF_ALL)

inf = float("inf")


def spherePWaveDt(radius, density, young):
    r"""P-wave critical timestep :math:`\Delta t_c = r/\sqrt{E/\rho}` (py/utils.py:38-46).

    >>> spherePWaveDt(1e-3,2400,30e9)
    2.8284271247461903e-07
    """
    return radius / math.sqrt(young / density)


def pWaveDt(S=None, noClumps=False):
    """DemFuncs::pWaveDt (pkg/dem/Funcs.cpp:116-141): min over uninodal spheres of r/sqrt(E/rho)."""
    dem = S.dem
    s = dem.par.soa
    if len(s) == 0:
        return inf
    sel = s.col("shape") == SHAPE_SPHERE
    if not np.any(sel):
        return inf
    mats = dem._mats
    young = np.array([m.young for m in mats])[s.col("mat")[sel]]
    dens = np.array([m.density for m in mats])[s.col("mat")[sel]]
    return float(np.min(s.col("radius")[sel] / np.sqrt(young / dens)))


def defaultMaterial():
    """FrictMat(density=1e3,young=1e7,ktDivKn=.2,tanPhi=tan(.5)) (py/utils.py:48-53)."""
    return FrictMat(density=1e3, young=1e7, ktDivKn=0.2, tanPhi=math.tan(0.5))


def defaultEngines(damping=0.0, gravity=None, verletDist=-0.05, kinSplit=False, dontCollect=False, noSlip=False,
                   noBreak=False, cp2=None, law=None, model=None, grid=False, dynDtPeriod=100, cpKw={}, lawKw={}):
    """py/utils.py:55-94: [Leapfrog, InsertionSortCollider, ContactLoop, (DynDt)]."""
    if gravity:
        raise ValueError("gravity MUST NOT be specified anymore, set DemField.gravity=... instead.")
    if grid:
        raise ValueError("GridCollider is not part of the GPU path; use the default InsertionSortCollider")
    if model:
        if cp2 or law:
            warnings.warn("cp2 and law args are ignored when model is provided.")
        cp2, law = model.getFunctors()
        damping = model.getNonviscDamping()
        distFactor = model.distFactor
    else:
        cp2 = [cp2 if cp2 else Cp2_FrictMat_FrictPhys()]
        law = [law if law else Law2_L6Geom_FrictPhys_IdealElPl(noSlip=noSlip, noBreak=noBreak, label="contactLaw")]
        distFactor = 1.0
    cp2[0].updateAttrs(cpKw)
    law[0].updateAttrs(lawKw)
    collider = InsertionSortCollider([Bo1_Sphere_Aabb(distFactor=distFactor), Bo1_Facet_Aabb(), Bo1_Wall_Aabb()],
                                     label="collider", verletDist=verletDist)
    ee = [
        Leapfrog(damping=damping, reset=True, kinSplit=kinSplit, dontCollect=dontCollect, label="leapfrog"),
        collider,
        ContactLoop([Cg2_Sphere_Sphere_L6Geom(distFactor=distFactor), Cg2_Facet_Sphere_L6Geom(), Cg2_Wall_Sphere_L6Geom()],
                    cp2, law, applyForces=True, label="contactLoop"),
    ]
    if dynDtPeriod > 0:
        ee.append(DynDt(stepPeriod=dynDtPeriod, label="dynDt"))
    return ee


def _mkDemNode(**kw):
    return Node(**kw)


def _commonBodySetup(b, nodes, mat, fixed=False):
    """py/utils.py:96-105"""
    if callable(mat) and not isinstance(mat, FrictMat):
        mat = mat()
    b.material = mat
    b.shape.nodes = nodes
    if len(nodes) == 1:
        b.updateMassInertia()
    else:
        for n in b.shape.nodes:
            n.dem.mass = 0
            n.dem.inertia = np.zeros(3)
    for n in b.shape.nodes:
        if fixed is None:
            pass
        elif fixed:
            n.dem.blocked = "xyzXYZ"
        else:
            n.dem.blocked = "".join("XYZ"[ax] for ax in (0, 1, 2) if n.dem.inertia[ax] == inf)


def sphere(center, radius, mat=defaultMaterial, fixed=False, wire=False, color=None, highlight=False,
           mask=DemField.defaultMovableMask):
    """py/utils.py:107-155"""
    b = Particle()
    b.shape = Sphere(radius=radius, color=color if color else random.random())
    b.shape.wire = wire
    _commonBodySetup(b, [center] if isinstance(center, Node) else [_mkDemNode(pos=center)], mat=mat, fixed=fixed)
    b.aspherical = False
    b.mask = mask
    return b


def wall(position, axis, sense=0, glAB=None, fixed=True, mass=0, color=None, mat=defaultMaterial, visible=True,
         mask=DemField.defaultBoundaryMask):
    """py/utils.py:177-199"""
    p = Particle()
    p.shape = Wall(sense=sense, axis=axis, color=color if color else random.random())
    if glAB:
        p.shape.glAB = glAB
    if not fixed and mass <= 0:
        raise ValueError("Non-fixed wall must have positive mass")
    if isinstance(position, (int, float)):
        pos2 = np.zeros(3)
        pos2[axis] = position
        node = _mkDemNode(pos=pos2)
    elif isinstance(position, Node):
        node = position
    else:
        node = _mkDemNode(pos=position)
    _commonBodySetup(p, [node], mat=mat, fixed=fixed)
    p.shape.nodes[0].dem.mass = mass
    p.aspherical = False
    p.mask = mask
    p.shape.visible = visible
    return p


def wallBox(box, which=(1, 1, 1, 1, 1, 1), **kw):
    """py/utils.py:201-210: walls at -x,+x,-y,+y,-z,+z with senses facing inwards. ``box`` is (min, max)."""
    mn, mx = np.asarray(box[0], dtype=float), np.asarray(box[1], dtype=float)
    ret = []
    if len(which) != 6:
        raise ValueError("Wall.makeBox: which must be a sequence of boolean-convertible.")
    for sense, ix, coord in [(1, 0, mn), (-1, 1, mx)]:
        for ax in (0, 1, 2):
            if not which[3 * ix + ax]:
                continue
            ret.append(wall(coord[ax], sense=sense, axis=ax, **kw))
    return ret


def facet(vertices, fakeVel=None, halfThick=0.0, fixed=True, wire=True, color=None, highlight=False, mat=defaultMaterial,
          visible=True, mask=DemField.defaultBoundaryMask):
    """py/utils.py:242-275"""
    p = Particle()
    if isinstance(vertices[0], Node):
        nodes = list(vertices)
    else:
        nodes = [_mkDemNode(pos=vertices[i]) for i in range(3)]
    p.shape = Facet(color=color if color else random.random())
    if fakeVel is not None:
        p.shape.fakeVel = np.asarray(fakeVel, dtype=float)
    p.shape.halfThick = halfThick
    p.shape.wire = wire
    _commonBodySetup(p, nodes, mat=mat, fixed=fixed)
    p.aspherical = False
    p.mask = mask
    p.shape.visible = visible
    return p


def unbalancedEnergy(S):
    """Kinetic over elastic energy (py/utils.py:816-822); NaN when either is missing or elast is 0."""
    if not S.trackEnergy:
        raise RuntimeError("Scene.trackEnergy==False")
    if "elast" not in S.energy or "kinetic" not in S.energy:
        return float("nan")
    if S.energy["elast"] == 0:
        return float("nan")
    return S.energy["kinetic"] / S.energy["elast"]


def _deprecatedUtilsFunction(old, new):
    import warnings
    warnings.warn("Function utils.%s is deprecated, use %s instead." % (old, new), stacklevel=3, category=DeprecationWarning)


def runningInBatch():
    """Deprecated alias of woo.batch.inBatch (py/utils.py:845-847)."""
    from . import batch
    _deprecatedUtilsFunction("runningInBatch", "woo.batch.inBatch")
    return batch.inBatch()


def waitIfBatch(S=None):
    """Deprecated alias of woo.batch.wait."""
    from . import batch
    _deprecatedUtilsFunction("waitIfBatch", "woo.batch.wait")
    return batch.wait(S)


def readParamsFromTable(*args, **kw):
    """Deprecated alias of woo.batch.readParamsFromTable."""
    from . import batch
    _deprecatedUtilsFunction("readParamsFromTable", "woo.batch.readParamsFromTable")
    return batch.readParamsFromTable(*args, **kw)


def runPreprocessorInBatch(*args, **kw):
    """Deprecated alias of woo.batch.runPreprocessor."""
    from . import batch
    _deprecatedUtilsFunction("runPreprocessorInBatch", "woo.batch.runPreprocessor")
    return batch.runPreprocessor(*args, **kw)


# DemField.minimalEngines is defaultEngines (py/_monkey/aliases.py:102)
DemField.minimalEngines = staticmethod(defaultEngines)
