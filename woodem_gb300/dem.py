"""``woo.dem`` counterparts for the hot path: data model, shapes, materials, functors, engines.

Class names and attribute names follow the reference so that scene scripts run
unchanged (pkg/dem/Particle.hpp, Sphere.hpp, Wall.hpp, Facet.hpp, FrictMat.hpp,
Hertz.hpp, IdealElPl.hpp, L6Geom.hpp, ContactLoop.hpp, InsertionSortCollider.hpp,
Leapfrog.hpp). Storage is structure-of-arrays: particles and nodes live in numpy
columns that are uploaded to the device as-is; Particle/Node objects handed to
scripts are lightweight views into those columns.
"""
import math
import numpy as np

from .core import Object, Engine, PeriodicEngine, Field, NaN
from ._soa import SoA

inf = float("inf")

# DemData flag bits (pkg/dem/Particle.hpp:179-186)
DOF_X, DOF_Y, DOF_Z, DOF_RX, DOF_RY, DOF_RZ = 1, 2, 4, 8, 16, 32
DOF_ALL = 63
CLUMP_CLUMPED, CLUMP_CLUMP, ENERGY_SKIP, GRAVITY_SKIP, TRACER_SKIP, DAMPING_SKIP = 64, 128, 256, 512, 1024, 2048

SHAPE_SPHERE, SHAPE_WALL, SHAPE_FACET = 0, 1, 2


# ------------------------------------------------------------------ nodes
_NODE_SPEC = {
    "pos": (np.float64, (3,), 0.0), "ori": (np.float64, (4,), 0.0), "vel": (np.float64, (3,), 0.0),
    "angVel": (np.float64, (3,), 0.0), "force": (np.float64, (3,), 0.0), "torque": (np.float64, (3,), 0.0),
    "mass": (np.float64, (), 0.0), "inertia": (np.float64, (3,), 0.0), "flags": (np.uint32, (), 0),
}


def _blocked_to_flags(s):
    f = 0
    for ch in s:
        if ch not in "xyzXYZ":
            raise ValueError("Invalid blocked DOF '%s' (must be in xyzXYZ)" % ch)
        f |= {"x": DOF_X, "y": DOF_Y, "z": DOF_Z, "X": DOF_RX, "Y": DOF_RY, "Z": DOF_RZ}[ch]
    return f


def _flags_to_blocked(f):
    return "".join(ch for ch, b in zip("xyzXYZ", (DOF_X, DOF_Y, DOF_Z, DOF_RX, DOF_RY, DOF_RZ)) if f & b)


class _Rec:
    """Attribute storage of a node or particle that is not (yet) in a container."""

    def __init__(self, spec):
        self.vals = {}
        for k, (dt, sh, fill) in spec.items():
            self.vals[k] = np.full(sh, fill, dtype=dt) if sh else dt(fill)


class DemData:
    """Dynamic state of a node (pkg/dem/Particle.hpp:169-274); a view onto its Node."""

    __slots__ = ("_node",)

    def __init__(self, _node=None, **kw):
        object.__setattr__(self, "_node", _node if _node is not None else Node())
        for k, v in kw.items():
            setattr(self, k, v)

    def _get(self, k):
        return self._node._get(k)

    def _set(self, k, v):
        self._node._set(k, v)

    vel = property(lambda s: s._get("vel"), lambda s, v: s._set("vel", v))
    angVel = property(lambda s: s._get("angVel"), lambda s, v: s._set("angVel", v))
    force = property(lambda s: s._get("force"), lambda s, v: s._set("force", v))
    torque = property(lambda s: s._get("torque"), lambda s, v: s._set("torque", v))
    mass = property(lambda s: float(s._get("mass")), lambda s, v: s._set("mass", v))
    inertia = property(lambda s: s._get("inertia"), lambda s, v: s._set("inertia", v))
    flags = property(lambda s: int(s._get("flags")), lambda s, v: s._set("flags", v))

    @property
    def blocked(self):
        return _flags_to_blocked(self.flags)

    @blocked.setter
    def blocked(self, s):
        self.flags = (self.flags & ~DOF_ALL) | _blocked_to_flags(s)

    gravitySkip = property(lambda s: bool(s.flags & GRAVITY_SKIP),
                           lambda s, v: setattr(s, "flags", (s.flags | GRAVITY_SKIP) if v else (s.flags & ~GRAVITY_SKIP)))
    dampingSkip = property(lambda s: bool(s.flags & DAMPING_SKIP),
                           lambda s, v: setattr(s, "flags", (s.flags | DAMPING_SKIP) if v else (s.flags & ~DAMPING_SKIP)))
    energySkip = property(lambda s: bool(s.flags & ENERGY_SKIP),
                          lambda s, v: setattr(s, "flags", (s.flags | ENERGY_SKIP) if v else (s.flags & ~ENERGY_SKIP)))

    @property
    def isAspherical(self):
        i = self.inertia
        return not (i[0] == i[1] and i[1] == i[2])

    def addParRef(self, p):
        return


class Node:
    """A point with position and orientation (core/Field.hpp:50-108) and its DemData."""

    @classmethod
    def load(cls, inFile, format="auto"):
        from . import _objio
        return _objio.load(inFile, format, cls)

    __slots__ = ("_store", "_i", "_rec")

    def __init__(self, pos=(0, 0, 0), ori=None, dem=None):
        object.__setattr__(self, "_store", None)
        object.__setattr__(self, "_i", -1)
        object.__setattr__(self, "_rec", _Rec(_NODE_SPEC))
        self._rec.vals["pos"][:] = pos
        self._rec.vals["ori"][:] = (1.0, 0.0, 0.0, 0.0) if ori is None else _quat_wxyz(ori)

    def _get(self, k):
        if self._store is None:
            return self._rec.vals[k]
        self._store._before_read()
        return self._store.soa.col(k)[self._i]

    def _set(self, k, v):
        if self._store is None:
            if self._rec.vals[k].shape:
                self._rec.vals[k][:] = v
            else:
                self._rec.vals[k] = self._rec.vals[k].dtype.type(v)
        else:
            self._store._before_read()
            self._store.soa.col(k)[self._i] = v
            self._store._after_write()

    pos = property(lambda s: s._get("pos"), lambda s, v: s._set("pos", v))

    @property
    def ori(self):
        return self._get("ori")

    @ori.setter
    def ori(self, q):
        self._set("ori", _quat_wxyz(q))

    @property
    def dem(self):
        return DemData(self)

    @dem.setter
    def dem(self, d):
        if d is None:
            return
        if isinstance(d, DemData) and d._node is not self:
            for k in ("vel", "angVel", "force", "torque", "mass", "inertia", "flags"):
                self._set(k, d._get(k))


def _quat_wxyz(q):
    q = np.asarray(q, dtype=float).ravel()
    if q.shape != (4,):
        raise ValueError("orientation must be a quaternion (w,x,y,z)")
    return q


class _NodeStore:
    def __init__(self, field):
        self.soa = SoA(_NODE_SPEC)
        self.field = field

    def _before_read(self):
        self.field._pull_state()

    def _after_write(self):
        self.field._state_written()

    def adopt(self, node):
        if node._store is self:
            return node._i
        if node._store is not None:
            raise ValueError("Node belongs to another DemField")
        i = self.soa.append(1, **node._rec.vals)
        object.__setattr__(node, "_store", self)
        object.__setattr__(node, "_i", i)
        object.__setattr__(node, "_rec", None)
        return i


# ------------------------------------------------------------------ shapes and materials
class Shape(Object):
    _attrs = {"color": 0.5, "wire": False, "visible": True, "highlight": False}

    def __init__(self, **kw):
        self.nodes = []
        super().__init__(**kw)


class Sphere(Shape):
    _attrs = {"radius": NaN}
    _kind = SHAPE_SPHERE

    @staticmethod
    def make(center, radius, **kw):
        from . import utils
        return utils.sphere(center, radius, **kw)

    def volume(self):
        return (4 / 3.0) * math.pi * self.radius ** 3


class Wall(Shape):
    _attrs = {"sense": 0, "axis": 0, "glAB": None}
    _kind = SHAPE_WALL

    @staticmethod
    def make(position, axis, sense=0, **kw):
        from . import utils
        return utils.wall(position, axis=axis, sense=sense, **kw)


class Facet(Shape):
    _attrs = {"fakeVel": lambda: np.zeros(3), "halfThick": 0.0}
    _kind = SHAPE_FACET

    def getNormal(self):
        p = [np.asarray(n.pos) for n in self.nodes]
        nn = np.cross(p[1] - p[0], p[2] - p[0])
        return nn / np.linalg.norm(nn)

    @staticmethod
    def make(vertices, **kw):
        from . import utils
        return utils.facet(vertices, **kw)


class Material(Object):
    _attrs = {"density": 1000.0, "id": -1}


class ElastMat(Material):
    _attrs = {"young": 1e9}


class FrictMat(ElastMat):
    """pkg/dem/FrictMat.hpp:18-28"""
    _attrs = {"tanPhi": 0.5, "ktDivKn": 0.2}


# ------------------------------------------------------------------ particles
_PAR_SPEC = {
    "shape": (np.int32, (), 0), "nodes": (np.int32, (3,), -1), "radius": (np.float64, (), 0.0),
    "axis": (np.int32, (), 0), "sense": (np.int32, (), 0), "halfThick": (np.float64, (), 0.0),
    "fakeVel": (np.float64, (3,), 0.0), "mat": (np.int32, (), 0), "mask": (np.uint32, (), 1),
}


class Particle(Object):
    """pkg/dem/Particle.hpp:26-123. Created detached by utils.sphere/wall/facet; after
    ``S.dem.par.add`` it reads and writes the container columns."""

    _attrs = {"mask": 1, "shape": None, "material": None, "aspherical": False}

    def __init__(self, **kw):
        object.__setattr__(self, "_cont", None)
        object.__setattr__(self, "_i", -1)
        super().__init__(**kw)

    # ``mat`` is the python alias of ``material``
    mat = property(lambda s: s.material, lambda s, v: setattr(s, "material", v))

    @property
    def id(self):
        return self._i

    def __setattr__(self, k, v):
        if k == "mask" and self.__dict__.get("_cont") is not None:
            self._cont._set_mask(self._i, v)
        object.__setattr__(self, k, v)

    def _node0(self):
        nn = self.shape.nodes
        if len(nn) != 1:
            raise RuntimeError("Particle #%d is not uninodal" % self.id)
        return nn[0]

    pos = property(lambda s: s._node0().pos, lambda s, v: setattr(s._node0(), "pos", v))
    ori = property(lambda s: s._node0().ori, lambda s, v: setattr(s._node0(), "ori", v))
    vel = property(lambda s: s._node0().dem.vel, lambda s, v: setattr(s._node0().dem, "vel", v))
    angVel = property(lambda s: s._node0().dem.angVel, lambda s, v: setattr(s._node0().dem, "angVel", v))
    mass = property(lambda s: s._node0().dem.mass)
    inertia = property(lambda s: s._node0().dem.inertia)
    f = property(lambda s: s._node0().dem.force)
    t = property(lambda s: s._node0().dem.torque)
    blocked = property(lambda s: s._node0().dem.blocked, lambda s, v: setattr(s._node0().dem, "blocked", v))
    nodes = property(lambda s: s.shape.nodes)

    @property
    def Ekt(self):
        return 0.5 * self.mass * float(np.dot(self.vel, self.vel))

    @property
    def Ekr(self):
        w = np.asarray(self.angVel)
        return 0.5 * float(np.dot(w, np.asarray(self.inertia) * w))

    @property
    def Ek(self):
        return self.Ekt + self.Ekr

    @property
    def con(self):
        return [c.id2 if c.id1 == self.id else c.id1 for c in self._cont.field.con._real_of(self.id)]

    @property
    def contacts(self):
        return {(c.id2 if c.id1 == self.id else c.id1): c for c in self._cont.field.con._real_of(self.id)}

    def updateMassInertia(self):
        """Shape::lumpMassInertia for the uninodal shapes (pkg/dem/Sphere.cpp:24-31, Wall.cpp:18-22)."""
        if isinstance(self.shape, Sphere):
            n = self.shape.nodes[0]
            m = (4 / 3.0) * math.pi * self.shape.radius ** 3 * self.material.density
            n.dem.mass = m
            n.dem.inertia = np.full(3, (2.0 / 5.0) * m * self.shape.radius ** 2)


class ParticleContainer:
    """S.dem.par (pkg/dem/ParticleContainer.hpp:47-210), structure-of-arrays backed."""

    def __init__(self, field):
        self.field = field
        self.soa = SoA(_PAR_SPEC)
        self._objs = {}
        self._shapes = {}

    def __len__(self):
        return len(self.soa)

    def _mat_index(self, m):
        return self.field._mat_index(m)

    def add(self, p, nodes=True):
        if isinstance(p, (list, tuple)):
            return [self.add(x) for x in p]
        if p._cont is not None:
            raise ValueError("Particle already in a container (id %d)" % p.id)
        sh = p.shape
        if sh is None or not hasattr(sh, "_kind"):
            raise ValueError("Unsupported shape %r: the GPU path handles Sphere, Wall and Facet" % (sh,))
        store = self.field._nodes
        idx = [store.adopt(n) for n in sh.nodes]
        if len(idx) != (3 if sh._kind == SHAPE_FACET else 1):
            raise ValueError("%s must have %d nodes" % (type(sh).__name__, 3 if sh._kind == SHAPE_FACET else 1))
        rec = dict(shape=sh._kind, nodes=idx + [-1] * (3 - len(idx)), mat=self._mat_index(p.material), mask=p.mask)
        if sh._kind == SHAPE_SPHERE:
            rec["radius"] = sh.radius
        elif sh._kind == SHAPE_WALL:
            rec["axis"], rec["sense"] = sh.axis, sh.sense
        else:
            rec["halfThick"] = sh.halfThick
            rec["fakeVel"] = np.asarray(sh.fakeVel, dtype=float)
        i = self.soa.append(1, **rec)
        object.__setattr__(p, "_cont", self)
        object.__setattr__(p, "_i", i)
        self._objs[i] = p
        self.field._structure_changed()
        return i

    def addSpheres(self, centers, radii, mat, mask=0b0101, fixed=False):
        """Bulk counterpart of ``add([utils.sphere(c, r, mat=mat) ...])`` for large scenes.
        Returns the id range. Mass and inertia follow Sphere::lumpMassInertia (pkg/dem/Sphere.cpp:24-31)."""
        centers = np.asarray(centers, dtype=float).reshape(-1, 3)
        radii = np.broadcast_to(np.asarray(radii, dtype=float), (len(centers),)).copy()
        n = len(centers)
        m = (4 / 3.0) * math.pi * radii ** 3 * mat.density
        inertia = np.repeat(((2.0 / 5.0) * m * radii ** 2)[:, None], 3, axis=1)
        nodes = self.field._nodes.soa
        n0 = nodes.append(n, pos=centers, ori=np.array([1.0, 0, 0, 0]), mass=m, inertia=inertia,
                          flags=np.uint32(DOF_ALL if fixed else 0))
        nidx = np.full((n, 3), -1, dtype=np.int32)
        nidx[:, 0] = np.arange(n0, n0 + n, dtype=np.int32)
        start = self.soa.append(n, shape=SHAPE_SPHERE, nodes=nidx, radius=radii, mat=self._mat_index(mat), mask=mask)
        self.field._structure_changed()
        return range(start, start + n)

    def __getitem__(self, i):
        if i < 0:
            i += len(self)
        if not 0 <= i < len(self):
            raise IndexError("Particle id out of range")
        p = self._objs.get(i)
        if p is None:
            p = self._make_view(i)
            self._objs[i] = p
        return p

    def _make_view(self, i):
        s = self.soa
        kind = int(s.col("shape")[i])
        store = self.field._nodes
        nodes = []
        for ni in s.col("nodes")[i]:
            if ni < 0:
                continue
            nd = Node.__new__(Node)
            object.__setattr__(nd, "_store", store)
            object.__setattr__(nd, "_i", int(ni))
            object.__setattr__(nd, "_rec", None)
            nodes.append(nd)
        if kind == SHAPE_SPHERE:
            sh = Sphere(radius=float(s.col("radius")[i]))
        elif kind == SHAPE_WALL:
            sh = Wall(axis=int(s.col("axis")[i]), sense=int(s.col("sense")[i]))
        else:
            sh = Facet(halfThick=float(s.col("halfThick")[i]), fakeVel=s.col("fakeVel")[i].copy())
        sh.nodes = nodes
        p = Particle(shape=sh, material=self.field._mats[int(s.col("mat")[i])], mask=int(s.col("mask")[i]))
        object.__setattr__(p, "_cont", self)
        object.__setattr__(p, "_i", i)
        return p

    def _set_mask(self, i, v):
        self.soa.col("mask")[i] = v
        self.field._structure_changed()

    def __iter__(self):
        for i in range(len(self)):
            yield self[i]

    def exists(self, i):
        return 0 <= i < len(self)

    def clear(self):
        self.soa.clear()
        self._objs.clear()
        self.field._nodes.soa.clear()
        self.field._structure_changed()


# ------------------------------------------------------------------ contacts (device-backed views)
class Contact:
    """Read-only view of one contact (pkg/dem/Contact.hpp:47-116) fetched from the device."""

    __slots__ = ("id1", "id2", "idA", "real", "cellDist", "_f", "_loc", "_cp", "_trsf")

    def __init__(self, id1, id2, idA, real, cellDist, f, loc, cp, trsf):
        self.id1, self.id2, self.idA, self.real = int(id1), int(id2), int(idA), bool(real)
        self.cellDist, self._f, self._loc, self._cp, self._trsf = cellDist, f, loc, cp, trsf

    @property
    def ids(self):
        return (min(self.id1, self.id2), max(self.id1, self.id2))

    @property
    def force(self):
        """Global force acting on particle pA."""
        return self._f

    @property
    def phys(self):
        class _P:
            pass
        ph = _P()
        ph.force = self._loc
        return ph

    @property
    def geom(self):
        class _G:
            pass
        g = _G()
        g.trsf = self._trsf.reshape(3, 3)
        g.contPt = self._cp
        return g


class ContactContainer:
    """S.dem.con (pkg/dem/ContactContainer.hpp). Iteration yields real contacts only, like the reference."""

    def __init__(self, field):
        self.field = field

    def _fetch(self):
        return self.field._contacts_snapshot()

    def __len__(self):
        return len(self._fetch()["id_lo"])

    def _view(self, d, i):
        return Contact(d["id_lo"][i], d["id_hi"][i], d["id_a"][i], d["real"][i], d["cell_dist"][i], d["fglob"][i],
                       d["local"][i], d["cpt"][i], d["trsf"][i])

    def __iter__(self):
        d = self._fetch()
        for i in np.nonzero(d["real"])[0]:
            yield self._view(d, i)

    def __getitem__(self, k):
        d = self._fetch()
        if isinstance(k, tuple):
            lo, hi = min(k), max(k)
            hit = np.nonzero((d["id_lo"] == lo) & (d["id_hi"] == hi))[0]
            if len(hit) == 0:
                raise IndexError("No contact ##%d+%d" % (lo, hi))
            return self._view(d, hit[0])
        n = len(d["id_lo"])
        if k < 0:
            k += n
        return self._view(d, k)

    def _real_of(self, pid):
        d = self._fetch()
        sel = np.nonzero(d["real"].astype(bool) & ((d["id_lo"] == pid) | (d["id_hi"] == pid)))[0]
        return [self._view(d, i) for i in sel]

    def countReal(self):
        return int(np.count_nonzero(self._fetch()["real"]))

    def realRatio(self):
        n = len(self)
        return self.countReal() / n if n else 0.0

    def exists(self, a, b):
        d = self._fetch()
        lo, hi = min(a, b), max(a, b)
        return bool(np.any((d["id_lo"] == lo) & (d["id_hi"] == hi)))

    def existsReal(self, a, b):
        d = self._fetch()
        lo, hi = min(a, b), max(a, b)
        return bool(np.any((d["id_lo"] == lo) & (d["id_hi"] == hi) & (d["real"] != 0)))


class DemField(Field):
    """pkg/dem/Particle.hpp:278-340."""

    defaultMovableMask = 0b0101
    defaultBoundaryMask = 0b0011
    defaultLoneMask = 0b0010
    defaultInletMask = 0b0101
    defaultOutletMask = 0b0100

    def __init__(self, gravity=(0, 0, 0), loneMask=0b0010, par=None, **kw):
        self._nodes = _NodeStore(self)
        self._mats = []
        self._mat_ids = {}
        self.scene = None
        self.par = ParticleContainer(self)
        self.con = ContactContainer(self)
        self._gravity = np.array(gravity, dtype=float)
        self.loneMask = loneMask
        super().__init__(**kw)
        if par:
            self.par.add(list(par))

    gravity = property(lambda s: s._gravity, lambda s, v: setattr(s, "_gravity", np.array(v, dtype=float)))

    @property
    def nodes(self):
        return [self.par[i].shape.nodes[0] for i in range(len(self.par))]

    def collectNodes(self):
        return 0

    def __setstate__(self, d):
        # materials are indexed by object identity, which unpickling changes
        self.__dict__.update(d)
        self._mat_ids = {id(m): i for i, m in enumerate(self._mats)}

    def _mat_index(self, m):
        if m is None:
            raise ValueError("Particle without material")
        k = id(m)
        if k not in self._mat_ids:
            self._mat_ids[k] = len(self._mats)
            self._mats.append(m)
        return self._mat_ids[k]

    # hooks into the device simulation owned by the scene
    def _sim(self):
        sc = self.scene
        return None if sc is None else sc._sim

    def _pull_state(self):
        if self.scene is not None:
            self.scene.sync()  # under the scene's lock: a background run pauses between chunks

    def _state_written(self):
        s = self._sim()
        if s is not None:
            s.host_written = True

    def _structure_changed(self):
        s = self._sim()
        if s is not None:
            s.dirty_structure = True

    def _contacts_snapshot(self):
        if self.scene is not None:
            with self.scene._lock():
                return self._contacts_snapshot_locked()
        return self._contacts_snapshot_locked()

    def _contacts_snapshot_locked(self):
        s = self._sim()
        if s is None:
            z = np.zeros(0, dtype=np.int32)
            zf = np.zeros((0, 3))
            return dict(id_lo=z, id_hi=z, id_a=z, real=z, cell_dist=np.zeros((0, 3), np.int32), fglob=zf, local=zf, cpt=zf,
                        trsf=np.zeros((0, 9)))
        return s.contacts()


# ------------------------------------------------------------------ functors
class Functor(Object):
    _attrs = {"label": ""}


class BoundFunctor(Functor):
    pass


class Bo1_Sphere_Aabb(BoundFunctor):
    """pkg/dem/Sphere.hpp:33-41"""
    _attrs = {"distFactor": -1.0}


class Bo1_Facet_Aabb(BoundFunctor):
    pass


class Bo1_Wall_Aabb(BoundFunctor):
    pass


class CGeomFunctor(Functor):
    pass


class Cg2_Any_Any_L6Geom__Base(CGeomFunctor):
    """pkg/dem/L6Geom.hpp:28-48"""
    _attrs = {"noRatch": False, "trsfRenorm": 100, "approxMask": 0}


class Cg2_Sphere_Sphere_L6Geom(Cg2_Any_Any_L6Geom__Base):
    _attrs = {"distFactor": 1.0}


class Cg2_Facet_Sphere_L6Geom(Cg2_Any_Any_L6Geom__Base):
    pass


class Cg2_Wall_Sphere_L6Geom(Cg2_Any_Any_L6Geom__Base):
    pass


class CPhysFunctor(Functor):
    pass


class Cp2_FrictMat_FrictPhys(CPhysFunctor):
    """pkg/dem/FrictMat.hpp:43-53"""
    _attrs = {"tanPhi": None}


class Cp2_FrictMat_HertzPhys(Cp2_FrictMat_FrictPhys):
    """pkg/dem/Hertz.hpp:23-34"""
    _attrs = {"poisson": 0.2, "gamma": 0.0, "en": NaN, "alpha": 0.0}


class LawFunctor(Functor):
    pass


class Law2_L6Geom_FrictPhys_IdealElPl(LawFunctor):
    """pkg/dem/IdealElPl.hpp:6-28"""
    _attrs = {"iniEqlb": False, "relRollStiff": 0.0, "relTwistStiff": 0.0, "rollTanPhi": 0.0, "noSlip": False,
              "noBreak": False, "noFrict": False}


class Law2_L6Geom_HertzPhys_DMT(LawFunctor):
    """pkg/dem/Hertz.hpp:39-77"""
    _attrs = {"noAttraction": True}


# Functors that utils.defaultEngines lists for shapes outside this path; accepted in the
# functor lists, they can never be dispatched because those shapes cannot be created here.
class _InertFunctor(Functor):
    pass


for _n in ("Bo1_InfCylinder_Aabb", "Bo1_Ellipsoid_Aabb", "Bo1_Rod_Aabb", "Bo1_Capsule_Aabb",
           "Cg2_InfCylinder_Sphere_L6Geom", "Cg2_Ellipsoid_Ellipsoid_L6Geom", "Cg2_Sphere_Ellipsoid_L6Geom",
           "Cg2_Wall_Ellipsoid_L6Geom", "Cg2_Wall_Facet_L6Geom", "Cg2_Rod_Sphere_L6Geom", "Cg2_Wall_Capsule_L6Geom",
           "Cg2_Capsule_Capsule_L6Geom", "Cg2_InfCylinder_Capsule_L6Geom", "Cg2_Facet_Capsule_L6Geom",
           "Cg2_Sphere_Capsule_L6Geom", "Cg2_Facet_Facet_L6Geom", "Cg2_Facet_InfCylinder_L6Geom"):
    globals()[_n] = type(_n, (_InertFunctor, BoundFunctor if _n.startswith("Bo1_") else CGeomFunctor), {})


# ------------------------------------------------------------------ dispatchers
class Dispatcher(list):
    """The functors of one dispatcher (core/Dispatcher.hpp:40-52): a list that is also the
    reference's dispatcher object, with ``functors`` and ``add``. Functors of another kind raise
    TypeError; a functor of a class already present is not added again (the first one stays)."""
    _functorType = Functor

    def __init__(self, functors=()):
        super().__init__()
        self.functors = functors

    @property
    def functors(self):
        return list(self)

    @functors.setter
    def functors(self, ff):
        del self[:]
        for f in ff:
            self.add(f)

    def add(self, f):
        if not isinstance(f, self._functorType):
            raise TypeError("%s accepts %s functors only, not %s" % (type(self).__name__, self._functorType.__name__,
                                                                      type(f).__name__))
        if not any(type(g).__name__ == type(f).__name__ for g in self):
            list.append(self, f)

    def __repr__(self):
        return "%s(%s)" % (type(self).__name__, list.__repr__(self))


class BoundDispatcher(Dispatcher):
    _functorType = BoundFunctor


class CGeomDispatcher(Dispatcher):
    _functorType = CGeomFunctor


class CPhysDispatcher(Dispatcher):
    _functorType = CPhysFunctor


class LawDispatcher(Dispatcher):
    _functorType = LawFunctor


def _dispatcherAttr(name, cls):
    key = "_" + name
    return property(lambda self: self.__dict__[key],
                    lambda self, v: self.__dict__.__setitem__(key, v if type(v) is cls else cls(v)))


# ------------------------------------------------------------------ engines
class Leapfrog(Engine):
    """pkg/dem/Leapfrog.hpp:42-61"""
    _attrs = {"damping": 0.2, "reset": False, "kinSplit": False, "dontCollect": False, "maxVelocitySq": NaN}


class ForceResetter(Engine):
    pass


class Collider(Engine):
    pass


class InsertionSortCollider(Collider):
    """pkg/dem/InsertionSortCollider.hpp:252-265. ``nFullRuns`` is read back from the device."""
    _attrs = {"forceInitSort": False, "noBoundOk": False, "sortAxis": 0, "sortThenCollide": False, "verletDist": -0.05,
              "maxVel2": 0.0, "nFullRuns": 0, "numReinit": 0, "ompTuneSort": (1, 1000, 0), "sortChunks": -1,
              "paraPeri": False,
              "boundDispatcher": lambda: [Bo1_Sphere_Aabb(), Bo1_Facet_Aabb(), Bo1_Wall_Aabb()]}
    boundDispatcher = _dispatcherAttr("boundDispatcher", BoundDispatcher)

    def __init__(self, boundFunctors=None, **kw):
        super().__init__(**kw)
        if boundFunctors:
            self.boundDispatcher = list(boundFunctors)

    def _functors(self):
        return list(self.boundDispatcher)


class ContactLoop(Engine):
    """pkg/dem/ContactLoop.hpp:108-124; special constructor ContactLoop([Cg2],[Cp2],[Law2])."""
    _attrs = {"evalStress": False, "applyForces": True, "updatePhys": False, "dist00": True, "reorderEvery": 1000,
              "alreadyWarnedNoCollider": False, "geoDisp": lambda: [], "phyDisp": lambda: [], "lawDisp": lambda: [],
              "stress": lambda: np.zeros((3, 3))}
    geoDisp = _dispatcherAttr("geoDisp", CGeomDispatcher)
    phyDisp = _dispatcherAttr("phyDisp", CPhysDispatcher)
    lawDisp = _dispatcherAttr("lawDisp", LawDispatcher)

    def __init__(self, geoms=None, physs=None, laws=None, **kw):
        super().__init__(**kw)
        if (geoms is None) != (laws is None):
            raise ValueError("Exactly 3 lists of functors must be given")
        if geoms is not None:
            self.geoDisp = list(geoms)
            self.phyDisp = list(physs or [])
            self.lawDisp = list(laws)

    def _functors(self):
        return self.geoDisp + self.phyDisp + self.lawDisp


class VtkExport(PeriodicEngine):
    """Writes the scene to VTK XML files when due (pkg/dem/VtkExport.hpp:30-90): spheres, meshes
    (facets, walls with glAB) and contacts, named ``{out}spheres.{step}.vtu``,
    ``{out}mesh.{step}.vtu`` and ``{out}con.{step}.vtp``; ``out`` may hold ``{tag}`` fields of
    Scene.tags. Runs on the host between queued device steps (woodem_gb300.vtk); the files are
    ASCII XML (``compress``/``ascii`` are accepted, multiblock output is not built)."""
    spheres, mesh, con, tri, all = 1, 2, 4, 8, 15
    _attrs = {"out": "", "compress": True, "ascii": False, "multiblock": False, "mask": 0, "what": 15,
              "sphereSphereOnly": False, "infError": True, "skipInvisible": True, "subdiv": 16, "thickFacetDiv": 1,
              "nanValue": 0.0, "outFiles": lambda: {}, "outTimes": lambda: [], "outSteps": lambda: []}
    _host = True

    def _runHost(self, S, step, time):
        from . import vtk
        if self.multiblock:
            raise NotImplementedError("VtkExport.multiblock is not built")
        S.sync()
        files = vtk.export(S, S._sim.contacts(), out=self.out, what=self.what, mask=self.mask,
                           sphereSphereOnly=self.sphereSphereOnly, infError=self.infError, nanValue=self.nanValue, step=step)
        for k, f in files.items():
            self.outFiles.setdefault(k, []).append(f)
        self.outTimes.append(time)
        self.outSteps.append(step)


class DynDt(PeriodicEngine):
    """Adjusts Scene.dt from the current stiffness of the contacts (pkg/dem/DynDt.hpp:5-25), as the
    engine after ContactLoop: the critical timestep is evaluated on the device, the new dt
    (dtSafety times it, growing by at most maxRelInc per step) takes effect after the step. With
    dryRun, only ``dt`` is set. FP64 precision mode; stepPeriod/virtPeriod activation."""
    _attrs = {"maxRelInc": 1e-4, "dryRun": False, "dt": NaN}
