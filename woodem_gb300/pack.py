"""``woo.pack`` counterpart: SpherePack, the sphere-packing container that scene scripts fill with
``makeCloud`` and hand to a scene with ``toSimulation`` (lib/sphere-pack/SpherePack.hpp:20-140,
lib/sphere-pack/SpherePack.cpp, py/pack.py:104-160).

Radii follow the reference's rules (a mean radius with a relative fuzz, a target count with a
porosity, or a piecewise-linear size distribution, by number or by mass); the spheres are placed
by the native random sequential insertion of ``wg_pack_rsa`` (woodem_gb300/csrc/wg_pack.cpp: up to
1000 candidate centres per sphere, uniformly in the box or the periodic cell, the first free one
accepted), so a packing of a million spheres takes seconds. The random stream is this library's
own (seeded), not the reference's.
"""
import math
import time

import numpy as np

from . import _native

RDIST_RMEAN, RDIST_NUM, RDIST_PSD = 0, 1, 2
MAX_TRY = 1000


def _rsa(radii, lo, hi, periodic, seed):
    """Place ``radii`` in the given order; returns the centres of the spheres placed (a prefix)."""
    r = np.ascontiguousarray(radii, dtype=float)
    out = np.zeros((len(r), 3))
    lo = np.ascontiguousarray(lo, dtype=float)
    hi = np.ascontiguousarray(hi, dtype=float)
    n = _native.lib().wg_pack_rsa(len(r), _native.ptr(r), _native.ptr(lo), _native.ptr(hi), 2 if periodic else 0,
                                  _native.ptr(np.zeros(4)), int(seed), MAX_TRY, _native.ptr(out))
    return out[:max(0, int(n))]


def _psdGetPiece(x, cumm):
    """SpherePack::psdGetPiece (SpherePack.cpp:283-291): the piece of the piecewise function with
    non-decreasing knots ``cumm`` that holds x, and x's normalised coordinate in it."""
    sz, i = len(cumm), 0
    while i < sz and cumm[i] <= x:
        i += 1
    if i == sz - 1 and cumm[i] <= x:
        return sz - 2, 1.0
    i -= 1
    return i, (x - cumm[i]) / (cumm[i + 1] - cumm[i])


def _pow3Interp(x, a, b):
    """Radius with a power-law (-3) distribution between a and b for uniform x in (0,1)."""
    return (x * (b ** -2 - a ** -2) + a ** -2) ** -0.5


class SpherePack:
    """Spheres (centre, radius) and, for a periodic packing, the cell size."""

    def __init__(self, lst=None):
        self.pack = []  # (centre as a 3-array, radius, clumpId)
        self.cellSize = np.zeros(3)
        self.userData = ""
        self.appliedPsdScaling = 1.0
        if lst is not None:
            self.fromList(lst)

    # container
    def reset(self):
        self.pack = []
        self.cellSize = np.zeros(3)
        self.userData = ""

    def add(self, c, r, clumpId=-1):
        self.pack.append((np.asarray(c, dtype=float).copy(), float(r), int(clumpId)))

    def __len__(self):
        return len(self.pack)

    def __iter__(self):
        return iter([(c, r) for c, r, _ in self.pack])

    def __getitem__(self, i):
        c, r, _ = self.pack[i]
        return (c, r)

    def fromList(self, lst):
        self.pack = []
        for item in lst:
            self.add(item[0], item[1], item[2] if len(item) > 2 else -1)

    def fromLists(self, centers, radii):
        if len(centers) != len(radii):
            raise ValueError("The same number of centers and radii must be given (%d != %d)" % (len(centers), len(radii)))
        self.pack = []
        for c, r in zip(centers, radii):
            self.add(c, r)

    def toList(self):
        return [(c, r, k) if k >= 0 else (c, r) for c, r, k in self.pack]

    def toCcRr(self):
        """(centres as an n×3 array, radii)."""
        return (np.array([c for c, _, _ in self.pack]).reshape(-1, 3), np.array([r for _, r, _ in self.pack]))

    def hasClumps(self):
        return any(k >= 0 for _, _, k in self.pack)

    def isPeriodic(self):
        return bool(np.any(self.cellSize != 0))

    def sphereVol(self):
        return (4 / 3.) * math.pi * sum(r ** 3 for _, r, _ in self.pack)

    def aabb(self):
        if not self.pack:
            return np.zeros(3), np.zeros(3)
        cc, rr = self.toCcRr()
        return (cc - rr[:, None]).min(axis=0), (cc + rr[:, None]).max(axis=0)

    def dim(self):
        mn, mx = self.aabb()
        return mx - mn

    # files (SpherePack::toFile/fromFile, SpherePack.cpp:73-130): "x y z r [clumpId]" per line,
    # "##PERIODIC:: sx sy sz" and "##USER-DATA:: ..." header lines
    def toFile(self, fname):
        if "\n" in self.userData:
            raise RuntimeError("SpherePack.userData must not contain newline.")
        clumps = self.hasClumps()
        with open(fname, "w") as f:
            if self.isPeriodic():
                f.write("##PERIODIC:: %r %r %r\n" % tuple(float(x) for x in self.cellSize))
            if self.userData:
                f.write("##USER-DATA:: %s\n" % self.userData)
            for c, r, k in self.pack:
                f.write("%r %r %r %r" % (float(c[0]), float(c[1]), float(c[2]), r) + (" %d" % k if clumps else "") + "\n")

    def fromFile(self, fname):
        import os
        if not os.path.exists(fname):
            raise ValueError("File with spheres `%s' doesn't exist." % fname)
        self.reset()
        with open(fname) as f:
            for lineNo, line in enumerate(f, 1):
                if line.startswith("##USER-DATA:: "):
                    self.userData = line[14:].rstrip("\n")
                    continue
                tok = line.split()
                if not tok:
                    continue
                if tok[0] == "##PERIODIC::":
                    if len(tok) != 4:
                        raise ValueError("Spheres file %s:%d contains ##PERIODIC::, but the line is malformed." % (fname, lineNo))
                    self.cellSize = np.array([float(t) for t in tok[1:]])
                    continue
                if len(tok) not in (4, 5):
                    raise ValueError("Spheres file %s:%d has %d columns (4 or 5 expected)." % (fname, lineNo, len(tok)))
                self.add([float(t) for t in tok[:3]], float(tok[3]), int(tok[4]) if len(tok) == 5 else -1)

    def cellRepeat(self, count):
        """Repeat a periodic packing count[i] times along each axis (SpherePack.cpp:264-281)."""
        if not self.isPeriodic():
            raise RuntimeError("cellRepeat cannot be used on non-periodic packing.")
        count = [int(x) for x in count]
        if min(count) <= 0:
            raise ValueError("Repeat count components must be positive.")
        orig = list(self.pack)
        for i in range(count[0]):
            for j in range(count[1]):
                for k in range(count[2]):
                    if i == j == k == 0:
                        continue
                    off = self.cellSize * np.array([i, j, k])
                    for c, r, _ in orig:
                        self.add(c + off, r)
        self.cellSize = self.cellSize * np.array(count)

    def psd(self, bins=10, mass=False):
        """(diameter bin edges, cumulative fraction passing) by number or by mass (SpherePack.cpp:293-311)."""
        if not self.pack:
            return [], []
        d = np.array([2 * r for _, r, _ in self.pack])
        minD, maxD = float(d.min()), float(d.max())
        if minD == maxD:
            minD, maxD = minD - .5, maxD + .5
        edges = [minD + i * (maxD - minD) / bins for i in range(bins + 1)]
        vol = float(np.sum((d / 2) ** 3))
        hist = np.zeros(bins)
        for x in d:
            b = min(int(bins * (x - minD) / (maxD - minD)), bins - 1)
            hist[b] += ((x / 2) ** 3 / vol) if mass else 1.0 / len(d)
        cumm = [0.0]
        for i in range(bins):
            cumm.append(min(1.0, cumm[-1] + hist[i]))
        return edges, cumm

    # generation
    def makeCloud(self, minCorner=(0, 0, 0), maxCorner=(0, 0, 0), rMean=-1, rRelFuzz=0, num=-1, periodic=False, porosity=-1,
                  psdSizes=(), psdCumm=(), distributeMass=False, seed=0, hSize=None):
        """Random loose packing (SpherePack::makeCloud, SpherePack.cpp:135-246): spheres in the box
        [minCorner, maxCorner] (or a periodic cell of that size), radii from ``rMean`` and
        ``rRelFuzz``, or from ``num`` and ``porosity``, or from the size distribution ``psdSizes``
        (diameters) / ``psdCumm`` (cumulative fraction, by mass with ``distributeMass``). With
        ``num`` > 0 the radii are the distribution's quantiles in decreasing order and a packing
        that does not fit is retried at a higher porosity with smaller spheres; with ``num`` < 0
        spheres are added until one cannot be placed. Returns the number of spheres."""
        if hSize is not None and np.any(np.asarray(hSize) != 0) and not np.allclose(np.asarray(hSize), np.diag(np.diag(hSize))):
            raise NotImplementedError("SpherePack.makeCloud with a non-diagonal hSize is not supported")
        mn = np.asarray(minCorner, dtype=float)
        mx = np.asarray(maxCorner, dtype=float)
        if hSize is not None and np.any(np.asarray(hSize) != 0):
            mx = mn + np.diag(np.asarray(hSize, dtype=float))
        size = mx - mn
        volume = float(np.prod(size))
        if volume == 0:
            raise ValueError("The box defined as null volume. Define at least maxCorner of the box, or hSize if periodic.")
        psdSizes, psdCumm = list(psdSizes), list(psdCumm)
        if porosity <= 0:
            porosity = 0.5
        mode, err = -1, False
        if rMean > 0:
            mode = RDIST_RMEAN
        elif num > 0 and not psdSizes:
            mode = RDIST_NUM
            rMean = (volume * (1 - porosity) / (math.pi * (4 / 3.) * (1 + rRelFuzz * rRelFuzz) * num)) ** (1 / 3.)
        psdRadii, psdCumm2 = [], []
        self.appliedPsdScaling = 1.0
        if psdSizes:
            err = mode >= 0
            mode = RDIST_PSD
            if len(psdSizes) != len(psdCumm):
                raise ValueError("SpherePack.makeCloud: psdSizes and psdCumm must have same dimensions (%d!=%d)"
                                 % (len(psdSizes), len(psdCumm)))
            if len(psdSizes) <= 1:
                raise ValueError("SpherePack.makeCloud: psdSizes must have at least 2 items")
            if psdCumm[0] != 0. and psdCumm[-1] != 1.:
                raise ValueError("SpherePack.makeCloud: first and last items of psdCumm *must* be exactly 0 and 1.")
            for i in range(len(psdSizes)):
                psdRadii.append(.5 * psdSizes[i])
                if distributeMass:
                    if i == 0:
                        psdCumm2.append(0.0)
                    else:
                        psdCumm2.append(psdCumm2[i - 1] + 3.0 * volume * (1 - porosity) / math.pi * (psdCumm[i] - psdCumm[i - 1])
                                        / (psdSizes[i] - psdSizes[i - 1]) * (psdSizes[i - 1] ** -2 - psdSizes[i] ** -2))
                if i > 0 and (psdSizes[i - 1] > psdSizes[i] or psdCumm[i - 1] > psdCumm[i]):
                    raise ValueError("SpherePack:makeCloud: psdSizes and psdCumm must be both non-decreasing.")
            if distributeMass:
                if num > 0 and psdCumm2[-1] < num:
                    self.appliedPsdScaling = (psdCumm2[-1] / num) ** (1. / 3.)
                    psdRadii = [r * self.appliedPsdScaling for r in psdRadii]
                psdCumm2 = [c / psdCumm2[-1] for c in psdCumm2]
        if err or mode < 0:
            raise ValueError("SpherePack.makeCloud: at least one of rMean, porosity, psdSizes & psdCumm arguments must be "
                             "specified. rMean can't be combined with psdSizes.")

        def radius(u):
            if mode in (RDIST_RMEAN, RDIST_NUM):
                if distributeMass:
                    return _pow3Interp(u, rMean * (1 - rRelFuzz), rMean * (1 + rRelFuzz))
                return rMean * (2 * (u - .5) * rRelFuzz + 1)
            if distributeMass:
                p, nrm = _psdGetPiece(u, psdCumm2)
                return _pow3Interp(nrm, psdRadii[p], psdRadii[p + 1])
            p, nrm = _psdGetPiece(u, psdCumm)
            return psdRadii[p] + nrm * (psdRadii[p + 1] - psdRadii[p])

        if seed == 0:
            seed = int(time.time() * 1e6) & 0x7fffffff
        rng = np.random.default_rng(seed)
        if num > 0:
            radii = [radius((num - i + 0.5) / (num + 1.)) for i in range(num)]
        else:
            # as many as fit: at most the box volume in spheres of the smallest radius drawn
            draws = rng.uniform(0, 1, 4096)
            rmin = max(min(radius(u) for u in draws), 1e-300)
            cap = int(min(2e7, volume / ((4 / 3.) * math.pi * rmin ** 3) + 16))
            radii = [radius(u) for u in rng.uniform(0, 1, cap)]
        if any(2 * r > s for r in radii[:1] for s in size):
            raise ValueError("SpherePack.makeCloud: spheres (r=%g) larger than the box" % max(radii))
        centres = _rsa(radii, mn, mx, periodic, seed)
        if num > 0 and len(centres) < num and mode != RDIST_RMEAN:
            # Exceeded the tries: retry with a higher porosity (SpherePack.cpp:235-243)
            return self.makeCloud(mn, mx, -1., rRelFuzz, num, periodic, porosity + (1 - porosity) / 10., psdSizes, psdCumm,
                                  distributeMass, seed + 1)
        if periodic:
            self.cellSize = size.copy()
        for c, r in zip(centres, radii):
            self.add(c, r)
        return len(self.pack)

    def fromSimulation(self, scene, dem=None):
        """Reset and fill from the spheres of ``scene`` (py/pack.py:71-97): centres as of the
        last run, radii; a periodic scene gives cellSize = diag(hSize) and raises RuntimeError
        for a cell whose hSize is not symmetric (sheared)."""
        from .dem import SHAPE_SPHERE
        self.reset()
        de = scene.dem if dem is None else dem
        scene.sync()
        par = de.par.soa
        sel = np.nonzero(np.asarray(par.col("shape")) == SHAPE_SPHERE)[0]
        pos = np.asarray(de._nodes.soa.col("pos"))[np.asarray(par.col("nodes"))[sel, 0]]
        for c, r in zip(pos, np.asarray(par.col("radius"))[sel]):
            self.add(c, r)
        if scene.periodic:
            h = np.asarray(scene.cell.hSize, dtype=float)
            if np.any(h - h.T != 0):
                raise RuntimeError("Only box-shaped (no shear) periodic boundary conditions can be represented with a "
                                   "pack.SpherePack object")
            self.cellSize = h.diagonal().copy()
        return self

    def fromDem(self, scene, dem):
        return self.fromSimulation(scene, dem)

    def toSimulation(self, scene, rot=None, **kw):
        """Add the spheres to ``scene`` (py/pack.py:104-160); a periodic packing makes the scene
        periodic with cell hSize = rot·diag(cellSize) and trsf the identity. ``rot``: a 3×3 matrix
        or a quaternion (w, x, y, z); ``kw`` go to utils.sphere (``mat`` defaults to
        utils.defaultMaterial()). Returns the ids added."""
        from . import utils
        from .dem import _quat_wxyz
        if self.hasClumps():
            raise NotImplementedError("clumps are not part of the GPU path")
        R = np.eye(3)
        if rot is not None:
            rot = np.asarray(rot, dtype=float)
            if rot.shape == (4,):
                w, x, y, z = _quat_wxyz(rot)
                R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                              [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                              [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
            else:
                R = rot.reshape(3, 3)
        if self.isPeriodic():
            scene.periodic = True
            scene.cell.hSize = R @ np.diag(self.cellSize)
            scene.cell.trsf = np.eye(3)
        if "mat" not in kw:
            kw["mat"] = utils.defaultMaterial()
        return scene.dem.par.add([utils.sphere(R @ c, r, **kw) for c, r, _ in self.pack])


# --- predicates (py/_packPredicates.cpp:51-295): solids that say whether a sphere (centre,
# radius as the padding) lies inside them, with an axis-aligned bounding box; combined with
# | (union), & (intersection), - (difference) and ^ (symmetric difference).
_INF = float("inf")


class Predicate:
    def __call__(self, pt, pad=0.0):
        raise NotImplementedError

    def aabb(self):
        raise NotImplementedError

    def center(self):
        mn, mx = self.aabb()
        return 0.5 * (np.asarray(mn) + np.asarray(mx))

    def dim(self):
        mn, mx = self.aabb()
        return np.asarray(mx) - np.asarray(mn)

    def __or__(self, B):
        return PredicateUnion(self, B)

    def __and__(self, B):
        return PredicateIntersection(self, B)

    def __sub__(self, B):
        return PredicateDifference(self, B)

    def __xor__(self, B):
        return PredicateSymmetricDifference(self, B)


class _PredicateBoolean(Predicate):
    def __init__(self, A, B):
        self.A, self.B = A, B


class PredicateUnion(_PredicateBoolean):
    def __call__(self, pt, pad=0.0):
        return self.A(pt, pad) or self.B(pt, pad)

    def aabb(self):
        (a0, a1), (b0, b1) = self.A.aabb(), self.B.aabb()
        return np.minimum(a0, b0), np.maximum(a1, b1)


class PredicateIntersection(_PredicateBoolean):
    def __call__(self, pt, pad=0.0):
        return self.A(pt, pad) and self.B(pt, pad)

    def aabb(self):
        (a0, a1), (b0, b1) = self.A.aabb(), self.B.aabb()
        return np.maximum(a0, b0), np.minimum(a1, b1)


class PredicateDifference(_PredicateBoolean):
    """Inside A and not inside B, B tested with the opposite padding."""

    def __call__(self, pt, pad=0.0):
        return self.A(pt, pad) and not self.B(pt, -pad)

    def aabb(self):
        return self.A.aabb()


class PredicateSymmetricDifference(_PredicateBoolean):
    def __call__(self, pt, pad=0.0):
        return self.A(pt, pad) != self.B(pt, pad)

    def aabb(self):
        (a0, a1), (b0, b1) = self.A.aabb(), self.B.aabb()
        return np.minimum(a0, b0), np.maximum(a1, b1)


class inSphere(Predicate):
    """Centre within the sphere (the reference's test |pt-c|-pad <= radius-pad: the padding cancels)."""

    def __init__(self, center, radius):
        self.c, self.radius = np.asarray(center, dtype=float), float(radius)

    def __call__(self, pt, pad=0.0):
        return float(np.linalg.norm(np.asarray(pt, dtype=float) - self.c)) - pad <= self.radius - pad

    def aabb(self):
        return self.c - self.radius, self.c + self.radius


class inAlignedHalfspace(Predicate):
    def __init__(self, axis, coord, lower=True):
        if axis not in (0, 1, 2):
            raise RuntimeError("inAlignedHalfSpace.axis: must be in {0,1,2} (not %s)" % axis)
        self.axis, self.coord, self.lower = int(axis), float(coord), bool(lower)

    def __call__(self, pt, pad=0.0):
        return pt[self.axis] + pad < self.coord if self.lower else pt[self.axis] - pad > self.coord

    def aabb(self):
        mn, mx = np.full(3, -_INF), np.full(3, _INF)
        (mx if self.lower else mn)[self.axis] = self.coord
        return mn, mx


class inAxisRange(Predicate):
    def __init__(self, axis, range):
        if axis not in (0, 1, 2):
            raise RuntimeError("inAxisRange.axis: must be in {0,1,2} (not %s)" % axis)
        self.axis, self.range = int(axis), (float(range[0]), float(range[1]))

    def __call__(self, pt, pad=0.0):
        return pt[self.axis] - pad >= self.range[0] and pt[self.axis] + pad <= self.range[1]

    def aabb(self):
        mn, mx = np.full(3, -_INF), np.full(3, _INF)
        mn[self.axis], mx[self.axis] = self.range
        return mn, mx


class inAlignedBox(Predicate):
    def __init__(self, minAabb, maxAabb=None):
        if maxAabb is None:  # a (min, max) pair
            minAabb, maxAabb = minAabb
        self.mn, self.mx = np.asarray(minAabb, dtype=float), np.asarray(maxAabb, dtype=float)

    def __call__(self, pt, pad=0.0):
        return all(self.mn[i] + pad <= pt[i] and self.mx[i] - pad >= pt[i] for i in range(3))

    def aabb(self):
        return self.mn.copy(), self.mx.copy()


class inCylinder(Predicate):
    """Between the caps at centre1 and centre2 and within radius of their axis."""

    def __init__(self, centerBottom, centerTop, radius):
        self.c1, self.c2 = np.asarray(centerBottom, dtype=float), np.asarray(centerTop, dtype=float)
        self.radius = float(radius)
        self.c12 = self.c2 - self.c1
        self.ht = float(np.linalg.norm(self.c12))

    def __call__(self, pt, pad=0.0):
        pt = np.asarray(pt, dtype=float)
        u = (pt.dot(self.c12) - self.c1.dot(self.c12)) / (self.ht * self.ht)
        if u * self.ht < pad or u * self.ht > self.ht - pad:
            return False
        return float(np.linalg.norm(np.cross(pt - self.c1, pt - self.c2))) / self.ht <= self.radius - pad

    def aabb(self):
        A, B = self.c1, self.c2
        k = np.array([math.sqrt((A[1] - B[1]) ** 2 + (A[2] - B[2]) ** 2), math.sqrt((A[0] - B[0]) ** 2 + (A[2] - B[2]) ** 2),
                      math.sqrt((A[0] - B[0]) ** 2 + (A[1] - B[1]) ** 2)]) / self.ht
        return np.minimum(A, B) - self.radius * k, np.maximum(A, B) + self.radius * k


def _filtered(self, predicate, recenter=True):
    """SpherePack.filtered (py/_packPredicates.cpp:364-395): the spheres inside ``predicate``
    (a clump goes when any of its spheres is outside); with ``recenter`` and a finite predicate,
    the packing is first moved so that the centres of the two bounding boxes coincide."""
    ret = SpherePack()
    ret.cellSize = self.cellSize.copy()
    off = np.zeros(3)
    pmn, pmx = predicate.aabb()
    if recenter and np.all(np.isfinite(np.asarray(pmx) - np.asarray(pmn))) and self.pack:
        smn, smx = self.aabb()
        off = 0.5 * (np.asarray(pmn) + np.asarray(pmx)) - 0.5 * (smn + smx)
    inside = [bool(predicate(c + off, r)) for c, r, _ in self.pack]
    gone = {k for (c, r, k), ok in zip(self.pack, inside) if not ok and k >= 0}
    for (c, r, k), ok in zip(self.pack, inside):
        if ok and (k < 0 or k not in gone):
            ret.add(c + off, r, k)
    return ret


SpherePack.filtered = _filtered


def filterSpherePack(predicate, spherePack, **kw):
    """The spheres of ``spherePack`` inside ``predicate``, recentred (py/pack.py:387-391)."""
    return spherePack.filtered(predicate)


def _finiteAabb(predicate):
    mn, mx = (np.asarray(v, dtype=float) for v in predicate.aabb())
    if not np.all(np.isfinite(mx - mn)):
        raise ValueError("Aabb of the predicate must not be infinite (didn't you use union | instead of intersection & for "
                         "unbounded predicate such as notInNotch?")
    return mn, mx


def regularOrtho(predicate, radius, gap, **kw):
    """Spheres of ``radius`` on an orthogonal grid of pitch 2·radius+gap inside ``predicate``
    (py/pack.py:323-332); ``kw`` go to utils.sphere."""
    from . import utils
    mn, mx = _finiteAabb(predicate)
    xx, yy, zz = [np.arange(mn[i] + radius, mx[i] - radius, 2 * radius + gap) for i in range(3)]
    return [utils.sphere((x, y, z), radius=radius, **kw) for x in xx for y in yy for z in zz if predicate((x, y, z), radius)]


def regularHexa(predicate, radius, gap, **kw):
    """Spheres of ``radius`` on the reference's hexagonal grid inside ``predicate``
    (py/pack.py:334-351): rows a=2·radius+gap apart within a row, rows a·√3/2 apart and shifted
    by a/2 alternately, layers a·√6/3 apart with odd layers shifted by a·√3/4 across the rows.
    That layer shift puts some centres of adjacent layers a·√(3/16+2/3) ≈ 0.924·a apart (closer
    than a), which is kept: the same call gives the same spheres as the reference."""
    from . import utils
    mn, mx = _finiteAabb(predicate)
    a = 2 * radius + gap
    hy, hz = a * math.sqrt(3) / 2., a * math.sqrt(6) / 3.
    dim = mx - mn
    out = []
    for i in range(int(dim[0] / a) + 1):
        for j in range(int(dim[1] / hy) + 1):
            for k in range(int(dim[2] / hz) + 1):
                x, y, z = mn[0] + radius + i * a, mn[1] + radius + j * hy, mn[2] + radius + k * hz
                if j % 2 == 0:
                    x += a / 2. if k % 2 == 0 else -a / 2.
                if k % 2 != 0:
                    x += a / 2.
                    y += hy / 2.
                if predicate((x, y, z), radius):
                    out.append(utils.sphere((x, y, z), radius=radius, **kw))
    return out
