"""Seeded synthetic scenes of the benchmark configurations.

Each builder returns a ready-to-run Scene assembled through the Woo-style API
(utils.wallBox, triangulated.cylinder, utils.defaultEngines, utils.pWaveDt); the
particle positions come from numpy's PCG64 generator or the seeded random
sequential insertion of libwoogpu (wg_pack_rsa). Boundary particles are added
before the spheres, so walls and facets take the lowest ids.
"""
import math

import numpy as np

from . import utils, triangulated, _native
from .core import Scene
from .dem import DemField, FrictMat, Cp2_FrictMat_HertzPhys, Law2_L6Geom_HertzPhys_DMT


def pack_rsa(radii, lo, hi, region=0, params=(0, 0, 0, 0), seed=0, max_attempts=2000, device=False):
    """Seeded random sequential insertion (largest spheres first). Returns centers in input order.
    ``device``: insert on the current GPU (wg_pack_rsa_device, rounds over a window of spheres)
    instead of the host (wg_pack_rsa); both give valid packings of the same statistics, not the
    same one."""
    radii = np.ascontiguousarray(radii, dtype=float)
    order = np.argsort(-radii, kind="stable")
    r_sorted = np.ascontiguousarray(radii[order])
    out = np.zeros((len(radii), 3))
    lo = np.ascontiguousarray(lo, dtype=float)
    hi = np.ascontiguousarray(hi, dtype=float)
    pr = np.ascontiguousarray(params, dtype=float)
    fn = _native.lib().wg_pack_rsa_device if device else _native.lib().wg_pack_rsa
    n = fn(len(radii), _native.ptr(r_sorted), _native.ptr(lo), _native.ptr(hi), int(region), _native.ptr(pr), int(seed),
           int(max_attempts), _native.ptr(out))
    if n < 0:
        raise RuntimeError("device random insertion failed (%s)" % ("CUDA error" if n == -1 else "invalid argument"))
    if n != len(radii):
        raise RuntimeError("random insertion placed only %d of %d spheres; enlarge the region" % (n, len(radii)))
    res = np.empty_like(out)
    res[order] = out
    return res


def box_settle(n=10000, seed=0, radius=5e-3, pitch=12e-3, dims=(22, 22, 21), box=((0, 0, 0), (0.3, 0.3, 0.6)), density=3000.0,
               young=1e7, ktDivKn=0.2, tanPhi=0.5, damping=0.2, verletRel=0.1, jitter=1e-3, precision="fp64"):
    """Box settle: spheres on a jittered cubic lattice (x fastest, first ``n`` sites), lattice
    centred in x and y and starting one pitch above z=0, six inward-facing walls, gravity
    (0,0,-9.81), dt = 0.3*pWaveDt, Leapfrog damping 0.2, verletDist = 0.1*radius, IdealElPl."""
    nx, ny, nz = dims
    if n > nx * ny * nz:
        raise ValueError("lattice too small")
    lo, hi = np.asarray(box[0], float), np.asarray(box[1], float)
    x0 = lo[0] + ((hi[0] - lo[0]) - (nx - 1) * pitch) / 2
    y0 = lo[1] + ((hi[1] - lo[1]) - (ny - 1) * pitch) / 2
    z0 = lo[2] + pitch
    i = np.arange(n)
    centers = np.stack([x0 + (i % nx) * pitch, y0 + ((i // nx) % ny) * pitch, z0 + (i // (nx * ny)) * pitch], axis=1)
    rng = np.random.default_rng(seed)
    centers = centers + rng.uniform(-jitter, jitter, size=(n, 3))
    S = Scene(fields=[DemField(gravity=(0, 0, -9.81))])
    S.gpu.precision = precision
    mat = FrictMat(density=density, young=young, ktDivKn=ktDivKn, tanPhi=tanPhi)
    S.dem.par.add(utils.wallBox((lo, hi), mat=mat))
    S.dem.par.addSpheres(centers, radius, mat)
    S.engines = utils.defaultEngines(damping=damping, verletDist=-verletRel, dynDtPeriod=0)
    S.dt = 0.3 * utils.pWaveDt(S)
    return S


def box_settle_small(n=1500, seed=0, precision="fp64", **kw):
    """The box-settle configuration on a smaller lattice (tests)."""
    side = int(math.ceil((n / 2.0) ** (1 / 3.0)))
    dims = (side, side, int(math.ceil(n / float(side * side))))
    pitch = kw.pop("pitch", 12e-3)
    w = (dims[0] + 3) * pitch
    h = 2 * (dims[2] + 3) * pitch
    return box_settle(n=n, seed=seed, pitch=pitch, dims=dims, box=((0, 0, 0), (w, w, h)), precision=precision, **kw)


def lognormal_radii(n, seed, median=3e-3, sigma=0.25, rmin=1.5e-3, rmax=6e-3):
    rng = np.random.default_rng(seed)
    return np.clip(median * np.exp(sigma * rng.standard_normal(n)), rmin, rmax)


def _segment_height(R, area):
    """Height z (relative to the axis) below which a circle of radius R has the given area."""
    lo, hi = -R, R
    for _ in range(100):
        z = 0.5 * (lo + hi)
        a = R * R * math.acos(-z / R) + z * math.sqrt(max(R * R - z * z, 0.0))
        if a < area:
            lo = z
        else:
            hi = z
    return 0.5 * (lo + hi)


def spatial_order(points, cell):
    """Permutation that lists ``points`` along a Morton (Z-order) curve over a grid of cubes of
    side ``cell`` (up to 2^21 cells per axis), so that particles close in space get close ids."""
    pts = np.asarray(points, dtype=float)
    if len(pts) == 0:
        return np.zeros(0, dtype=np.int64)
    q = np.floor((pts - pts.min(axis=0)) / float(cell)).astype(np.uint64)
    q = np.minimum(q, np.uint64((1 << 21) - 1))

    def spread(v):
        v = v & np.uint64(0x1FFFFF)
        v = (v | (v << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
        v = (v | (v << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
        v = (v | (v << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
        v = (v | (v << np.uint64(2))) & np.uint64(0x1249249249249249)
        return v

    code = spread(q[:, 0]) | (spread(q[:, 1]) << np.uint64(1)) | (spread(q[:, 2]) << np.uint64(2))
    return np.argsort(code, kind="stable")


def settle(S, steps, g_factor=30.0, damping=0.3, precision="fp32", relax_steps=0, relax_damping=0.3, zero=True, relax_stages=4):
    """Compact a loose packing into a resting bed on the GPU: run ``steps`` steps under gravity
    multiplied by ``g_factor`` with Leapfrog damping ``damping``, then bring gravity back to the
    scene's own in ``relax_stages`` geometric stages (g_factor^(3/4), ^(1/2), ^(1/4), 1 for four)
    of ``relax_steps/relax_stages`` steps each with damping ``relax_damping``, so that the elastic
    energy stored under the high gravity leaves the bed gradually instead of launching it. Then
    restore the scene's gravity, damping and precision, zero the forces and torques (and with
    ``zero`` the velocities) of the free nodes, and reset Scene.step/time. The contact history is
    dropped (the next run starts from the positions)."""
    lf = S.engines[0]
    g0 = np.array(S.dem.gravity, dtype=float)
    d0, p0 = lf.damping, S.gpu.precision
    S.close()
    S.dem.gravity = g0 * g_factor
    lf.damping = damping
    S.gpu.precision = precision
    S.run(steps)
    if relax_steps:
        for k in range(1, relax_stages + 1):
            S.close()
            S.dem.gravity = g0 * g_factor ** ((relax_stages - k) / float(relax_stages))
            lf.damping = relax_damping
            S.run(max(1, relax_steps // relax_stages))
    S.close()
    S.dem.gravity = g0
    lf.damping = d0
    S.gpu.precision = p0
    nd = S.dem._nodes.soa
    free = (nd.col("flags") & 63) != 63
    for k in (("vel", "angVel", "force", "torque") if zero else ("force", "torque")):
        nd.col(k)[free] = 0.0
    S.step = 0
    S.time = 0.0
    return S


def _drum_scene(centers, radii, diameter, length, div, axDiv, density, young, poisson, en, tanPhi, omega, verletRel, precision):
    R = diameter / 2.0
    S = Scene(fields=[DemField(gravity=(0, 0, -9.81))])
    S.gpu.precision = precision
    mat = FrictMat(density=density, young=young, tanPhi=tanPhi)
    drum = triangulated.cylinder((0, 0, 0), (length, 0, 0), R, div=div, axDiv=axDiv, capA=True, capB=True, wallCaps=True,
                                 angVel=omega, mat=mat)
    S.dem.par.add(drum)
    S.dem.par.addSpheres(centers, radii, mat)
    S.engines = utils.defaultEngines(cp2=Cp2_FrictMat_HertzPhys(poisson=poisson, en=en, gamma=0.0, alpha=0.0),
                                     law=Law2_L6Geom_HertzPhys_DMT(), verletDist=-verletRel, dynDtPeriod=0, damping=0.0)
    S.dt = 0.3 * utils.pWaveDt(S)
    return S


def hertz_drum(n=1_000_000, seed=0, diameter=1.2, length=0.6, div=201, axDiv=50, fill_fraction=0.40, density=2500.0,
               young=1e8, poisson=0.25, en=0.6, tanPhi=0.5, omega=1.0, verletRel=0.1, precision="fp64",
               median=3e-3, sigma=0.25, rmin=1.5e-3, rmax=6e-3, settle_steps=0, settle_g=40.0, relax_steps=None, order=True):
    """Rotating drum: x-axis cylinder (diameter x length) meshed into 2*(div-1)*axDiv facets with
    outward normals and fakeVel for angular velocity ``omega``, two rotating Wall end caps,
    lognormal radii, Hertz contacts with viscous damping (en), gravity (0,0,-9.81),
    dt = 0.3*pWaveDt, verletDist = 0.1*min radius. Spheres are placed by seeded random
    sequential insertion (solid fraction ``fill_fraction``) in the lower part of the drum whose
    height is chosen to hold them. With ``settle_steps`` the fill is compacted into a resting bed
    on the GPU (``settle``: ``settle_g`` times gravity, then ``relax_steps`` steps easing back to 1 g) and the
    scene is rebuilt from the settled positions. With ``order`` the spheres are numbered along a
    Morton curve of their positions (cells of one largest diameter), so that spheres in contact
    have nearby ids; walls and facets keep the lowest ids."""
    R = diameter / 2.0
    radii = lognormal_radii(n, seed, median, sigma, rmin, rmax)
    vol = float(np.sum((4 / 3.0) * math.pi * radii ** 3))
    margin = 1e-4
    usable = length - 2 * margin
    area = vol / fill_fraction / usable
    Ri = R - margin
    zf = _segment_height(Ri, min(area, 0.97 * math.pi * Ri * Ri))
    centers = pack_rsa(radii, (margin, -Ri, -Ri), (length - margin, Ri, zf), region=1, params=(0.0, 0.0, Ri, zf), seed=seed + 7)
    args = (diameter, length, div, axDiv, density, young, poisson, en, tanPhi, omega, verletRel)
    vel = angVel = None
    if settle_steps:
        S0 = _drum_scene(centers, radii, *args, precision)
        settle(S0, settle_steps, g_factor=settle_g, relax_steps=(3 * settle_steps) // 4 if relax_steps is None else relax_steps,
               relax_damping=0.8, zero=True)
        centers, vel, angVel = (_sphere_nodes(S0, k) for k in ("pos", "vel", "angVel"))
        S0 = None
    if order:
        perm = spatial_order(centers, 2 * rmax)
        centers, radii = centers[perm], radii[perm]
        if vel is not None:
            vel, angVel = vel[perm], angVel[perm]
    S = _drum_scene(centers, radii, *args, precision)
    if vel is not None:
        # the bed starts from the state it settled to
        _sphere_nodes(S, "vel", vel)
        _sphere_nodes(S, "angVel", angVel)
    return S


def hertz_drum_from_state(centers, radii, vel=None, angVel=None, diameter=1.2, length=0.6, div=201, axDiv=50, density=2500.0,
                          young=1e8, poisson=0.25, en=0.6, tanPhi=0.5, omega=1.0, verletRel=0.1, precision="fp64"):
    """The drum of ``hertz_drum`` around given sphere centres and radii (in sphere order), with the
    given sphere velocities: rebuilds a scene from a stored state (host only, no device work)."""
    S = _drum_scene(np.asarray(centers, float), np.asarray(radii, float), diameter, length, div, axDiv, density, young, poisson,
                    en, tanPhi, omega, verletRel, precision)
    if vel is not None:
        _sphere_nodes(S, "vel", np.asarray(vel, float))
    if angVel is not None:
        _sphere_nodes(S, "angVel", np.asarray(angVel, float))
    return S


def sphere_radii(S):
    """Radii of the spheres of a scene, in sphere order."""
    from . import _plan
    A = _plan.compile_scene(S)
    return A.particles["radius"][A.particles["shape"] == 0].copy()


def _sphere_nodes(S, col, value=None):
    """Read (or write) a node column for the spheres of a scene, in sphere order."""
    from . import _plan
    nd = S.dem._nodes.soa
    A = _plan.compile_scene(S)
    nodes = A.particles["nodes"][A.particles["shape"] == 0, 0]
    if value is None:
        return nd.col(col)[nodes].copy()
    nd.col(col)[nodes] = value


def periodic_shear(n=200_000, seed=0, rmin=2e-3, rmax=4e-3, density=2600.0, young=5e7, tanPhi=0.4, ktDivKn=0.2,
                   fill_fraction=0.35, shear_rate=1.0, damping=0.2, verletRel=0.1, precision="fp64", compress_steps=0,
                   compress_rate=None, centers=None, compress_to=0.55, pack_device=False):
    """Periodic simple shear: ``n`` spheres with radii uniform in [rmin, rmax] placed by seeded random
    sequential insertion in a periodic cube sized to solid fraction ``fill_fraction``; IdealElPl
    contacts, Leapfrog damping ``damping``, dt = 0.3*pWaveDt, verletDist = 0.1*rmin,
    Cell.homoDeform = HomoGradV2. With ``compress_steps`` the cell is first compressed isotropically
    (nextGradV = -compress_rate*I, by default the rate that brings the fill to ``compress_to`` in
    that many steps); then nextGradV is set to the simple shear with xz component ``shear_rate``. Given
    ``centers``, those positions are used instead of the random insertion (a state to restore);
    ``pack_device`` makes the insertion on the GPU (``pack_rsa(device=True)``)."""
    from .core import Cell
    rng = np.random.default_rng(seed)
    radii = rng.uniform(rmin, rmax, n)
    vol = float(np.sum((4 / 3.0) * math.pi * radii ** 3))
    side = (vol / fill_fraction) ** (1 / 3.0)
    if centers is None:
        centers = pack_rsa(radii, (0, 0, 0), (side, side, side), region=2, seed=seed + 11, device=pack_device)
    S = Scene(fields=[DemField(gravity=(0, 0, 0))])
    S.gpu.precision = precision
    S.periodic = True
    S.cell.setBox(side, side, side)
    S.cell.homoDeform = Cell.HomoGradV2
    mat = FrictMat(density=density, young=young, tanPhi=tanPhi, ktDivKn=ktDivKn)
    S.dem.par.addSpheres(centers, radii, mat)
    S.engines = utils.defaultEngines(damping=damping, verletDist=-verletRel, dynDtPeriod=0)
    S.dt = 0.3 * utils.pWaveDt(S)
    if compress_steps:
        rate = compress_rate
        if rate is None:
            rate = math.log((compress_to / fill_fraction) ** (1 / 3.0)) / (compress_steps * S.dt)
        S.cell.nextGradV = -rate * np.eye(3)
        S.run(compress_steps)
    g = np.zeros((3, 3))
    g[0, 2] = shear_rate
    S.cell.nextGradV = g
    return S


def box_settle_scaled(n, radius, seed=0, density=3000.0, young=1e7, tanPhi=0.5, ktDivKn=0.2, damping=0.2, verletRel=0.1,
                      precision="fp64"):
    """A box settle of ``n`` spheres of one ``radius``: the lattice of the 10k-sphere box settle (pitch
    2.4 radius, jitter 0.2 radius, two stacked layers per column of the square footprint) in a box
    with a free column of three pitches around it and twice the lattice height."""
    pitch = 2.4 * radius
    side = int(math.ceil((n / 2.0) ** (1 / 3.0)))
    dims = (side, side, int(math.ceil(n / float(side * side))))
    w = (dims[0] + 3) * pitch
    h = 2 * (dims[2] + 3) * pitch
    return box_settle(n=n, seed=seed, radius=radius, pitch=pitch, dims=dims, box=((0, 0, 0), (w, w, h)), density=density,
                      young=young, ktDivKn=ktDivKn, tanPhi=tanPhi, damping=damping, verletRel=verletRel, jitter=0.2 * radius,
                      precision=precision)


def batch_study(n_scenes=256, seed=0, nmin=1000, nmax=50000, rmin=3e-3, rmax=6e-3, precision="fp64"):
    """Parametric study of independent box settles: sphere counts log-uniform in [nmin, nmax], one
    radius per scene uniform in [rmin, rmax], tanPhi log-uniform in [0.2, 0.8], young log-uniform in
    [1e6, 1e8] Pa, Leapfrog damping uniform in [0, 0.4]; each scene is a ``box_settle_scaled``.
    Returns the list of scenes and the table of their parameters."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(math.log(nmin), math.log(nmax), n_scenes)).astype(int)
    r = rng.uniform(rmin, rmax, n_scenes)
    tp = np.exp(rng.uniform(math.log(0.2), math.log(0.8), n_scenes))
    E = np.exp(rng.uniform(math.log(1e6), math.log(1e8), n_scenes))
    d = rng.uniform(0.0, 0.4, n_scenes)
    scenes = [box_settle_scaled(int(n[k]), float(r[k]), seed=seed * 1000 + k, young=float(E[k]), tanPhi=float(tp[k]),
                                damping=float(d[k]), precision=precision) for k in range(n_scenes)]
    table = {"n": n, "radius": r, "tanPhi": tp, "young": E, "damping": d}
    return scenes, table


class BoxSettle:
    """Preprocessor of a box settle (``box_settle_scaled``): set the attributes, call it, get the
    Scene. ``stopAtStep`` is copied to the scene, so that a table runner knows how many steps each
    line wants. Used as the simulation of parameter tables (``woo.batch.runPreprocessor``)."""

    def __init__(self, n=2000, radius=4e-3, seed=0, density=3000.0, young=1e7, tanPhi=0.5, ktDivKn=0.2, damping=0.2,
                 verletRel=0.1, precision="fp64", stopAtStep=0):
        self.n, self.radius, self.seed, self.density, self.young = n, radius, seed, density, young
        self.tanPhi, self.ktDivKn, self.damping, self.verletRel = tanPhi, ktDivKn, damping, verletRel
        self.precision, self.stopAtStep = precision, stopAtStep

    def checkAttrTypes(self):
        for k in ("n", "seed", "stopAtStep"):
            v = getattr(self, k)
            if int(v) != v:
                raise TypeError("%s must be an integer (%r)" % (k, v))
            setattr(self, k, int(v))
        if self.precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32' (%r)" % self.precision)

    def __call__(self):
        S = box_settle_scaled(int(self.n), float(self.radius), seed=int(self.seed), density=float(self.density),
                              young=float(self.young), tanPhi=float(self.tanPhi), ktDivKn=float(self.ktDivKn),
                              damping=float(self.damping), verletRel=float(self.verletRel), precision=self.precision)
        S.stopAtStep = int(self.stopAtStep)
        return S
