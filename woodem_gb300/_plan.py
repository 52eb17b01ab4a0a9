"""Compile a Woo-style scene (engine list + DemField) into the flat description of
include/woo_gpu.h, and drive the device simulation behind ``Scene.run``.

The engine list is validated against what the GPU path implements: the order
[Leapfrog(reset=True), InsertionSortCollider, ContactLoop] of utils.defaultEngines
(py/utils.py:55-94) with the Sphere/Facet/Wall functors and one Cp2/Law2 pair.
Anything else raises (no silent fallback).
"""
import math
import numpy as np

from . import _native


class GpuConfig:
    """GPU-only knobs, kept off the reference classes so scene scripts stay unchanged.

    precision: 'fp64' (plain, bitwise-reproducible against the FP64 oracle) or
               'fp32' (contact geometry and force laws in FP32, FP64 accumulation).
    device:    CUDA device index.
    """

    def __init__(self, precision="fp64", device=0):
        self.precision = precision
        self.device = device


class SceneArrays:
    """The flat arrays and configuration handed to the C ABI (and to the CPU oracle in tests)."""

    def __init__(self):
        self.nodes = {}
        self.particles = {}
        self.materials = {}
        self.config = {}

    @property
    def n_nodes(self):
        return len(self.nodes["pos"])

    @property
    def n_particles(self):
        return len(self.particles["shape"])


def _find(engines, cls):
    return [e for e in engines if isinstance(e, cls) and not e.dead]


def compile_scene(S):
    from . import dem
    if not S.fields:
        raise ValueError("Scene has no fields")
    D = S.dem
    # engines that run on the host between device steps (VtkExport) are not part of the device plan
    eng = [e for e in S.engines if not getattr(e, "dead", False) and not getattr(e, "_host", False)]
    kinds = []
    for e in eng:
        if isinstance(e, dem.Leapfrog):
            kinds.append("leapfrog")
        elif isinstance(e, dem.InsertionSortCollider):
            kinds.append("collider")
        elif isinstance(e, dem.ContactLoop):
            kinds.append("loop")
        elif isinstance(e, dem.DynDt):
            kinds.append("dyndt")
        else:
            raise NotImplementedError("Engine %s is not part of the GPU path" % type(e).__name__)
    if kinds not in (["leapfrog", "collider", "loop"], ["leapfrog", "collider", "loop", "dyndt"]):
        raise NotImplementedError("The GPU path runs the engine sequence [Leapfrog, InsertionSortCollider, ContactLoop"
                                  "(, DynDt)] (got %s)" % kinds)
    lf, col, loop = eng[:3]
    dyn = eng[3] if len(eng) == 4 else None
    if not lf.reset:
        raise NotImplementedError("Leapfrog.reset=False is not part of the GPU path (use reset=True)")
    cfg = {}
    if not (S.dt > 0 and math.isfinite(S.dt)):
        # Scene::doOneStep (core/Scene.cpp:332-352): dt = dtSafety times the smallest critical dt of
        # the engines and fields. Engines give Inf, DynDt too while no contact is real (before the
        # first step); the DemField gives pWaveDt without clumps (pkg/dem/Particle.cpp:372-377).
        from .utils import pWaveDt
        crit = pWaveDt(S, noClumps=True)
        if not math.isfinite(crit):
            raise RuntimeError("Failed to obtain meaningful dt from engines and fields automatically.")
        S.dt = S.dtSafety * crit
    cfg["dt"] = float(S.dt)
    cfg["dt_safety"] = float(S.dtSafety)
    cfg["next_dt"] = float(S.nextDt) if (S.nextDt > 0 and math.isfinite(S.nextDt)) else float("nan")
    cfg["time"] = float(S.time)
    cfg["track_energy"] = int(bool(S.trackEnergy))
    cfg["kin_split"] = int(bool(lf.kinSplit))
    if dyn is not None:
        if dyn.realPeriod > 0:
            raise NotImplementedError("DynDt.realPeriod (wall-clock activation) is not part of the GPU path")
        if not (1.0 + dyn.maxRelInc != 1.0 and dyn.maxRelInc > 0):
            raise ValueError("DynDt: maxRelInc too small (1.0+maxRelInc==1.0)")
        cfg.update(dyndt=1, dyndt_dry_run=int(bool(dyn.dryRun)), dyndt_step_modulo=int(bool(dyn.stepModulo)),
                   dyndt_init_run=int(bool(dyn.initRun)), dyndt_step_period=int(dyn.stepPeriod), dyndt_n_do=int(dyn.nDo),
                   dyndt_n_done=int(dyn.nDone), dyndt_step_last=int(dyn.stepLast), dyndt_step_prev=int(dyn.stepPrev),
                   dyndt_virt_period=float(dyn.virtPeriod), dyndt_virt_last=float(dyn.virtLast),
                   dyndt_virt_prev=float(dyn.virtPrev), dyndt_max_rel_inc=float(dyn.maxRelInc))
    cfg["gravity"] = np.asarray(D.gravity, dtype=float)
    cfg["lone_mask"] = int(D.loneMask)
    cfg["deterministic"] = 1
    cfg["step"] = int(S.step)
    cfg["damping"] = float(lf.damping)
    cfg["reset"] = 1
    cfg["verlet_dist"] = float(col.verletDist)
    df = -1.0
    for f in col.boundDispatcher:
        if isinstance(f, dem.Bo1_Sphere_Aabb):
            df = float(f.distFactor)
    cfg["bo1_sphere_dist_factor"] = df
    cfg["sort_axis"] = int(col.sortAxis)
    cfg["apply_forces"] = int(bool(loop.applyForces))
    cfg["eval_stress"] = int(bool(loop.evalStress))
    if loop.updatePhys:
        raise NotImplementedError("ContactLoop.updatePhys=True is not part of the GPU path")
    # geometry functors: common L6Geom attributes must agree
    geo = [g for g in loop.geoDisp if isinstance(g, dem.Cg2_Any_Any_L6Geom__Base)]
    if not any(isinstance(g, dem.Cg2_Sphere_Sphere_L6Geom) for g in geo):
        raise NotImplementedError("ContactLoop needs Cg2_Sphere_Sphere_L6Geom")
    for a in ("trsfRenorm", "approxMask", "noRatch"):
        vals = {getattr(g, a) for g in geo}
        if len(vals) != 1:
            raise NotImplementedError("Cg2 functors with different %s values are not supported" % a)
    g0 = geo[0]
    cfg["trsf_renorm"] = int(g0.trsfRenorm)
    cfg["approx_mask"] = int(g0.approxMask)
    cfg["no_ratch"] = int(bool(g0.noRatch))
    ss = [g for g in geo if isinstance(g, dem.Cg2_Sphere_Sphere_L6Geom)][0]
    cfg["cg2_ss_dist_factor"] = float(ss.distFactor)
    if abs(ss.distFactor) != 1.0 or df > 0 and df != 1.0:
        raise NotImplementedError("distFactor != 1 (distant contacts) is not part of the GPU path")
    have_fs = any(isinstance(g, dem.Cg2_Facet_Sphere_L6Geom) for g in geo)
    have_ws = any(isinstance(g, dem.Cg2_Wall_Sphere_L6Geom) for g in geo)
    cp2 = [f for f in loop.phyDisp if isinstance(f, dem.CPhysFunctor)]
    law = [f for f in loop.lawDisp if isinstance(f, dem.LawFunctor)]
    if len(cp2) != 1 or len(law) != 1:
        raise NotImplementedError("exactly one Cp2 and one Law2 functor are supported")
    cp2, law = cp2[0], law[0]
    if isinstance(cp2, dem.Cp2_FrictMat_HertzPhys):
        cfg["phys"] = 1
        cfg["hz_poisson"] = float(cp2.poisson)
        cfg["hz_gamma"] = float(cp2.gamma)
        cfg["hz_en"] = float(cp2.en)
        cfg["hz_alpha"] = float(cp2.alpha)
        if cp2.alpha != 0:
            raise NotImplementedError("Cp2_FrictMat_HertzPhys.alpha!=0 (Schwarz model) is not part of the GPU path")
    elif isinstance(cp2, dem.Cp2_FrictMat_FrictPhys):
        cfg["phys"] = 0
        if cp2.tanPhi is not None:
            raise NotImplementedError("Cp2_FrictMat_FrictPhys.tanPhi (MatchMaker) is not part of the GPU path")
    else:
        raise NotImplementedError("Cp2 functor %s is not part of the GPU path" % type(cp2).__name__)
    if isinstance(law, dem.Law2_L6Geom_HertzPhys_DMT):
        if cfg["phys"] != 1:
            raise NotImplementedError("Law2_L6Geom_HertzPhys_DMT needs Cp2_FrictMat_HertzPhys")
        cfg["law"] = 1
        cfg["hz_no_attraction"] = int(bool(law.noAttraction))
    elif isinstance(law, dem.Law2_L6Geom_FrictPhys_IdealElPl):
        if cfg["phys"] != 0:
            raise NotImplementedError("HertzPhys contacts with Law2_L6Geom_FrictPhys_IdealElPl are not part of the GPU path")
        cfg["law"] = 0
        if law.iniEqlb:
            raise NotImplementedError("Law2_L6Geom_FrictPhys_IdealElPl.iniEqlb is not part of the GPU path")
        if law.relRollStiff > 0 and law.rollTanPhi > 0:
            raise NotImplementedError("rolling/twisting resistance is not part of the GPU path")
        cfg["no_slip"] = int(bool(law.noSlip))
        cfg["no_break"] = int(bool(law.noBreak))
        cfg["no_frict"] = int(bool(law.noFrict))
    else:
        raise NotImplementedError("Law2 functor %s is not part of the GPU path" % type(law).__name__)
    cfg["periodic"] = int(bool(S.isPeriodic))
    cell = S.cell
    cfg["homo_deform"] = int(cell.homoDeform)
    cfg["cell_hsize"] = np.asarray(cell.hSize, dtype=float)
    cfg["cell_trsf"] = np.asarray(cell.trsf, dtype=float)
    cfg["cell_gradv"] = np.asarray(cell.gradV, dtype=float)
    cfg["cell_next_gradv"] = np.asarray(cell.nextGradV, dtype=float)
    cfg["precision"] = {"fp64": 0, "fp32": 1}[S.gpu.precision]

    A = SceneArrays()
    A.config = cfg
    ns = D._nodes.soa
    A.nodes = {k: np.ascontiguousarray(ns.col(k)) for k in ("pos", "ori", "vel", "angVel", "force", "torque", "mass",
                                                            "inertia", "flags")}
    ps = D.par.soa
    A.particles = {k: np.ascontiguousarray(ps.col(k)) for k in ("shape", "nodes", "radius", "axis", "sense", "halfThick",
                                                                "fakeVel", "mat", "mask")}
    # functor availability: shape pairs without a functor never become real (ContactLoop.cpp:145-148)
    shp = A.particles["shape"]
    if (np.any(shp == 2) and not have_fs) or (np.any(shp == 1) and not have_ws):
        raise NotImplementedError("scene has facets/walls but the ContactLoop lacks their Cg2 functor")
    if dyn is not None and np.any(shp == 2):
        fn = A.particles["nodes"][shp == 2].ravel()
        if np.any((A.nodes["flags"][fn[fn >= 0]] & 63) != 63):
            raise NotImplementedError("DynDt with facet nodes that are not fully blocked (their stiffness includes the "
                                      "facets' internal forces) is not part of the GPU path")
    mats = D._mats
    for m in mats:
        from .dem import FrictMat
        if not isinstance(m, FrictMat):
            raise NotImplementedError("material %s is not FrictMat" % type(m).__name__)
    A.materials = {
        "density": np.array([m.density for m in mats], dtype=float),
        "young": np.array([m.young for m in mats], dtype=float),
        "tanPhi": np.array([m.tanPhi for m in mats], dtype=float),
        "ktDivKn": np.array([m.ktDivKn for m in mats], dtype=float),
    }
    return A


class Simulation:
    """Device simulation of one Scene."""

    def __init__(self, S):
        self.S = S
        self.t0 = float(S.time)  # Scene.time at upload; the device counts the time run since
        self.A = compile_scene(S)
        self.dirty_structure = False
        self.host_written = False
        self.host_stale = False
        self.H = _native.Handle(S.gpu.device)
        L, h = self.H.L, self.H.h
        A = self.A
        cfg = _native.make_config(_native.wg_config, A.config)
        self.H.check(L.wg_set_config(h, cfg), "set_config")
        m = A.materials
        self.H.check(L.wg_set_materials(h, len(m["density"]), _native.ptr(m["density"]), _native.ptr(m["young"]),
                                        _native.ptr(m["tanPhi"]), _native.ptr(m["ktDivKn"])), "set_materials")
        nd = A.nodes
        self.H.check(L.wg_set_nodes(h, A.n_nodes, _native.ptr(nd["pos"]), _native.ptr(nd["ori"]), _native.ptr(nd["vel"]),
                                    _native.ptr(nd["angVel"]), _native.ptr(nd["force"]), _native.ptr(nd["torque"]),
                                    _native.ptr(nd["mass"]), _native.ptr(nd["inertia"]),
                                    _native.ptr(nd["flags"], _native.P_U32)), "set_nodes")
        p = A.particles
        self.H.check(L.wg_set_particles(h, A.n_particles, _native.ptr(p["shape"], _native.P_I32),
                                        _native.ptr(p["nodes"], _native.P_I32), _native.ptr(p["radius"]),
                                        _native.ptr(p["axis"], _native.P_I32), _native.ptr(p["sense"], _native.P_I32),
                                        _native.ptr(p["halfThick"]), _native.ptr(p["fakeVel"]),
                                        _native.ptr(p["mat"], _native.P_I32), _native.ptr(p["mask"], _native.P_U32)),
                     "set_particles")
        self._contacts = None

    def close(self):
        if self.H is not None:
            self.pull()
            self.H.close()
            self.H = None

    def push(self):
        if not self.host_written:
            return
        nd = self.S.dem._nodes.soa
        L, h = self.H.L, self.H.h
        arrs = [np.ascontiguousarray(nd.col(k)) for k in ("pos", "ori", "vel", "angVel", "force", "torque")]
        self.H.check(L.wg_put_state(h, *[_native.ptr(a) for a in arrs]), "put_state")
        self.host_written = False

    def run(self, n):
        self.push()
        L, h = self.H.L, self.H.h
        if self.S.isPeriodic:
            # Cell.nextGradV set between runs takes effect at the next step (core/Cell.hpp:152)
            g = np.ascontiguousarray(np.asarray(self.S.cell.nextGradV, dtype=float).reshape(9))
            self.H.check(L.wg_set_next_gradv(h, _native.ptr(g)), "set_next_gradv")
        self._push_dt()
        self._push_energy()
        self.H.check(L.wg_run(h, int(n)), "run")
        self.host_stale = True
        self._contacts = None
        st = self.stats()
        self.S.step = int(st.step)
        self.S.time = self.t0 + float(st.time)
        self._pull_dt()
        self._pull_energy()
        for e in self.S.engines:
            from .dem import InsertionSortCollider
            if isinstance(e, InsertionSortCollider):
                e.nFullRuns = int(st.n_full_runs)
                if e.verletDist < 0:
                    pass
        if self.S.isPeriodic:
            hs = np.zeros(9)
            tr = np.zeros(9)
            gv = np.zeros(9)
            L.wg_get_cell(h, _native.ptr(hs), _native.ptr(tr), _native.ptr(gv))
            self.S.cell.hSize = hs.reshape(3, 3)
            self.S.cell.trsf = tr.reshape(3, 3)
            self.S.cell._gradV = gv.reshape(3, 3)
            from .dem import ContactLoop
            for e in self.S.engines:
                if isinstance(e, ContactLoop):
                    e.stress = np.array(st.stress).reshape(3, 3)

    def dyndt(self):
        st = _native.wg_dyndt_state()
        self.H.check(self.H.L.wg_get_dyndt(self.H.h, C_byref(st)), "get_dyndt")
        return st

    def _push_dt(self):
        """Scene.dt or Scene.nextDt set on the host since the last run."""
        S = self.S
        nxt = float(S.nextDt) if (S.nextDt > 0 and math.isfinite(S.nextDt)) else float("nan")
        st = self.dyndt()
        if S.dt != st.dt or not (nxt == st.next_dt or (math.isnan(nxt) and math.isnan(st.next_dt))):
            if not (S.dt > 0 and math.isfinite(S.dt)):
                raise ValueError("Scene.dt must be positive and finite")
            self.H.check(self.H.L.wg_set_dt(self.H.h, float(S.dt), nxt), "set_dt")

    def _push_energy(self):
        """Scene.energy entries of the device changed on the host (set, added, cleared)."""
        E = self.S.energy
        if not (self.S.trackEnergy and E._dirty):
            return
        names = _native.ENERGY_NAMES
        v = np.array([E._vals.get(k, 0.0) for k in names])
        c = np.array([1 if k in E._vals else 0 for k in names], np.int32)
        self.H.check(self.H.L.wg_set_energy(self.H.h, _native.ptr(v), _native.ptr(c, _native.P_I32)), "set_energy")
        E._dirty = False

    def _pull_energy(self):
        if not self.S.trackEnergy:
            return
        names = _native.ENERGY_NAMES
        v = np.zeros(len(names))
        c = np.zeros(len(names), np.int32)
        self.H.check(self.H.L.wg_get_energy(self.H.h, _native.ptr(v), _native.ptr(c, _native.P_I32)), "get_energy")
        E = self.S.energy
        for k, name in enumerate(names):
            if c[k]:
                E._vals[name] = float(v[k])
        E._resettable.update(n for n in ("kinetic", "kinTrans", "kinRot", "elast") if n in E._vals)

    def _pull_dt(self):
        """Scene.dt/nextDt and the DynDt counters after a run."""
        from .dem import DynDt
        st = self.dyndt()
        self.S.dt = float(st.dt)
        self.S.nextDt = float(st.next_dt)
        for e in self.S.engines:
            if isinstance(e, DynDt) and not e.dead:
                e.nDone, e.stepLast, e.stepPrev = int(st.n_done), int(st.step_last), int(st.step_prev)
                e.virtLast, e.virtPrev = float(st.virt_last), float(st.virt_prev)
                e.dt = float(st.dyndt_dt)

    def stats(self):
        st = _native.wg_stats()
        self.H.check(self.H.L.wg_get_stats(self.H.h, C_byref(st)), "get_stats")
        return st

    def pull(self):
        if not self.host_stale or self.H is None:
            return
        nd = self.S.dem._nodes.soa
        n = len(nd)
        out = {k: np.empty((n, w)) for k, w in (("pos", 3), ("ori", 4), ("vel", 3), ("angVel", 3), ("force", 3), ("torque", 3))}
        self.H.check(self.H.L.wg_get_nodes(self.H.h, *[_native.ptr(out[k]) for k in ("pos", "ori", "vel", "angVel", "force",
                                                                                         "torque")]), "get_nodes")
        self.host_stale = False
        for k, v in out.items():
            nd.col(k)[:] = v

    def contacts(self):
        if self._contacts is not None:
            return self._contacts
        self._contacts = read_contacts(self.H.L, self.H.h, "wg")
        return self._contacts

    def timing(self):
        tot = _ctypes_double()
        ph = np.zeros(4)
        nl = _ctypes_int64()
        self.H.L.wg_get_timing(self.H.h, C_byref(tot), _native.ptr(ph), C_byref(nl))
        return tot.value, ph, nl.value


def C_byref(x):
    import ctypes
    return ctypes.byref(x)


def _ctypes_double():
    import ctypes
    return ctypes.c_double()


def _ctypes_int64():
    import ctypes
    return ctypes.c_int64()


def read_contacts(L, h, prefix):
    """Fetch the contact list through <prefix>_num_contacts / <prefix>_get_contacts."""
    n = getattr(L, prefix + "_num_contacts")(h)
    if n < 0:
        raise RuntimeError("num_contacts failed")
    d = dict(id_lo=np.empty(n, np.int32), id_hi=np.empty(n, np.int32), id_a=np.empty(n, np.int32), real=np.empty(n, np.int32),
             cell_dist=np.empty((n, 3), np.int32), fglob=np.empty((n, 3)), local=np.empty((n, 3)), cpt=np.empty((n, 3)),
             trsf=np.empty((n, 9)))
    P32 = _native.P_I32
    r = getattr(L, prefix + "_get_contacts")(h, _native.ptr(d["id_lo"], P32), _native.ptr(d["id_hi"], P32),
                                             _native.ptr(d["id_a"], P32), _native.ptr(d["real"], P32),
                                             _native.ptr(d["cell_dist"], P32), _native.ptr(d["fglob"]), _native.ptr(d["local"]),
                                             _native.ptr(d["cpt"]), _native.ptr(d["trsf"]))
    if r != 0:
        raise RuntimeError("get_contacts failed")
    return d
