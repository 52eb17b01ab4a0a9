"""Batches of independent scenes advanced together on one GPU.

A parametric study in the reference runs many Scene objects, each with its own engine loop
(``woo-batch`` over a parameter table, py/batch.py). Here the scenes of a batch share one device
simulation: their particles, nodes and materials are concatenated, each scene keeps its own
configuration (dt, gravity, Leapfrog damping, verletDist, contact laws and their parameters,
Scene.step) and the kernels of one step (Leapfrog, collider, ContactLoop) cover every scene at
once, so a step of the whole batch costs a few launches instead of a few per scene. Particles of
different scenes never interact: each scene has its own broad-phase grid.

The results of a scene do not depend on the batch it runs in: its particles are updated with
the same operations in the same order as when it runs alone (the per-particle force sum follows
the ids of the scene's own particles, which keep their relative order). Each scene keeps its own
Scene.dt and DynDt engine (pkg/dem/DynDt.cpp:93-113): its critical timestep is the minimum over
its own nodes, and its dt changes at the steps where it would change with the scene alone.
"""
import ctypes as C

import numpy as np

from . import _native, _plan


class Batch:
    """Scenes ``scenes`` (each built like a single scene: a DemField, the engine list
    [Leapfrog, InsertionSortCollider, ContactLoop], Scene.dt) in one device simulation."""

    def __init__(self, scenes, device=0):
        self.scenes = list(scenes)
        if not self.scenes:
            raise ValueError("empty batch")
        if any(getattr(e, "_host", False) and not e.dead for S in self.scenes for e in S.engines):
            raise NotImplementedError("engines that run on the host (VtkExport) are not run in a Batch")
        self.arrays = [_plan.compile_scene(S) for S in self.scenes]
        if any(A.config.get("track_energy") for A in self.arrays):
            raise NotImplementedError("energy tracking (Scene.trackEnergy) is not supported in a Batch")
        prec = {A.config["precision"] for A in self.arrays}
        if len(prec) != 1:
            raise ValueError("the scenes of a batch share one precision mode")
        K = len(self.scenes)
        self.node_start = np.zeros(K + 1, np.int64)
        self.par_start = np.zeros(K + 1, np.int64)
        mat_start = np.zeros(K + 1, np.int64)
        for k, A in enumerate(self.arrays):
            self.node_start[k + 1] = self.node_start[k] + A.n_nodes
            self.par_start[k + 1] = self.par_start[k] + A.n_particles
            mat_start[k + 1] = mat_start[k] + len(A.materials["density"])
        cat = lambda key, grp: np.ascontiguousarray(np.concatenate([getattr(A, grp)[key] for A in self.arrays]))
        nodes = {k: cat(k, "nodes") for k in ("pos", "ori", "vel", "angVel", "force", "torque", "mass", "inertia", "flags")}
        mats = {k: cat(k, "materials") for k in ("density", "young", "tanPhi", "ktDivKn")}
        parts = {k: cat(k, "particles") for k in ("shape", "radius", "axis", "sense", "halfThick", "fakeVel", "mask")}
        pn, pm = [], []
        for k, A in enumerate(self.arrays):
            nd = A.particles["nodes"].astype(np.int32)
            pn.append(np.where(nd >= 0, nd + self.node_start[k], -1))
            pm.append(A.particles["mat"].astype(np.int32) + mat_start[k])
        parts["nodes"] = np.ascontiguousarray(np.concatenate(pn).astype(np.int32))
        parts["mat"] = np.ascontiguousarray(np.concatenate(pm).astype(np.int32))
        self.n_nodes = int(self.node_start[-1])
        self.n_particles = int(self.par_start[-1])

        self.H = _native.Handle(self.scenes[0].gpu.device if device is None else device)
        L, h = self.H.L, self.H.h
        cfgs = (_native.wg_config * K)(*[_native.make_config(_native.wg_config, A.config) for A in self.arrays])
        pstart = np.ascontiguousarray(self.par_start, dtype=np.int64)
        self.H.check(L.wg_set_scenes(h, K, C.cast(cfgs, C.c_void_p), pstart.ctypes.data_as(C.POINTER(C.c_int64))), "set_scenes")
        p = _native.ptr
        self.H.check(L.wg_set_materials(h, len(mats["density"]), p(mats["density"]), p(mats["young"]), p(mats["tanPhi"]),
                                        p(mats["ktDivKn"])), "set_materials")
        self.H.check(L.wg_set_nodes(h, self.n_nodes, p(nodes["pos"]), p(nodes["ori"]), p(nodes["vel"]), p(nodes["angVel"]),
                                    p(nodes["force"]), p(nodes["torque"]), p(nodes["mass"]), p(nodes["inertia"]),
                                    p(nodes["flags"], _native.P_U32)), "set_nodes")
        self.H.check(L.wg_set_particles(h, self.n_particles, p(parts["shape"], _native.P_I32), p(parts["nodes"], _native.P_I32),
                                        p(parts["radius"]), p(parts["axis"], _native.P_I32), p(parts["sense"], _native.P_I32),
                                        p(parts["halfThick"]), p(parts["fakeVel"]), p(parts["mat"], _native.P_I32),
                                        p(parts["mask"], _native.P_U32)), "set_particles")
        self.stale = False

    def run(self, n):
        """Advance every scene of the batch by ``n`` steps (Scene.run(n) for each); each scene
        keeps its own Scene.dt, Scene.nextDt and DynDt engine (the batch's chunks of queued steps
        end where any scene's DynDt is due)."""
        from .dem import DynDt
        L, h = self.H.L, self.H.h
        self.H.check(L.wg_run(h, int(n)), "run")
        self.stale = True
        for k, S in enumerate(self.scenes):
            st = self.scene_stats(k)
            S.step = int(st.step)
            S.time = float(st.time)
            d = _native.wg_dyndt_state()
            self.H.check(L.wg_get_scene_dyndt(h, k, C.byref(d)), "get_scene_dyndt")
            S.dt = float(d.dt)
            S.nextDt = float(d.next_dt)
            for e in S.engines:
                if isinstance(e, DynDt) and not e.dead:
                    e.nDone, e.stepLast, e.stepPrev = int(d.n_done), int(d.step_last), int(d.step_prev)
                    e.virtLast, e.virtPrev = float(d.virt_last), float(d.virt_prev)
                    e.dt = float(d.dyndt_dt)

    def scene_stats(self, k):
        st = _native.wg_stats()
        self.H.check(self.H.L.wg_get_scene_stats(self.H.h, int(k), C.cast(C.byref(st), C.c_void_p)), "get_scene_stats")
        return st

    def pull(self):
        """Bring the node state of every scene back into its host containers."""
        if not self.stale:
            return
        out = {k: np.empty((self.n_nodes, w)) for k, w in (("pos", 3), ("ori", 4), ("vel", 3), ("angVel", 3), ("force", 3),
                                                            ("torque", 3))}
        self.H.check(self.H.L.wg_get_nodes(self.H.h, *[_native.ptr(out[k]) for k in ("pos", "ori", "vel", "angVel", "force",
                                                                                         "torque")]), "get_nodes")
        for k, S in enumerate(self.scenes):
            nd = S.dem._nodes.soa
            a, b = self.node_start[k], self.node_start[k + 1]
            for key, v in out.items():
                nd.col(key)[:] = v[a:b]
        self.stale = False

    def contacts(self, k):
        """Contacts of scene k in its own particle ids (the listing of Simulation.contacts)."""
        c = _plan.read_contacts(self.H.L, self.H.h, "wg")
        a, b = self.par_start[k], self.par_start[k + 1]
        sel = (c["id_lo"] >= a) & (c["id_lo"] < b)
        out = {key: v[sel] for key, v in c.items()}
        for key in ("id_lo", "id_hi", "id_a"):
            out[key] = (out[key] - a).astype(np.int32)
        return out

    def timing(self):
        tot = C.c_double()
        ph = np.zeros(4)
        nl = C.c_int64()
        self.H.L.wg_get_timing(self.H.h, C.byref(tot), _native.ptr(ph), C.byref(nl))
        return tot.value, ph, nl.value

    def close(self):
        if self.H is not None:
            self.pull()
            self.H.close()
            self.H = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# parameter tables of woo-batch (py/batch.py), feeding Batch
from ._table import (TableParamReader, cartProdParamTable, dbFormatVersion, dbReadResults, dbToJSON, dbToSpread,  # noqa: E402,F401
                     inBatch, options, readParamsFromTable, runPreprocessor, runTable, planTable, wait, writeResults)

if __name__ == "__main__":
    import sys
    from ._table import main
    sys.exit(main())
