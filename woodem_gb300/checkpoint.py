"""Checkpoint and resume of a scene's device state.

``save(S, path)`` writes one flat ``.npz`` file: the node state (pos, ori, vel, angVel, force,
torque), the contact container with the persistent contact state (``wg_get_contact_state``),
Scene.step/time/dt, the counters of a DynDt engine, Scene.energy and the periodic cell (hSize,
trsf, gradV, nextGradV). ``load(S, path)``
puts that state into a scene built the same way (the same particles, materials and engines:
a fingerprint of the compiled description is checked) and uploads it; the next step starts with
a collider full run that keeps the state of the real contacts, as the reference's Scene.load
invalidates the collider (pkg/dem/InsertionSortCollider.hpp:221). In FP64 mode the resumed run
continues bitwise as the saved one would have.
"""
import ctypes as C
import hashlib
import json

import numpy as np

from . import _native, _plan

_NODE_COLS = ("pos", "ori", "vel", "angVel", "force", "torque")
# configuration entries that describe the state, not the scene
_STATE_CFG = ("step", "time", "dt", "next_dt", "cell_hsize", "cell_trsf", "cell_gradv", "cell_next_gradv", "dyndt_n_done",
              "dyndt_step_last", "dyndt_step_prev", "dyndt_virt_last", "dyndt_virt_prev")
# DynDt counters (PeriodicEngine) saved with the state
_DYNDT_ATTRS = ("nDone", "stepLast", "stepPrev", "virtLast", "virtPrev")


def fingerprint(A):
    """Hash of a compiled scene description (particles, materials, node constants, engine
    configuration) without its evolving state."""
    h = hashlib.sha256()
    for d in (A.particles, A.materials):
        for k in sorted(d):
            h.update(k.encode())
            h.update(np.ascontiguousarray(d[k]).tobytes())
    for k in ("mass", "inertia", "flags"):
        h.update(k.encode())
        h.update(np.ascontiguousarray(A.nodes[k]).tobytes())
    for k in sorted(A.config):
        if k in _STATE_CFG:
            continue
        h.update(k.encode())
        h.update(np.ascontiguousarray(np.asarray(A.config[k])).tobytes())
    return h.hexdigest()


def contact_snapshot(S):
    """The contact container of S's device simulation with its persistent state
    (``wg_get_contact_state``): {con_key, con_flags, con_step0, con_cell_dist, con_state,
    state_cols}."""
    sim = S._sim
    L, h = sim.H.L, sim.H.h
    ncols = int(L.wg_contact_state_cols(h))
    n = C.c_int64()
    r = L.wg_get_contact_state(h, 0, C.byref(n), None, None, None, None, None)
    if r not in (0, _native.WG_ERR_CAPACITY):
        sim.H.check(r, "get_contact_state")
    m = n.value
    key = np.empty(m, np.uint64)
    flags = np.empty(m, np.uint32)
    step0 = np.empty(m, np.int32)
    cdist = np.empty(m, np.int32)
    cols = np.empty((m, ncols))
    if m:
        sim.H.check(L.wg_get_contact_state(h, m, C.byref(n), key.ctypes.data, flags.ctypes.data, step0.ctypes.data, cdist.ctypes.data,
                                           cols.ctypes.data), "get_contact_state")
    return {"con_key": key, "con_flags": flags, "con_step0": step0, "con_cell_dist": cdist, "con_state": cols,
            "state_cols": ncols}


def restore_contacts(S, snap):
    """Upload the contact container ``snap`` (of contact_snapshot) into S's device simulation,
    creating it from S's host state; the next step starts with a full collider run that keeps the
    state of the real contacts."""
    sim = S._ensure_sim()
    L, h = sim.H.L, sim.H.h
    key = np.ascontiguousarray(snap["con_key"], np.uint64)
    m = len(key)
    ncols = int(snap["state_cols"])
    cols = np.ascontiguousarray(snap["con_state"], float).reshape(m, ncols)
    sim.H.check(L.wg_set_contact_state(h, m, key.ctypes.data, np.ascontiguousarray(snap["con_flags"], np.uint32).ctypes.data,
                                       np.ascontiguousarray(snap["con_step0"], np.int32).ctypes.data,
                                       np.ascontiguousarray(snap["con_cell_dist"], np.int32).ctypes.data, cols.ctypes.data,
                                       ncols), "set_contact_state")


def save(S, path):
    """Write the device state of scene S (which has run at least once) to ``path``."""
    sim = S._sim
    if sim is None:
        raise RuntimeError("the scene has no device state to save; run it first")
    S.sync()
    nd = S.dem._nodes.soa
    arrays = {"node_" + k: np.array(nd.col(k)) for k in _NODE_COLS}
    snap = contact_snapshot(S)
    ncols = snap.pop("state_cols")
    arrays.update(snap)
    meta = {"step": int(S.step), "time": float(S.time), "dt": float(S.dt), "precision": S.gpu.precision,
            "periodic": bool(S.isPeriodic), "n_nodes": int(len(nd)), "state_cols": ncols, "fingerprint": fingerprint(sim.A)}
    dyn = _dyndt(S)
    if dyn is not None:
        meta["dyndt"] = {k: getattr(dyn, k) for k in _DYNDT_ATTRS}
    if S.trackEnergy:
        meta["energy"] = dict(S.energy._vals)
    if S.isPeriodic:
        for k in ("hSize", "trsf", "gradV", "nextGradV"):
            arrays["cell_" + k] = np.array(getattr(S.cell, k), dtype=float)
    np.savez(path, meta=np.array(json.dumps(meta)), **arrays)


def _dyndt(S):
    from .dem import DynDt
    for e in S.engines:
        if isinstance(e, DynDt) and not e.dead:
            return e
    return None


def load(S, path):
    """Resume scene S (built as the saved one was) from the state saved in ``path``."""
    with np.load(path) as data:
        meta = json.loads(str(data["meta"]))
        arrays = {k: np.array(data[k]) for k in data.files if k != "meta"}
    S._invalidate()
    if S.gpu.precision != meta["precision"]:
        raise ValueError("the checkpoint was saved in precision mode %s" % meta["precision"])
    nd = S.dem._nodes.soa
    if len(nd) != meta["n_nodes"]:
        raise ValueError("the checkpoint holds %d nodes, the scene %d" % (meta["n_nodes"], len(nd)))
    if fingerprint(_plan.compile_scene(S)) != meta["fingerprint"]:
        raise ValueError("the checkpoint was saved from a different scene (particles, materials or engines)")
    for k in _NODE_COLS:
        nd.col(k)[:] = arrays["node_" + k]
    S.step = meta["step"]
    S.time = meta["time"]
    S.dt = meta["dt"]
    dyn = _dyndt(S)
    if (dyn is None) != ("dyndt" not in meta):
        raise ValueError("the checkpoint and the scene differ in having a DynDt engine")
    if dyn is not None:
        for k, v in meta["dyndt"].items():
            setattr(dyn, k, v)
    if "energy" in meta:
        S.energy.clear()
        for k, v in meta["energy"].items():
            S.energy[k] = v
    if meta["periodic"]:
        S.cell.hSize = arrays["cell_hSize"]
        S.cell.trsf = arrays["cell_trsf"]
        S.cell.setCurrGradV(arrays["cell_gradV"])
        S.cell.nextGradV = arrays["cell_nextGradV"]
    restore_contacts(S, dict({k: arrays[k] for k in ("con_key", "con_flags", "con_step0", "con_cell_dist", "con_state")},
                             state_cols=meta["state_cols"]))
    return S
