"""ctypes wrapper of the CPU oracle (test infrastructure only).

Feeds the same flat scene description as the GPU library (woodem_gb300._plan.SceneArrays)
to libwoo_oracle.so and reads back node state and contacts in the same formats.
"""
import ctypes as C
import os

import numpy as np

from woodem_gb300 import _native
from woodem_gb300._plan import read_contacts

HERE = os.path.dirname(os.path.abspath(__file__))
_L = {}


def lib(fast=False):
    """The parity build (bitwise comparisons) or, with ``fast``, the timing build of the CPU baseline."""
    if fast in _L:
        return _L[fast]
    from . import build as _b  # noqa
    path = os.path.join(HERE, "_build", "libwoo_oracle_fast.so" if fast else "libwoo_oracle.so")
    if not os.path.exists(path):
        _b.build()
    L = C.CDLL(path)
    P_D, P_I32, P_U32 = _native.P_D, _native.P_I32, _native.P_U32
    sig = {
        "wo_create": (C.c_void_p, []),
        "wo_destroy": (None, [C.c_void_p]),
        "wo_last_error": (C.c_char_p, [C.c_void_p]),
        "wo_set_threads": (C.c_int, [C.c_void_p, C.c_int]),
        "wo_set_config": (C.c_int, [C.c_void_p, C.POINTER(_native.wg_config)]),
        "wo_set_materials": (C.c_int, [C.c_void_p, C.c_int32, P_D, P_D, P_D, P_D]),
        "wo_set_nodes": (C.c_int, [C.c_void_p, C.c_int64, P_D, P_D, P_D, P_D, P_D, P_D, P_D, P_D, P_U32]),
        "wo_set_particles": (C.c_int, [C.c_void_p, C.c_int64, P_I32, P_I32, P_D, P_I32, P_I32, P_D, P_D, P_I32, P_U32]),
        "wo_run": (C.c_int, [C.c_void_p, C.c_int64]),
        "wo_collide_only": (C.c_int, [C.c_void_p]),
        "wo_get_nodes": (C.c_int, [C.c_void_p, P_D, P_D, P_D, P_D, P_D, P_D]),
        "wo_get_stats": (C.c_int, [C.c_void_p, C.POINTER(_native.wg_stats)]),
        "wo_get_dyndt": (C.c_int, [C.c_void_p, C.POINTER(_native.wg_dyndt_state)]),
        "wo_get_energy": (C.c_int, [C.c_void_p, _native.P_D, _native.P_I32]),
        "wo_num_contacts": (C.c_int64, [C.c_void_p]),
        "wo_get_contacts": (C.c_int, [C.c_void_p, P_I32, P_I32, P_I32, P_I32, P_I32, P_D, P_D, P_D, P_D]),
        "wo_kinetic_energy": (C.c_int, [C.c_void_p, P_D]),
        "wo_get_aabbs": (C.c_int, [C.c_void_p, P_D, P_D]),
        "wo_get_cell": (C.c_int, [C.c_void_p, P_D, P_D, P_D]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _L[fast] = L
    return L


class Oracle:
    """One oracle scene built from SceneArrays."""

    def __init__(self, A, threads=1, deterministic=True, fast=False):
        self.L = L = lib(fast)
        self.h = L.wo_create()
        self.n_nodes = A.n_nodes
        L.wo_set_threads(self.h, int(threads))
        cfg = dict(A.config)
        cfg["deterministic"] = 1 if deterministic else 0
        self._check(L.wo_set_config(self.h, _native.make_config(_native.wg_config, cfg)), "set_config")
        m = A.materials
        p = _native.ptr
        self._check(L.wo_set_materials(self.h, len(m["density"]), p(m["density"]), p(m["young"]), p(m["tanPhi"]),
                                       p(m["ktDivKn"])), "set_materials")
        nd = A.nodes
        self._check(L.wo_set_nodes(self.h, A.n_nodes, p(nd["pos"]), p(nd["ori"]), p(nd["vel"]), p(nd["angVel"]),
                                   p(nd["force"]), p(nd["torque"]), p(nd["mass"]), p(nd["inertia"]),
                                   p(nd["flags"], _native.P_U32)), "set_nodes")
        pa = A.particles
        I32, U32 = _native.P_I32, _native.P_U32
        self._check(L.wo_set_particles(self.h, A.n_particles, p(pa["shape"], I32), p(pa["nodes"], I32), p(pa["radius"]),
                                       p(pa["axis"], I32), p(pa["sense"], I32), p(pa["halfThick"]), p(pa["fakeVel"]),
                                       p(pa["mat"], I32), p(pa["mask"], U32)), "set_particles")

    def _check(self, r, what):
        if r != 0:
            raise RuntimeError("oracle %s: %s" % (what, self.L.wo_last_error(self.h).decode()))

    def run(self, n):
        self._check(self.L.wo_run(self.h, int(n)), "run")

    def collide_only(self):
        self._check(self.L.wo_collide_only(self.h), "collide_only")

    def nodes(self):
        n = self.n_nodes
        out = {k: np.empty((n, w)) for k, w in (("pos", 3), ("ori", 4), ("vel", 3), ("angVel", 3), ("force", 3), ("torque", 3))}
        p = _native.ptr
        self._check(self.L.wo_get_nodes(self.h, p(out["pos"]), p(out["ori"]), p(out["vel"]), p(out["angVel"]),
                                        p(out["force"]), p(out["torque"])), "get_nodes")
        return out

    def energy(self):
        """Scene.energy as {name: value} of the entries that exist."""
        v = np.zeros(len(_native.ENERGY_NAMES))
        c = np.zeros(len(_native.ENERGY_NAMES), np.int32)
        self._check(self.L.wo_get_energy(self.h, _native.ptr(v), _native.ptr(c, _native.P_I32)), "get_energy")
        return {n: float(v[k]) for k, n in enumerate(_native.ENERGY_NAMES) if c[k]}

    def dyndt(self):
        st = _native.wg_dyndt_state()
        self._check(self.L.wo_get_dyndt(self.h, C.byref(st)), "get_dyndt")
        return st

    def stats(self):
        st = _native.wg_stats()
        self.L.wo_get_stats(self.h, C.byref(st))
        return st

    def contacts(self):
        return read_contacts(self.L, self.h, "wo")

    def aabbs(self, n):
        mn, mx = np.empty((n, 3)), np.empty((n, 3))
        self.L.wo_get_aabbs(self.h, _native.ptr(mn), _native.ptr(mx))
        return mn, mx

    def cell(self):
        hs, tr, gv = np.zeros(9), np.zeros(9), np.zeros(9)
        self.L.wo_get_cell(self.h, _native.ptr(hs), _native.ptr(tr), _native.ptr(gv))
        return hs.reshape(3, 3), tr.reshape(3, 3), gv.reshape(3, 3)

    def close(self):
        if self.h:
            self.L.wo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
