"""ctypes binding of libwoogpu.so (include/woo_gpu.h).

The product path has no CPU fallback: if the library is missing or fails to load,
every entry point raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwoogpu.so")

WG_OK = 0
WG_ERR_CAPACITY = -5
ERRORS = {-1: ValueError, -2: RuntimeError, -3: RuntimeError, -4: NotImplementedError, -5: MemoryError, -6: RuntimeError,
          -7: RuntimeError}


class wg_config(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("gravity", C.c_double * 3), ("lone_mask", C.c_uint32), ("deterministic", C.c_int32),
        ("step", C.c_int64), ("damping", C.c_double), ("reset", C.c_int32), ("_pad0", C.c_int32),
        ("verlet_dist", C.c_double), ("bo1_sphere_dist_factor", C.c_double), ("sort_axis", C.c_int32),
        ("apply_forces", C.c_int32), ("cg2_ss_dist_factor", C.c_double), ("trsf_renorm", C.c_int32),
        ("approx_mask", C.c_int32), ("no_ratch", C.c_int32), ("phys", C.c_int32), ("law", C.c_int32),
        ("no_slip", C.c_int32), ("no_break", C.c_int32), ("no_frict", C.c_int32), ("hz_poisson", C.c_double),
        ("hz_gamma", C.c_double), ("hz_en", C.c_double), ("hz_alpha", C.c_double), ("hz_no_attraction", C.c_int32),
        ("periodic", C.c_int32), ("homo_deform", C.c_int32), ("eval_stress", C.c_int32),
        ("cell_hsize", C.c_double * 9), ("cell_trsf", C.c_double * 9), ("cell_gradv", C.c_double * 9),
        ("cell_next_gradv", C.c_double * 9), ("precision", C.c_int32), ("_pad1", C.c_int32),
        ("dyndt", C.c_int32), ("dyndt_dry_run", C.c_int32), ("dyndt_step_modulo", C.c_int32), ("dyndt_init_run", C.c_int32),
        ("dyndt_step_period", C.c_int64), ("dyndt_n_do", C.c_int64), ("dyndt_n_done", C.c_int64),
        ("dyndt_step_last", C.c_int64), ("dyndt_step_prev", C.c_int64), ("dyndt_virt_period", C.c_double),
        ("dyndt_virt_last", C.c_double), ("dyndt_virt_prev", C.c_double), ("dyndt_max_rel_inc", C.c_double),
        ("dt_safety", C.c_double), ("next_dt", C.c_double), ("time", C.c_double), ("track_energy", C.c_int32),
        ("kin_split", C.c_int32),
    ]

# Scene.energy entries in the order of WG_ENERGY_NAMES (include/woo_gpu.h)
ENERGY_NAMES = ("kinetic", "kinTrans", "kinRot", "grav", "nonviscDamp", "elast", "plast", "broken", "viscN", "viscT", "gradV")


class wg_dyndt_state(C.Structure):
    _fields_ = [("dt", C.c_double), ("next_dt", C.c_double), ("dyndt_dt", C.c_double), ("crit_dt", C.c_double),
                ("n_done", C.c_int64), ("step_last", C.c_int64), ("step_prev", C.c_int64), ("n_evals", C.c_int64),
                ("virt_last", C.c_double), ("virt_prev", C.c_double)]


class wg_stats(C.Structure):
    _fields_ = [("step", C.c_int64), ("n_full_runs", C.c_int64), ("n_contacts", C.c_int64), ("n_real", C.c_int64),
                ("time", C.c_double), ("verlet_dist", C.c_double), ("stress", C.c_double * 9)]


def make_config(cls, d):
    """Fill a ctypes config struct (wg_config or the oracle's identical layout) from a dict."""
    c = cls()
    for k, v in d.items():
        f = getattr(c, k)
        if isinstance(f, C.Array):
            for i, x in enumerate(np.asarray(v, dtype=float).ravel()):
                f[i] = x
        else:
            setattr(c, k, v)
    return c


_lib = None

P_D = C.POINTER(C.c_double)
P_I32 = C.POINTER(C.c_int32)
P_U32 = C.POINTER(C.c_uint32)
P_I64 = C.POINTER(C.c_int64)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libwoogpu.so is not built (run __graft_entry__.build() or python -m woodem_gb300._build); "
                          "the GPU path has no CPU fallback")
    L = C.CDLL(LIB_PATH)
    sig = {
        "wg_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
        "wg_destroy": (None, [C.c_void_p]),
        "wg_last_error": (C.c_char_p, [C.c_void_p]),
        "wg_set_config": (C.c_int, [C.c_void_p, C.POINTER(wg_config)]),
        "wg_set_materials": (C.c_int, [C.c_void_p, C.c_int32, P_D, P_D, P_D, P_D]),
        "wg_set_nodes": (C.c_int, [C.c_void_p, C.c_int64, P_D, P_D, P_D, P_D, P_D, P_D, P_D, P_D, P_U32]),
        "wg_set_particles": (C.c_int, [C.c_void_p, C.c_int64, P_I32, P_I32, P_D, P_I32, P_I32, P_D, P_D, P_I32, P_U32]),
        "wg_run": (C.c_int, [C.c_void_p, C.c_int64]),
        "wg_run_host": (C.c_int, [C.c_void_p, C.c_int64, P_D, P_D, P_D, P_D, P_D, P_D]),
        "wg_put_state": (C.c_int, [C.c_void_p, P_D, P_D, P_D, P_D, P_D, P_D]),
        "wg_get_nodes": (C.c_int, [C.c_void_p, P_D, P_D, P_D, P_D, P_D, P_D]),
        "wg_get_stats": (C.c_int, [C.c_void_p, C.POINTER(wg_stats)]),
        "wg_get_dyndt": (C.c_int, [C.c_void_p, C.POINTER(wg_dyndt_state)]),
        "wg_get_scene_dyndt": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(wg_dyndt_state)]),
        "wg_set_dt": (C.c_int, [C.c_void_p, C.c_double, C.c_double]),
        "wg_get_energy": (C.c_int, [C.c_void_p, P_D, P_I32]),
        "wg_set_energy": (C.c_int, [C.c_void_p, P_D, P_I32]),
        "wg_set_next_gradv": (C.c_int, [C.c_void_p, P_D]),
        "wg_set_scenes": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_int64)]),
        "wg_get_scene_stats": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
        "wg_set_launch": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
        "wg_slot_load": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, P_D, P_D, P_D, P_D, P_D, P_D, P_U32, P_I32, P_D,
                                   P_I32, P_I32, P_I32, P_U32, C.c_int32, P_D, P_D, P_D, P_D, C.c_int64]),
        "wg_slot_clear": (C.c_int, [C.c_void_p, C.c_int32]),
        "wg_slot_status": (C.c_int, [C.c_void_p, C.c_int32, P_I64, P_I64]),
        "wg_get_slot_nodes": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, P_D, P_D, P_D, P_D, P_D, P_D]),
        "wg_get_cell": (C.c_int, [C.c_void_p, P_D, P_D, P_D]),
        "wg_num_contacts": (C.c_int64, [C.c_void_p]),
        "wg_get_contacts": (C.c_int, [C.c_void_p, P_I32, P_I32, P_I32, P_I32, P_I32, P_D, P_D, P_D, P_D]),
        "wg_collide_only": (C.c_int, [C.c_void_p]),
        "wg_get_aabbs": (C.c_int, [C.c_void_p, P_D, P_D]),
        "wg_get_timing": (C.c_int, [C.c_void_p, P_D, P_D, P_I64]),
        "wg_profiler": (C.c_int, [C.c_int]),
        "wg_contact_state_cols": (C.c_int32, [C.c_void_p]),
        "wg_get_contact_state": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int64), C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p]),
        "wg_set_contact_state": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_int32]),
        "wg_host_alloc": (C.c_void_p, [C.c_int64]),
        "wg_host_free": (None, [C.c_void_p]),
        "wg_broadphase_noalloc": (C.c_int, [C.c_int32, P_D, P_D, P_U32, C.c_uint32, C.c_int64, P_I32, P_I32, P_I64]),
        "wg_broadphase_noalloc_error": (C.c_char_p, []),
        "wg_pack_rsa": (C.c_int64, [C.c_int64, P_D, P_D, P_D, C.c_int32, P_D, C.c_uint64, C.c_int64, P_D]),
        "wg_pack_rsa_device": (C.c_int64, [C.c_int64, P_D, P_D, P_D, C.c_int32, P_D, C.c_uint64, C.c_int64, P_D]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def ptr(a, t=P_D):
    if a is None:
        return C.cast(None, t)
    return a.ctypes.data_as(t)


class Handle:
    """Owns one wg_scene."""

    def __init__(self, device=0):
        L = lib()
        h = C.c_void_p()
        r = L.wg_create(C.byref(h), int(device))
        if r != WG_OK:
            raise ERRORS.get(r, RuntimeError)("wg_create: " + L.wg_last_error(None).decode())
        self.h = h
        self.L = L

    def check(self, r, what):
        if r != WG_OK:
            msg = self.L.wg_last_error(self.h).decode()
            raise ERRORS.get(r, RuntimeError)("%s: %s" % (what, msg))

    def close(self):
        if self.h:
            self.L.wg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
