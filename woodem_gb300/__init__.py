"""woodem_gb300: the per-step DEM hot path of Woo (InsertionSortCollider -> ContactLoop with
Sphere/Facet/Wall L6Geom functors, FrictPhys/IdealElPl and Hertz laws -> Leapfrog) on a GB300.

Submodules mirror Woo's scripting layout so that ``import woodem_gb300 as woo`` runs
existing scene scripts: ``woo.core.Scene``, ``woo.dem.*``, ``woo.utils.*``,
``woo.triangulated.cylinder``, ``woo.pack.SpherePack``, ``woo.batch`` (parameter tables). The
step loop itself runs in libwoogpu.so (C ABI in include/woo_gpu.h); there is no CPU fallback.
"""
from . import core, dem, utils, triangulated, pack, batch  # noqa: F401
from .core import Scene, Cell  # noqa: F401

__all__ = ["core", "dem", "utils", "triangulated", "pack", "batch", "Scene", "Cell"]
