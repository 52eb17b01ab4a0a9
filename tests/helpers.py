"""Shared helpers of the test-suite: scene construction and oracle/GPU comparison."""
import numpy as np

import woodem_gb300 as woo
from woodem_gb300 import utils, _plan
from woodem_gb300.dem import (DemField, FrictMat, Cp2_FrictMat_HertzPhys, Law2_L6Geom_HertzPhys_DMT)


def two_spheres(gap=1e-6, v0=1.0, r=0.05, hertz=True, mat=None, fixed_a=False, offset=(0, 0, 0), dt=None, damping=0.0,
                verlet=-0.05):
    """Two equal spheres on the y axis approaching each other with relative speed v0."""
    S = woo.core.Scene(fields=[DemField()])
    m = mat or FrictMat(density=1e3, young=1e8, ktDivKn=.2, tanPhi=.5)
    off = np.asarray(offset, float)
    a = utils.sphere(off + (0, 0, 0), r, fixed=fixed_a, mat=m)
    b = utils.sphere(off + (0, 2 * r + gap, 0), r, mat=m)
    S.dem.par.add([a, b])
    a.vel = (0, 0 if fixed_a else v0 / 2, 0)
    b.vel = (0, -v0 / 2 if not fixed_a else -v0, 0)
    if hertz:
        S.engines = utils.defaultEngines(damping=damping, cp2=Cp2_FrictMat_HertzPhys(gamma=0, en=0, poisson=.2),
                                         law=Law2_L6Geom_HertzPhys_DMT(), dynDtPeriod=0, verletDist=verlet)
    else:
        S.engines = utils.defaultEngines(damping=damping, dynDtPeriod=0, verletDist=verlet)
    S.dt = dt if dt else 0.3 * utils.pWaveDt(S)
    return S


def assert_contacts_equal(a, b, bitwise=True, rtol=0.0, atol=0.0):
    assert np.array_equal(a["id_lo"], b["id_lo"]), "contact pair sets differ (lo ids)"
    assert np.array_equal(a["id_hi"], b["id_hi"]), "contact pair sets differ (hi ids)"
    assert np.array_equal(a["real"], b["real"]), "real flags differ"
    assert np.array_equal(a["id_a"], b["id_a"]), "contact orientation (pA) differs"
    for k in ("fglob", "local", "cpt"):
        if bitwise:
            assert np.array_equal(a[k], b[k]), "contact %s differs (max abs %g)" % (k, np.max(np.abs(a[k] - b[k])) if len(a[k]) else 0)
        else:
            np.testing.assert_allclose(a[k], b[k], rtol=rtol, atol=atol)


def brute_force_pairs(A, mn, mx):
    """{(i,j): closed AABB overlap and masks allow} for the boxes mn/mx (n x 3)."""
    n = len(mn)
    mask = A.particles["mask"].astype(np.int64)
    lone = A.config["lone_mask"]
    ov = np.ones((n, n), bool)
    for k in range(3):
        ov &= (mn[:, None, k] <= mx[None, :, k]) & (mx[:, None, k] >= mn[None, :, k])
    mm = mask[:, None] & mask[None, :]
    ov &= (mm != 0) & ((mm & lone) == 0)
    i, j = np.nonzero(np.triu(ov, 1))
    return set(zip(i.tolist(), j.tolist()))
