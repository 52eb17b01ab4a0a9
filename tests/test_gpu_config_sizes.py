"""Parity at the sizes of the benchmark configurations themselves.

* 1M-sphere rotating Hertz drum (20 000 facets, 2 rotating wall caps), compacted on the GPU:
  FP64 plain mode against the FP64 oracle, bitwise, over at least 80 steps and until a collider
  full run after the first one; FP32-force mode against FP64 from the same state after one step.
* 200 000-sphere periodic cell, compressed to solid fraction 0.62 and sheared (xz rate 1/s):
  FP64 plain mode against the oracle, bitwise (cellDist, the cell and ContactLoop.stress
  included); FP32-force mode against FP64: forces, stress tensor and coordination number.
* 10 000-sphere box settle: the whole 20 000 steps of the configuration in FP64, bitwise.

Tolerances (written here; the same definitions as in test_gpu_fp32 and test_gpu_parity):
  * FP64 plain: bitwise positions, velocities, forces, torques, contact set and per-contact state;
    node orientation within 1e-14 (sin/cos last bit); ContactLoop.stress within 1e-12 relative
    (the oracle adds the contact terms in another order).
  * FP32-force against FP64, one step from the same state: per-contact global force within 1e-5
    of the contact force for contacts above 1e-4 of the largest force, and within 1e-9 of the
    largest force below that (the FP32-force overlap is exact to ~2^-46 of the centre distance,
    which is a growing fraction of an ever smaller overlap), per-particle net force within
    1e-5 of the particle's largest contact force (particles whose largest contact force is above
    1e-6 of the largest one: the same cut as for contacts), stress tensor within 1e-5 (Frobenius, relative),
    identical coordination number (same contact set and real flags).
"""
import os

import numpy as np
import pytest

from woodem_gb300 import scenes, _plan, _native
from woodem_gb300.dem import ContactLoop

pytestmark = pytest.mark.gpu

THREADS = max(1, os.cpu_count() or 1)


def _oracle(A):
    from oracle.oracle import Oracle
    return Oracle(A, threads=THREADS, deterministic=True)


def _nodes(S):
    S.sync()
    nd = S.dem._nodes.soa
    return {k: nd.col(k).copy() for k in ("pos", "ori", "vel", "angVel", "force", "torque")}


def _overlap_peri(mn, mx, a, b, size):
    """InsertionSortCollider::spatialOverlapPeri (pkg/dem/InsertionSortCollider.cpp:903-957) for
    one pair: whether the boxes overlap in the periodic cell of the given edge lengths, and the
    periods (cellDist) of the overlap."""
    periods = [0, 0, 0]
    for ax in range(3):
        dim = size[ax]
        m1, m2 = mn[a, ax], mn[b, ax]
        if np.isinf(m1) or np.isinf(m2):
            continue
        rel = lambda x, x0: ((x - x0) / dim - np.floor((x - x0) / dim)) * dim
        w = m2 if rel(m1, m2) < rel(m2, m1) else m1

        def wrap(x):
            xn = (x - w) / dim
            p = np.floor(xn)
            return w + (xn - p) * dim, int(p)
        (mn1, p1), (mx1, _) = wrap(mn[a, ax]), wrap(mx[a, ax])
        (mn2, p2), (mx2, _) = wrap(mn[b, ax]), wrap(mx[b, ax])
        periods[ax] = p1 - p2
        if not (mn1 <= mx2 and mx1 >= mn2):
            return False, periods
    return True, periods


def _assert_bitwise(S, O):
    g, o = _nodes(S), O.nodes()
    for k in ("pos", "vel", "angVel", "force", "torque"):
        assert np.array_equal(g[k], o[k]), "%s differs (max abs %g)" % (k, np.max(np.abs(g[k] - o[k])))
    assert np.max(np.abs(g["ori"] - o["ori"])) <= 1e-14
    cg, co = S._sim.contacts(), O.contacts()
    kg = cg["id_lo"].astype(np.int64) << 32 | cg["id_hi"].astype(np.int64)
    ko = co["id_lo"].astype(np.int64) << 32 | co["id_hi"].astype(np.int64)
    if S.isPeriodic and not np.array_equal(kg, ko):
        # The reference's periodic insertion sort makes one pass over its circular bound lists
        # (InsertionSortCollider.cpp:718-791); a pass can leave an inversion next to the wrap
        # point, and an overlap that begins there is found only at a later inversion of that
        # pair. The GPU computes the exact overlap set, so it may hold such a pair earlier: it
        # must be a pair that is not real and whose boxes overlap (spatialOverlapPeri, with
        # cellDist its periods); the pairs of both sets must be the same otherwise.
        assert np.all(np.isin(ko, kg)), "pairs of the oracle missing on the GPU: %s" % ko[~np.isin(ko, kg)][:5]
        extra = ~np.isin(kg, ko)
        A = _plan.compile_scene(S)
        mn, mx = np.empty((A.n_particles, 3)), np.empty((A.n_particles, 3))
        S._sim.H.check(S._sim.H.L.wg_get_aabbs(S._sim.H.h, _native.ptr(mn), _native.ptr(mx)), "get_aabbs")
        size = np.linalg.norm(np.asarray(S.cell.hSize, float), axis=0)
        for i in np.nonzero(extra)[0]:
            a, b = int(cg["id_lo"][i]), int(cg["id_hi"][i])
            ov, per = _overlap_peri(mn, mx, a, b, size)
            assert cg["real"][i] == 0 and ov and list(cg["cell_dist"][i]) == per, \
                "GPU pair (%d, %d) is not an overlap the oracle has yet to find" % (a, b)
        print("%d pair(s) found by the GPU ahead of the reference's periodic insertion sort" % int(extra.sum()))
        cg = {k: v[~extra] for k, v in cg.items()}
    assert np.array_equal(cg["id_lo"], co["id_lo"]) and np.array_equal(cg["id_hi"], co["id_hi"]), \
        "pair sets differ: %d gpu vs %d oracle" % (len(cg["id_lo"]), len(co["id_lo"]))
    assert np.array_equal(cg["real"], co["real"]) and np.array_equal(cg["id_a"], co["id_a"])
    assert np.array_equal(cg["cell_dist"], co["cell_dist"])
    for k in ("fglob", "local", "cpt"):
        assert np.array_equal(cg[k], co[k]), "contact %s differs (max abs %g)" % (k, np.max(np.abs(cg[k] - co[k])))
    r = cg["real"] != 0
    assert np.array_equal(cg["trsf"][r], co["trsf"][r])
    assert S._sim.stats().n_full_runs == O.stats().n_full_runs
    return int(np.count_nonzero(r)), len(r)


def _state(S):
    S.sync()
    nd = S.dem._nodes.soa
    st = {k: nd.col(k).copy() for k in ("pos", "ori", "vel", "angVel", "force", "torque")}
    if S.isPeriodic:
        st["_cell"] = (np.array(S.cell.hSize, float), np.array(S.cell.trsf, float), np.array(S.cell._gradV, float),
                       np.array(S.cell.nextGradV, float))
    return st


def _restore(S, st):
    S.close()
    nd = S.dem._nodes.soa
    for k, v in st.items():
        if k != "_cell":
            nd.col(k)[:] = v
    if "_cell" in st:
        hs, tr, gv, ngv = st["_cell"]
        S.cell.hSize, S.cell.trsf, S.cell._gradV, S.cell.nextGradV = hs.copy(), tr.copy(), gv.copy(), ngv.copy()
    S.step = 0
    S.time = 0.0


def _one_step_errors(S64, S32, A):
    """Contact and particle force errors of FP32 against FP64 after one step from the same state."""
    c64, c32 = S64._sim.contacts(), S32._sim.contacts()
    assert np.array_equal(c64["id_lo"], c32["id_lo"]) and np.array_equal(c64["id_hi"], c32["id_hi"])
    assert np.array_equal(c64["real"], c32["real"]), "real flags differ after one step"
    real = c64["real"] != 0
    F64, F32 = c64["fglob"][real], c32["fglob"][real]
    mag = np.linalg.norm(F64, axis=1)
    rel_contact = np.linalg.norm(F64 - F32, axis=1) / np.maximum(mag, 1e-4 * mag.max())
    f64, f32 = _nodes(S64)["force"], _nodes(S32)["force"]
    fmax = np.zeros(A.n_particles)
    np.maximum.at(fmax, np.concatenate([c64["id_lo"][real], c64["id_hi"][real]]), np.concatenate([mag, mag]))
    sph = (A.particles["shape"] == 0) & (fmax > 1e-6 * mag.max())
    nodes = A.particles["nodes"][:, 0]
    rel_part = np.linalg.norm(f64[nodes[sph]] - f32[nodes[sph]], axis=1) / fmax[sph]
    return rel_contact, rel_part, int(np.count_nonzero(real))


# ------------------------------------------------------------------------------ 1M Hertz drum
@pytest.fixture(scope="module")
def drum_1m(gpu_lib):
    """The benchmark drum: 1 000 000 lognormal spheres (median 3 mm), a 1.2 m x 0.6 m drum of
    20 000 facets and 2 rotating wall caps, Hertz DMT; the random fill compacted on the GPU as the
    benchmark does (16 000 steps at 40 g, 12 000 easing back to 1 g), so that the bed carries
    millions of real contacts, facet and cap contacts included. Returns the sphere state."""
    S = scenes.hertz_drum(n=1_000_000, seed=0, precision="fp64", settle_steps=16000, settle_g=40.0)
    st = {k: scenes._sphere_nodes(S, k) for k in ("pos", "vel", "angVel")}
    st["radius"] = scenes.sphere_radii(S)
    S.close()
    return st


def _drum(st, prec):
    return scenes.hertz_drum_from_state(st["pos"], st["radius"], st["vel"], st["angVel"], precision=prec)


def test_drum_1m_fp64_bitwise(drum_1m):
    S = _drum(drum_1m, "fp64")
    O = _oracle(_plan.compile_scene(S))
    done = 0
    for k in (1, 19, 60):
        S.run(k)
        O.run(k)
        done += k
        n_real, n_con = _assert_bitwise(S, O)
    # on until the window holds a full run after the first one (every ~30 steps in the settled bed)
    while O.stats().n_full_runs < 2 and done < 400:
        S.run(40)
        O.run(40)
        done += 40
        n_real, n_con = _assert_bitwise(S, O)
    print("1M drum: %d contacts, %d real, %d full runs, bitwise over %d steps" % (n_con, n_real, O.stats().n_full_runs, done))
    assert n_real > 1_000_000 and O.stats().n_full_runs >= 2
    A = _plan.compile_scene(S)
    facet_or_wall = A.particles["shape"][S._sim.contacts()["id_lo"]] != 0
    assert np.count_nonzero(facet_or_wall & (S._sim.contacts()["real"] != 0)) > 1000
    O.close()
    S.close()


def test_drum_1m_fp32_force_error(drum_1m):
    S64, S32 = _drum(drum_1m, "fp64"), _drum(drum_1m, "fp32")
    # 50 steps of FP64 first, so that the contacts carry history (trsf, uN of earlier steps)
    S64.run(50)
    st = _state(S64)
    for S, prec in ((S64, "fp64"), (S32, "fp32")):
        _restore(S, st)
        S.gpu.precision = prec
        S.run(1)
    rc, rp, n_real = _one_step_errors(S64, S32, _plan.compile_scene(S64))
    print("1M drum, one step: %d real contacts; contact force rel err max %.2e p99 %.2e; net force rel err max %.2e" %
          (n_real, rc.max(), np.percentile(rc, 99), rp.max()))
    assert n_real > 1_000_000
    assert rc.max() <= 1e-5 and rp.max() <= 1e-5
    S64.close()
    S32.close()


# ------------------------------------------------------------------------------ 200k periodic shear
@pytest.fixture(scope="module")
def shear_200k(gpu_lib):
    """200 000 spheres (r uniform in [2, 4] mm, E 5e7, tanPhi 0.4) inserted at solid fraction 0.35
    in a periodic cube and compressed isotropically to 0.62 in 30 000 FP32 steps (a packing that
    keeps its contacts); then the shear gradient (xz 1/s) is set. Returns the state."""
    S = scenes.periodic_shear(n=200_000, seed=0, fill_fraction=0.35, shear_rate=1.0, precision="fp32", compress_steps=30000,
                              compress_to=0.62)
    return _state(S)


def _shear(st, prec):
    S = scenes.periodic_shear(n=200_000, seed=0, fill_fraction=0.35, shear_rate=1.0, precision=prec, centers=st["pos"])
    [e for e in S.engines if isinstance(e, ContactLoop)][0].evalStress = True
    _restore(S, st)
    return S


def test_shear_200k_fp64_bitwise(shear_200k):
    S = _shear(shear_200k, "fp64")
    O = _oracle(_plan.compile_scene(S))
    for k in (1, 19, 40):
        S.run(k)
        O.run(k)
        n_real, n_con = _assert_bitwise(S, O)
        hs, tr, gv = O.cell()
        assert np.array_equal(np.asarray(S.cell.hSize), hs) and np.array_equal(np.asarray(S.cell.trsf), tr)
        sg = np.array([e for e in S.engines if isinstance(e, ContactLoop)][0].stress)
        so = np.array(O.stats().stress).reshape(3, 3)
        assert np.linalg.norm(sg - so) <= 1e-12 * np.linalg.norm(so)
    shifted = np.any(S._sim.contacts()["cell_dist"] != 0, axis=1) & (S._sim.contacts()["real"] != 0)
    print("200k shear: %d contacts, %d real (%d across the cell boundary), bitwise over 60 steps" %
          (n_con, n_real, int(shifted.sum())))
    assert n_real > 300_000 and shifted.sum() > 1000
    O.close()
    S.close()


def test_shear_200k_fp32_errors(shear_200k):
    S64, S32 = _shear(shear_200k, "fp64"), _shear(shear_200k, "fp32")
    S64.run(50)
    st = _state(S64)
    for S, prec in ((S64, "fp64"), (S32, "fp32")):
        _restore(S, st)
        S.gpu.precision = prec
        S.run(1)
    A = _plan.compile_scene(S64)
    rc, rp, n_real = _one_step_errors(S64, S32, A)
    s64 = np.array([e for e in S64.engines if isinstance(e, ContactLoop)][0].stress)
    s32 = np.array([e for e in S32.engines if isinstance(e, ContactLoop)][0].stress)
    srel = np.linalg.norm(s32 - s64) / np.linalg.norm(s64)
    z64 = 2.0 * S64._sim.stats().n_real / 200_000
    z32 = 2.0 * S32._sim.stats().n_real / 200_000
    print("200k shear, one step: contact force rel err max %.2e p99 %.2e; net force %.2e; stress %.2e; Z %.4f vs %.4f" %
          (rc.max(), np.percentile(rc, 99), rp.max(), srel, z32, z64))
    assert n_real > 300_000
    assert rc.max() <= 1e-5 and rp.max() <= 1e-5 and srel <= 1e-5 and z32 == z64
    S64.close()
    S32.close()


# ------------------------------------------------------------------------------ 10k box settle
def test_box_settle_10k_full_run_bitwise(gpu_lib):
    """The whole box-settle configuration: 10 000 spheres, 20 000 steps, FP64, bitwise, checked
    every 5 000 steps."""
    S = scenes.box_settle(n=10000, seed=0)
    O = _oracle(_plan.compile_scene(S))
    for _ in range(4):
        S.run(5000)
        O.run(5000)
        n_real, n_con = _assert_bitwise(S, O)
    print("10k box: %d contacts, %d real after 20 000 steps, %d full runs" % (n_con, n_real, O.stats().n_full_runs))
    assert n_real > 20_000
    O.close()
    S.close()
