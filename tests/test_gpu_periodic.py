"""Periodic cell on the GPU against the oracle.

FP64: bitwise positions, velocities, forces, torques, contact sets with their cell distances and
per-contact state, and the cell itself (hSize, trsf) step after step, under a constant velocity
gradient that compresses and shears the cell (Cell.homoDeform = HomoGradV2). ContactLoop.stress is
a sum whose order differs between the two (tree on the GPU, OpenMP critical section on the CPU):
relative 1e-12.
FP32-force mode: per-step contact and particle force error <= 1e-5 (the tolerance of the FP32 mode).
"""
import numpy as np
import pytest

from woodem_gb300 import scenes, _plan
from woodem_gb300.core import Cell

from test_gpu_parity import _gpu_nodes, _compare_nodes, _compare_contacts
from test_gpu_fp32 import _clone_state, _run_mode, _force_errors
from test_oracle_pbc import pbc_scene, fast_periodic_scene, _overlap_peri

pytestmark = pytest.mark.gpu


def _oracle(S):
    from oracle.oracle import Oracle
    return Oracle(_plan.compile_scene(S), threads=4, deterministic=True)


def _shear_scene(n=1500, seed=3, precision="fp64"):
    S = scenes.periodic_shear(n=n, seed=seed, fill_fraction=0.42, shear_rate=0.0, precision=precision)
    g = -15.0 * np.eye(3)
    g[0, 2] = 30.0
    S.cell.nextGradV = g
    S.engines[2].evalStress = True
    return S


def test_periodic_compress_shear_bitwise(gpu_lib):
    S = _shear_scene()
    A = _plan.compile_scene(S)
    O = _oracle(S)
    shapes = A.particles["shape"]
    nodes_of = A.particles["nodes"][:, 0]
    crossing = 0
    for _ in range(8):
        S.run(250)
        O.run(250)
        _compare_nodes(_gpu_nodes(S), O.nodes(), shapes, nodes_of)
        cg, co = S._sim.contacts(), O.contacts()
        _compare_contacts(cg, co)
        assert np.array_equal(cg["cell_dist"], co["cell_dist"])
        crossing = max(crossing, int(np.count_nonzero(np.any(cg["cell_dist"] != 0, axis=1) & (cg["real"] != 0))))
        hs, tr, gv = O.cell()
        assert np.array_equal(S.cell.hSize, hs) and np.array_equal(S.cell.trsf, tr)
        assert S._sim.stats().n_full_runs == O.stats().n_full_runs
    assert crossing > 10  # real contacts through the periodic boundary were exercised
    sg = np.array(S._sim.stats().stress)
    so = np.array(O.stats().stress)
    assert np.abs(so).max() > 0
    np.testing.assert_allclose(sg, so, rtol=1e-12, atol=1e-12 * np.abs(so).max())


def test_periodic_fp32_force_error(gpu_lib):
    S = _shear_scene(n=2000, seed=5)
    S.run(1500)
    S.close()
    A = _plan.compile_scene(S)
    st = _clone_state(S)
    hs = S.cell.hSize.copy()
    trsf = S.cell.trsf.copy()
    out = {}
    for prec in ("fp64", "fp32"):
        S.cell.hSize = hs.copy()
        S.cell.trsf = trsf.copy()
        out[prec] = _run_mode(S, st, prec, 1)
    (c64, f64), (c32, f32) = out["fp64"], out["fp32"]
    rc, rp = _force_errors(c64, c32, f64, f32, A)
    assert len(rc) > 500
    print("periodic 1 step: contact rel err max %.2e; particle rel err max %.2e" % (rc.max(), rp.max()))
    assert rc.max() <= 1e-5 and rp.max() <= 1e-5


def test_pbc_cross_cell_contact_gpu(gpu_lib):
    """The two-sphere periodic scene of pbc.py: the same cell, nodes and contact (cell distance
    (0, 0, -10)) as the oracle after a few steps of HomoGradV2."""
    S, _ = pbc_scene(Cell.HomoGradV2, 1e-6)
    O = _oracle(S)
    S.run(5)
    O.run(5)
    A = _plan.compile_scene(S)
    _compare_nodes(_gpu_nodes(S), O.nodes(), A.particles["shape"], A.particles["nodes"][:, 0])
    cg = S._sim.contacts()
    assert tuple(cg["cell_dist"][0]) == (0, 0, -10)
    _compare_contacts(cg, O.contacts())
    hs, tr, _ = O.cell()
    assert np.array_equal(S.cell.hSize, hs)


def test_particle_larger_than_half_cell(gpu_lib):
    S, _ = pbc_scene(Cell.HomoGradV2, 1e-6)
    S.cell.setBox(0.8, 2.5, 3)  # sphere diameter 1 > 0.4
    with pytest.raises(RuntimeError, match="larger than half of the cell"):
        S.run(1)


def test_gpu_holds_the_overlap_the_periodic_sort_misses(gpu_lib):
    """The scene of test_oracle_pbc.test_periodic_insertion_sort_can_miss_an_overlap on the GPU
    (FP64): after 26 steps its pair set is the exact overlap set of its boxes -- the pair (1, 28)
    that the oracle's one-pass periodic sort leaves out included, with periods (0, 0, 1) as
    cellDist -- and otherwise the oracle's; that pair is not real, and the states are bitwise
    equal."""
    S = fast_periodic_scene()
    O = _oracle(S)
    S.run(26)
    O.run(26)
    A = _plan.compile_scene(S)
    n = A.n_particles
    mn, mx = np.empty((n, 3)), np.empty((n, 3))
    from woodem_gb300 import _native
    S._sim.H.check(S._sim.H.L.wg_get_aabbs(S._sim.H.h, _native.ptr(mn), _native.ptr(mx)), "get_aabbs")
    size = np.linalg.norm(np.asarray(S.cell.hSize, float), axis=0)
    cg, co = S._sim.contacts(), O.contacts()
    kg = list(zip(cg["id_lo"].tolist(), cg["id_hi"].tolist()))
    ko = set(zip(co["id_lo"].tolist(), co["id_hi"].tolist()))
    exact = {(a, b) for a in range(n) for b in range(a + 1, n) if _overlap_peri(mn, mx, a, b, size)[0]}
    real = {k for k, rl in zip(kg, cg["real"].tolist()) if rl}
    assert set(kg) == exact | real
    assert set(kg) - ko == {(1, 28)}
    i = kg.index((1, 28))
    assert cg["real"][i] == 0 and list(cg["cell_dist"][i]) == [0, 0, 1]
    g, o = _gpu_nodes(S), O.nodes()
    for k in ("pos", "vel", "angVel", "force", "torque"):
        assert np.array_equal(g[k], o[k]), k
    O.close()
    S.close()
