"""Long runs of the FP32-force mode compared statistically with FP64 plain mode (which is bitwise
the oracle's): trajectories of many interacting spheres are chaotic, so individual positions part
after a few thousand steps, but the histories of the macroscopic quantities must agree.

* The 10 000-sphere box settle, its whole 20 000 steps from the jittered lattice: the kinetic
  energy history (sampled every 500 steps) within 3 % of its peak at every sample, and at the end
  the coordination number within 2 %, the mean sphere height within 0.5 %, the height of the bed
  top within 1 %.
* A sheared periodic packing (40 000 spheres compressed to solid fraction 0.62, then 4 000 steps
  of xz shear): the stress tensor (ContactLoop.stress) history within 5 % of its norm and the
  coordination number within 3 % at every sample.
"""
import numpy as np
import pytest

from woodem_gb300 import scenes, _plan
from woodem_gb300.dem import ContactLoop

pytestmark = pytest.mark.gpu


def _kinetic(S):
    S.sync()
    A = _plan.compile_scene(S)
    sph = A.particles["nodes"][A.particles["shape"] == 0, 0]
    nd = A.nodes
    v, w = nd["vel"][sph], nd["angVel"][sph]
    return float(0.5 * np.sum(nd["mass"][sph] * np.sum(v * v, axis=1)) + 0.5 * np.sum(nd["inertia"][sph] * w * w))


def test_box_settle_10k_histories(gpu_lib):
    out = {}
    for prec in ("fp64", "fp32"):
        S = scenes.box_settle(n=10000, seed=0, precision=prec)
        ke = []
        for _ in range(40):
            S.run(500)
            ke.append(_kinetic(S))
        z = scenes._sphere_nodes(S, "pos")[:, 2]
        out[prec] = (np.array(ke), 2.0 * S._sim.stats().n_real / 10000, float(z.mean()), float(np.percentile(z, 99.5)))
        S.close()
    k64, z64, m64, t64 = out["fp64"]
    k32, z32, m32, t32 = out["fp32"]
    print("KE peak %.4g J; max history difference %.3g of the peak; Z %.4f vs %.4f; mean z %.5f vs %.5f" %
          (k64.max(), np.max(np.abs(k32 - k64)) / k64.max(), z32, z64, m32, m64))
    assert np.max(np.abs(k32 - k64)) <= 0.03 * k64.max()
    assert abs(z32 - z64) <= 0.02 * z64 and abs(m32 - m64) <= 0.005 * m64 and abs(t32 - t64) <= 0.01 * t64


def test_periodic_shear_histories(gpu_lib):
    base = scenes.periodic_shear(n=40000, seed=1, fill_fraction=0.35, shear_rate=1.0, precision="fp32", compress_steps=20000,
                                 compress_to=0.62)
    base.sync()
    nd = base.dem._nodes.soa
    st = {k: nd.col(k).copy() for k in ("pos", "ori", "vel", "angVel", "force", "torque")}
    cell = (np.array(base.cell.hSize), np.array(base.cell.trsf), np.array(base.cell._gradV), np.array(base.cell.nextGradV))
    base.close()
    out = {}
    for prec in ("fp64", "fp32"):
        S = scenes.periodic_shear(n=40000, seed=1, fill_fraction=0.35, shear_rate=1.0, precision=prec, centers=st["pos"])
        loop = [e for e in S.engines if isinstance(e, ContactLoop)][0]
        loop.evalStress = True
        for k, v in st.items():
            S.dem._nodes.soa.col(k)[:] = v
        S.cell.hSize, S.cell.trsf, S.cell._gradV, S.cell.nextGradV = (c.copy() for c in cell)
        sig, z = [], []
        for _ in range(8):
            S.run(500)
            sig.append(np.array(loop.stress))
            z.append(2.0 * S._sim.stats().n_real / 40000)
        out[prec] = (np.array(sig), np.array(z))
        S.close()
    s64, z64 = out["fp64"]
    s32, z32 = out["fp32"]
    nrm = np.linalg.norm(s64.reshape(len(s64), 9), axis=1)
    diff = np.linalg.norm((s32 - s64).reshape(len(s64), 9), axis=1)
    print("stress history: max difference %.3g of the norm; Z %s vs %s" % (np.max(diff / nrm), z32.round(3), z64.round(3)))
    assert z64.min() > 2.0  # a loaded packing with contacts throughout
    assert np.all(diff <= 0.05 * nrm) and np.all(np.abs(z32 - z64) <= 0.03 * z64)
