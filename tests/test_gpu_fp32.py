"""FP32-force mode against the FP64 path (which is bitwise equal to the FP64 oracle).

Tolerances (relative, written here):
  * per-contact global force after one step from the same state:   1e-5 of the contact force for
    contacts above 1e-4 of the largest force, 1e-9 of the largest force below that (the overlap
    is exact to ~2^-46 of the centre distance: a growing fraction of an ever smaller overlap)
  * per-particle net force, normalised by the particle's largest contact force: 1e-5 (particles
    whose largest contact force is above 1e-6 of the largest of all, the cut used for contacts)
  * after 20 steps from the same state (errors compound through the trajectory): 1e-3
  * long runs are compared statistically (trajectories are chaotic): kinetic energy,
    coordination number and packing height within a few percent.
"""
import numpy as np
import pytest

from woodem_gb300 import scenes, _plan

pytestmark = pytest.mark.gpu


def _settled_box(n=2000, steps=16000):
    S = scenes.box_settle_small(n=n, seed=2)
    S.run(steps)
    S.close()
    return S


def _clone_state(S):
    nd = S.dem._nodes.soa
    return {k: nd.col(k).copy() for k in ("pos", "ori", "vel", "angVel", "force", "torque")}


def _restore(S, st):
    nd = S.dem._nodes.soa
    for k, v in st.items():
        nd.col(k)[:] = v
    S.step = 0


def _run_mode(S, st, prec, steps):
    S.close()
    _restore(S, st)
    S.gpu.precision = prec
    S.run(steps)
    c = S._sim.contacts()
    S.sync()
    nd = S.dem._nodes.soa
    f = nd.col("force").copy()
    S.close()
    return c, f


def _force_errors(c64, c32, f64, f32, A, same_set=True):
    k64 = c64["id_lo"].astype(np.int64) << 32 | c64["id_hi"]
    k32 = c32["id_lo"].astype(np.int64) << 32 | c32["id_hi"]
    if same_set:
        assert np.array_equal(k64, k32)
    common, i64, i32 = np.intersect1d(k64, k32, return_indices=True)
    c64 = {k: v[i64] for k, v in c64.items()}
    c32 = {k: v[i32] for k, v in c32.items()}
    real = (c64["real"] != 0) & (c32["real"] != 0)
    F64, F32 = c64["fglob"][real], c32["fglob"][real]
    mag = np.linalg.norm(F64, axis=1)
    rel_contact = np.linalg.norm(F64 - F32, axis=1) / np.maximum(mag, 1e-4 * mag.max())
    # per particle: net force error normalised by the largest contact force on the particle
    npart = A.n_particles
    fmax = np.zeros(npart)
    ids = np.concatenate([c64["id_lo"][real], c64["id_hi"][real]])
    mm = np.concatenate([mag, mag])
    np.maximum.at(fmax, ids, mm)
    sph = (A.particles["shape"] == 0) & (fmax > 1e-6 * mag.max())
    nodes = A.particles["nodes"][:, 0]
    rel_part = np.linalg.norm(f64[nodes[sph]] - f32[nodes[sph]], axis=1) / fmax[sph]
    return rel_contact, rel_part


def test_fp32_per_step_force_error_box():
    S = _settled_box()
    A = _plan.compile_scene(S)
    st = _clone_state(S)
    c64, f64 = _run_mode(S, st, "fp64", 1)
    c32, f32 = _run_mode(S, st, "fp32", 1)
    rc, rp = _force_errors(c64, c32, f64, f32, A)
    assert len(rc) > 500
    print("box 1 step: contact rel err max %.2e p99 %.2e; particle rel err max %.2e" % (rc.max(), np.percentile(rc, 99), rp.max()))
    assert rc.max() <= 1e-5 and rp.max() <= 1e-5
    c64, f64 = _run_mode(S, st, "fp64", 20)
    c32, f32 = _run_mode(S, st, "fp32", 20)
    rc, rp = _force_errors(c64, c32, f64, f32, A, same_set=False)
    print("box 20 steps: contact rel err max %.2e p99 %.2e" % (rc.max(), np.percentile(rc, 99)))
    assert rc.max() <= 1e-3


def test_fp32_per_step_force_error_drum():
    S = scenes.hertz_drum(n=6000, seed=3, diameter=0.3, length=0.12, div=41, axDiv=8, fill_fraction=0.3, settle_steps=16000)
    A = _plan.compile_scene(S)
    st = _clone_state(S)
    S.run(200)  # let contacts with facets and caps form under the configured gravity
    S.close()
    st = _clone_state(S)
    c64, f64 = _run_mode(S, st, "fp64", 1)
    c32, f32 = _run_mode(S, st, "fp32", 1)
    rc, rp = _force_errors(c64, c32, f64, f32, A)
    assert len(rc) > 500
    print("drum 1 step: contact rel err max %.2e p99 %.2e; particle rel err max %.2e" % (rc.max(), np.percentile(rc, 99), rp.max()))
    assert rc.max() <= 1e-5 and rp.max() <= 1e-5


def test_fp32_long_run_statistics():
    """Box settle run 4000 steps in both modes: kinetic energy, coordination number and mean
    sphere height agree statistically (trajectories themselves diverge)."""
    out = {}
    for prec in ("fp64", "fp32"):
        S = scenes.box_settle_small(n=2000, seed=4, precision=prec)
        S.run(4000)
        c = S._sim.contacts()
        S.sync()
        nd = S.dem._nodes.soa
        A = _plan.compile_scene(S)
        sph = A.particles["shape"] == 0
        v = nd.col("vel")[A.particles["nodes"][sph, 0]]
        m = nd.col("mass")[A.particles["nodes"][sph, 0]]
        ek = 0.5 * np.sum(m * np.sum(v * v, axis=1))
        z = np.mean(nd.col("pos")[A.particles["nodes"][sph, 0], 2])
        real = c["real"] != 0
        ss = real & (A.particles["shape"][c["id_lo"]] == 0) & (A.particles["shape"][c["id_hi"]] == 0)
        coord = 2.0 * np.count_nonzero(ss) / np.count_nonzero(sph)
        out[prec] = (ek, z, coord)
        S.close()
    e64, z64, c64 = out["fp64"]
    e32, z32, c32 = out["fp32"]
    print("fp64 Ek %.4e z %.5f Z %.3f | fp32 Ek %.4e z %.5f Z %.3f" % (e64, z64, c64, e32, z32, c32))
    assert abs(z32 - z64) <= 0.02 * z64
    assert abs(c32 - c64) <= 0.05 * max(c64, 1.0)
    assert abs(e32 - e64) <= 0.25 * max(e64, e32) + 1e-12
