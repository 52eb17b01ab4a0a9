"""Checkpoint and resume (woodem_gb300.checkpoint): a run saved at step k and resumed from the
file in a freshly built scene continues as the uninterrupted run: FP64 mode bitwise (walls with
more than 64 contacts: tree-summed forces, relative 1e-12), FP32-force mode within FP32
rounding grown over the resumed steps."""
import numpy as np
import pytest

from woodem_gb300 import scenes, checkpoint, _plan

pytestmark = pytest.mark.gpu


def _nodes(S):
    S.sync()
    nd = S.dem._nodes.soa
    return {k: nd.col(k).copy() for k in ("pos", "ori", "vel", "angVel", "force", "torque")}


def _walls(S):
    A = _plan.compile_scene(S)
    return A.particles["nodes"][A.particles["shape"] == 1, 0]


def _peri(precision):
    S = scenes.periodic_shear(n=400, seed=21, fill_fraction=0.4, shear_rate=0.0, precision=precision)
    g = -10.0 * np.eye(3)
    g[0, 2] = 20.0
    S.cell.nextGradV = g
    return S


BUILDERS = {
    "box": (lambda p: scenes.box_settle_small(n=1200, seed=5, precision=p), 300, 300),
    "drum": (lambda p: scenes.hertz_drum(n=2500, seed=2, diameter=0.3, length=0.12, div=31, axDiv=6, fill_fraction=0.3,
                                         precision=p), 250, 250),
    "periodic": (_peri, 150, 150),
}


@pytest.mark.parametrize("kind", sorted(BUILDERS))
def test_resume_fp64_bitwise(kind, tmp_path, gpu_lib):
    build, n1, n2 = BUILDERS[kind]
    path = str(tmp_path / "state.npz")
    S1 = build("fp64")
    S1.run(n1)
    checkpoint.save(S1, path)
    S1.run(n2)
    ref, step1, time1 = _nodes(S1), S1.step, S1.time
    cell1 = np.array(S1.cell.hSize) if S1.isPeriodic else None
    walls = _walls(S1)
    S1.close()
    S2 = checkpoint.load(build("fp64"), path)
    assert S2.step == n1
    S2.run(n2)
    got = _nodes(S2)
    assert S2.step == step1 and S2.time == pytest.approx(time1, rel=1e-12)
    if cell1 is not None:
        assert np.array_equal(np.array(S2.cell.hSize), cell1)
    other = np.ones(len(ref["pos"]), bool)
    other[walls] = False
    for k in ("pos", "ori", "vel", "angVel", "force", "torque"):
        assert np.array_equal(ref[k][other], got[k][other]), "%s differs after resume (max %g)" % (k, np.max(np.abs(ref[k] - got[k])))
        if len(walls):
            np.testing.assert_allclose(got[k][walls], ref[k][walls], rtol=1e-12, atol=1e-12 * max(1e-30, np.abs(ref[k][walls]).max()))
    S2.close()


def test_resume_fp32(tmp_path, gpu_lib):
    build, n1, n2 = BUILDERS["box"]
    path = str(tmp_path / "state32.npz")
    S1 = build("fp32")
    S1.run(n1)
    checkpoint.save(S1, path)
    S1.run(100)
    ref = _nodes(S1)
    n_real1 = S1._sim.stats().n_real
    S1.close()
    S2 = checkpoint.load(build("fp32"), path)
    S2.run(100)
    got = _nodes(S2)
    # the resumed first step takes the saved FP64 forces (truncated to FP32) where the
    # uninterrupted one took the compensated FP32 sums: an FP32 rounding, grown over 100 steps
    assert np.max(np.abs(got["pos"] - ref["pos"])) <= 1e-9
    assert abs(S2._sim.stats().n_real - n_real1) <= 2
    S2.close()


def test_checkpoint_of_another_scene_is_refused(tmp_path, gpu_lib):
    path = str(tmp_path / "a.npz")
    S1 = scenes.box_settle_small(n=300, seed=1)
    S1.run(10)
    checkpoint.save(S1, path)
    S1.close()
    with pytest.raises(ValueError):
        checkpoint.load(scenes.box_settle_scaled(300, 0.007, seed=1), path)


@pytest.mark.parametrize("kind", ["box", "periodic"])
def test_scene_save_load_resume(kind, tmp_path, gpu_lib):
    """Scene.save / Scene.load (the scene pickled with its contact container) resume like the
    checkpoint: FP64 bitwise."""
    import woodem_gb300 as woo
    build, n1, n2 = BUILDERS[kind]
    path = str(tmp_path / "scene.bin.gz")
    S1 = build("fp64")
    S1.run(n1)
    S1.save(path)
    S1.run(n2)
    ref, step1 = _nodes(S1), S1.step
    S1.close()
    S2 = woo.core.Scene.load(path)
    assert S2.step == n1
    S2.run(n2)
    got = _nodes(S2)
    assert S2.step == step1
    for k in ("pos", "vel", "angVel", "force", "torque"):
        assert np.array_equal(ref[k], got[k]), k
