"""Checkpoint fingerprint on the CPU: equal for scenes built the same way, whatever their
evolving state (positions, step, cell), different for another scene (particles, materials)."""

from woodem_gb300 import scenes, checkpoint, _plan


def test_fingerprint_identifies_the_scene_not_its_state():
    a = _plan.compile_scene(scenes.box_settle_scaled(300, 0.004, seed=1))
    b = _plan.compile_scene(scenes.box_settle_scaled(300, 0.004, seed=2))  # other positions only
    c = _plan.compile_scene(scenes.box_settle_scaled(300, 0.005, seed=1))  # other radii
    assert checkpoint.fingerprint(a) == checkpoint.fingerprint(b)
    assert checkpoint.fingerprint(a) != checkpoint.fingerprint(c)
    b.config["step"] = 12345
    b.nodes["pos"] = b.nodes["pos"] + 1.0
    assert checkpoint.fingerprint(a) == checkpoint.fingerprint(b)


def test_scene_save_load_description(tmp_path):
    """Scene.save / Scene.load / saveTmp / loadTmp / deepcopy (lib/object/ObjectIO.hpp) of a scene
    that has not run: the compiled description, engines, tags and energy entries come back."""
    import numpy as np
    import woodem_gb300 as woo
    from woodem_gb300 import scenes, _plan
    from woodem_gb300.dem import DynDt
    S = scenes.hertz_drum(n=300, seed=1, diameter=0.2, length=0.08, div=17, axDiv=4, fill_fraction=0.3)
    S.engines = list(S.engines) + [DynDt(stepPeriod=7, nDone=3)]
    S.trackEnergy = True
    S.energy["grav"] = 1.5
    S.tags["title"] = "saved"
    A = _plan.compile_scene(S)
    for S2 in (woo.core.Scene.load(_saved(S, str(tmp_path / "s.bin.gz"))), woo.core.Scene.load(_saved(S, str(tmp_path / "s.bin"))),
               _tmp(S), S.deepcopy()):
        A2 = _plan.compile_scene(S2)
        for grp in ("particles", "nodes", "materials"):
            for k in getattr(A, grp):
                assert np.array_equal(getattr(A, grp)[k], getattr(A2, grp)[k]), (grp, k)
        assert A2.config.keys() == A.config.keys()
        assert S2.engines[-1].nDone == 3 and S2.energy["grav"] == 1.5 and S2.tags["title"] == "saved"
        assert S2.dem.scene is S2 and S2 is not S and "_pendingContacts" not in S2.__dict__
        # a particle added with a loaded material takes that material's index
        nm = len(S2.dem._mats)
        m2 = S2.dem.par[len(S2.dem.par) - 1].material
        S2.dem.par.add(woo.utils.sphere((0, 0, 0), radius=0.003, mat=m2))
        assert len(S2.dem._mats) == nm and S2.dem.par[len(S2.dem.par) - 1].material is m2
    import pytest
    with pytest.raises(KeyError):
        woo.core.Scene.loadTmp("nothing saved under this name")


def _saved(S, path):
    S.save(path)
    return path


def _tmp(S):
    import woodem_gb300 as woo
    S.saveTmp("t")
    return woo.core.Scene.loadTmp("t")
