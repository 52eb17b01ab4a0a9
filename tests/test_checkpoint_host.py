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
