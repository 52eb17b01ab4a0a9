"""A woo-batch parameter table run on the GPU: every line's scene, run as part of its table's
batches, ends bitwise where the same line's scene ends when run alone, and the results
database holds one row per line with the line's title and results."""
import numpy as np
import pytest

from woodem_gb300 import batch, scenes, _plan, _table

pytestmark = pytest.mark.gpu

STUDY = """# box settles: two step counts, two precisions
n radius young! tanPhi! damping precision stopAtStep
300 3e-3 1e7 0.5 0.2 'fp64' 300
400 = 3e7 0.3 0.1 = =
350 4e-3 1e6 * 0 = 450
250 = = 0.4 = 'fp32' 300
300 3e-3 1e7 0.5 0.2 'fp32' =
"""

PERI = """n shear
300 0
400 20
"""


def _state(S):
    S.sync()
    out = {k: S.dem._nodes.soa.col(k).copy() for k in ("pos", "vel", "angVel", "force", "torque")}
    A = _plan.compile_scene(S)
    return out, A.particles["nodes"][A.particles["shape"] == 1, 0]


def _same(a, b, walls):
    other = np.ones(len(a["pos"]), bool)
    other[walls] = False
    for k in a:
        assert np.array_equal(a[k][other], b[k][other]), "%s differs (max %g)" % (k, np.max(np.abs(a[k] - b[k])))
        if len(walls):
            np.testing.assert_allclose(a[k][walls], b[k][walls], rtol=1e-12, atol=1e-12 * max(1e-30, np.abs(a[k][walls]).max()))


def test_table_lines_same_as_alone(tmp_path, gpu_lib):
    tab = tmp_path / "study.txt"
    tab.write_text(STUDY)
    db = str(tmp_path / "study.sqlite")
    pre = scenes.BoxSettle()
    plan = batch.runTable(str(tab), pre, dryRun=True)
    assert plan == [("batch", 300, [3, 4]), ("batch", 450, [5]), ("batch", 300, [6, 7])]
    done = batch.runTable(str(tab), pre, results=db)
    rows = {r["batchTableLine"]: r for r in batch.dbReadResults(db)}
    assert sorted(rows) == [3, 4, 5, 6, 7]
    for l, S in done.items():
        got, walls = _state(S)
        alone = _table.buildLine(pre, str(tab), l)
        alone.run(alone.stopAtStep)
        ref, _ = _state(alone)
        n_real = int(np.count_nonzero(alone._sim.contacts()["real"]))
        alone.close()
        _same(ref, got, walls)
        r = rows[l]
        assert r["title"] == S.tags["title"] and r["batchtable"] == str(tab)
        assert r["misc"]["step"] == S.stopAtStep == S.step and r["misc"]["nReal"] == n_real
        assert r["misc"]["Ek"] == _table.sceneResults(S, {"real": np.ones(1)})["Ek"]


def _peri_scene():
    """Builder of a periodic line: reads its parameters with readParamsFromTable."""
    import woodem_gb300 as woo
    probe = woo.Scene()
    batch.readParamsFromTable(probe, n=200, shear=0.0)
    t = probe.lab.table
    S = scenes.periodic_shear(n=int(t.n), seed=int(t.n), fill_fraction=0.4, shear_rate=0.0, precision="fp64")
    g = -10.0 * np.eye(3)
    g[0, 2] = float(t.shear)
    S.cell.nextGradV = g
    S.tags.update({k: probe.tags[k] for k in ("line", "title")})
    return S


def test_periodic_lines_run_alone(tmp_path, gpu_lib):
    tab = tmp_path / "peri.txt"
    tab.write_text(PERI)
    db = str(tmp_path / "peri.sqlite")
    assert batch.runTable(str(tab), _peri_scene, steps=150, dryRun=True) == [("single", 150, [2]), ("single", 150, [3])]
    done = batch.runTable(str(tab), _peri_scene, steps=150, results=db)
    for l, S in done.items():
        got, walls = _state(S)
        alone = _table.buildLine(_peri_scene, str(tab), l)
        alone.run(150)
        ref, _ = _state(alone)
        alone.close()
        _same(ref, got, walls)
    rows = batch.dbReadResults(db)
    assert [r["title"] for r in rows] == ["n=300,shear=0", "n=400,shear=20"]
