"""Parameter tables of woo-batch (py/batch.py) on the CPU: the table reader against the known
answers of the reference's own doctests, the parameter assignment of readParamsFromTable and
runPreprocessor, the results database, line selection and the grouping of lines into batches."""
import collections
import sqlite3

import numpy as np
import pytest

from woodem_gb300 import batch, scenes
from woodem_gb300 import _table


def _write(tmp_path, text, name="table.txt"):
    f = tmp_path / name
    f.write_text(text)
    return str(f)


# The table of the TableParamReader doctest (py/batch.py:650-657) as text, and the dict that
# doctest prints for it (py/batch.py:666-685): '...' continuation columns, bang columns in the
# synthesized title, '=' repeats, '#' comments, an empty line counted, a repeated title.
DOCTEST_TABLE = """head1 important2! head3 ... ... !OMP_NUM_THREADS! abcd
1 1.1 1. 1 5 1.2 1.3
a b HE AD _3 c d ### comment
# empty line
1 = = = = = g
"""
DOCTEST_DICT = {
    2: {"!OMP_NUM_THREADS": "1.2", "abcd": "1.3", "head1": "1", "head3": "1.15", "important2": "1.1",
        "title": "important2=1.1,OMP_NUM_THREADS=1.2"},
    3: {"!OMP_NUM_THREADS": "c", "abcd": "d", "head1": "a", "head3": "HEAD_3", "important2": "b",
        "title": "important2=b,OMP_NUM_THREADS=c"},
    5: {"!OMP_NUM_THREADS": "c", "abcd": "g", "head1": "1", "head3": "HEAD_3", "important2": "b",
        "title": "important2=b,OMP_NUM_THREADS=c__line=5__"},
}


def test_reader_doctest(tmp_path):
    assert batch.TableParamReader(_write(tmp_path, DOCTEST_TABLE)).paramDict() == DOCTEST_DICT


def test_cartesian_product_doctest(tmp_path):
    """cartProdParamTable doctest (py/batch.py:838-903): 12 lines, continuation columns joined,
    '*woo.unit' and brackets dropped from the titles, repeated cells written as '='."""
    pp = collections.OrderedDict()
    pp["pattern"] = ["ortho", "hexa"]
    pp["radius", "..."] = [(r, '*woo.unit["mm"]') for r in (1, 2, 3)]
    pp["gravity", "...", "..."] = [("(0,0,", g, ")") for g in (9.81, 20)]
    out = str(tmp_path / "prod.txt")
    assert batch.cartProdParamTable(params=pp, out=out) == 12
    d = batch.TableParamReader(out).paramDict()
    assert sorted(d) == list(range(2, 14))
    k = 2
    for pat in ("ortho", "hexa"):
        for r in (1, 2, 3):
            for g in ("9.81", "20"):
                assert d[k] == {"pattern": pat, "radius": '%d*woo.unit["mm"]' % r, "gravity": "(0,0,%s)" % g,
                                "title": "pattern=%s,radius=%dmm,gravity=(0,0,%s)" % (pat, r, g)}
                k += 1
    lines = open(out).read().split("\n")
    assert lines[2].split() == ["=", "=", "=", "=", "20", "="]


def test_reader_title_column_and_first_line(tmp_path):
    f = _write(tmp_path, "\n\na title\n1 one\n= two\n")
    d = batch.TableParamReader(f).paramDict()
    assert d == {4: {"a": "1", "title": "one"}, 5: {"a": "1", "title": "two"}}
    d = batch.TableParamReader(f, firstLine=1).paramDict()
    assert sorted(d) == [5, 6]


def test_reader_no_bangs_uses_all_columns(tmp_path):
    d = batch.TableParamReader(_write(tmp_path, "a b c\n1 - *\n2 x y extra\n")).paramDict()
    assert d[2]["title"] == "a=1" and d[3]["title"] == "a=2,b=x,c=y"
    assert "extra" not in d[3].values()


@pytest.mark.parametrize("text,msg", [
    ("a b\n= 1\n", "nonexistent value"),
    ("... b\n1 2\n", "continuation"),
    ("a b c\n1 2\n", "columns"),
    ("# only a comment\n\n", "no column titles"),
])
def test_reader_errors(tmp_path, text, msg):
    with pytest.raises(ValueError, match=msg):
        batch.TableParamReader(_write(tmp_path, text))


def test_reader_spreadsheet_refused(tmp_path):
    with pytest.raises(NotImplementedError, match="xlrd"):
        batch.TableParamReader(str(tmp_path / "t.xls"))


def test_line_lists():
    av = {2: 0, 3: 0, 4: 0, 5: 0, 8: 0, 11: 0, 12: 0}
    assert _table.parseLineList("2,3-5,8,11-13", av) == [2, 3, 4, 5, 8, 11, 12]
    assert _table.parseLineList(None, av) == [2, 3, 4, 5, 8, 11, 12]
    assert _table.parseLineList("8,2,8", av) == [8, 2]
    with pytest.raises(ValueError):
        _table.parseLineList("7", av)


class _Batch:
    def __init__(self, table, line):
        self.saved = (batch.options.batchTable, batch.options.batchLine)
        batch.options.batchTable, batch.options.batchLine = table, line

    def __enter__(self):
        return self

    def __exit__(self, *a):
        batch.options.batchTable, batch.options.batchLine = self.saved


def test_read_params_from_table(tmp_path):
    """py/batch.py:512-580: table values evaluated, '*' keeps the default, '-' skips the column,
    '!' columns ignored, tags and the explicit/default lists set."""
    import woodem_gb300 as woo
    f = _write(tmp_path, "radius young! tanPhi damping !THREADS\n2e-3*2 1e7 * - 4\nsqrt(4) = 0.3 0.1 4\n")
    S = woo.Scene()
    with _Batch(f, 2):
        batch.readParamsFromTable(S, radius=1.0, young=2.0, tanPhi=0.5, damping=0.2, extra=7)
    t = S.lab.table
    assert (t.radius, t.young, t.tanPhi, t.damping, t.extra) == (4e-3, 1e7, 0.5, 0.2, 7)
    assert S.tags["line"] == "l2" and S.tags["title"] == "young=1e7"
    assert S.tags["idt"] == S.tags["id"] + ".young=1e7" and S.tags["tid"] == "young=1e7." + S.tags["id"]
    assert t.explicitParams_ == "radius=2e-3*2,young=1e7,tanPhi=0.5"
    assert set(t.defaultParams_.split(",")) == {"tanPhi=0.5", "damping=0.2", "extra=7"}
    S2 = woo.Scene()
    with _Batch(f, 3):
        batch.readParamsFromTable(S2, under="pp", radius=1.0, young=2.0, tanPhi=0.5, damping=0.2)
    assert (S2.lab.pp.radius, S2.lab.pp.young, S2.lab.pp.tanPhi, S2.lab.pp.damping) == (2.0, 1e7, 0.3, 0.1)
    with _Batch(f, 2):
        with pytest.raises(NameError):
            batch.readParamsFromTable(woo.Scene(), radius=1.0, young=2.0, tanPhi=0.5)
        S3 = woo.Scene()
        batch.readParamsFromTable(S3, unknownOk=True, radius=1.0, young=2.0, tanPhi=0.5)
        assert S3.lab.table.radius == 4e-3
    with _Batch(f, 9):
        with pytest.raises(RuntimeError, match="line number 9"):
            batch.readParamsFromTable(woo.Scene(), radius=1.0)
    S4 = woo.Scene()
    batch.readParamsFromTable(S4, radius=1.0)  # not in a batch: defaults
    assert S4.lab.table.radius == 1.0 and S4.tags["line"] == "l!"
    with pytest.raises(EnvironmentError):
        batch.readParamsFromTable(woo.Scene(), noTableOk=False, radius=1.0)


class _Inner:
    def __init__(self):
        self.tanPhi = 0.5


class _Pre:
    def __init__(self):
        self.n, self.radius, self.mat, self.note = 10, 1.0, _Inner(), "x"
        self.checked = False

    def checkAttrTypes(self):
        self.checked = True

    def __call__(self):
        import woodem_gb300 as woo
        S = woo.Scene()
        S.tags["made"] = (self.n, self.radius, self.mat.tanPhi, self.note, self.checked)
        return S


def test_run_preprocessor(tmp_path):
    """py/batch.py:583-631: dotted names reach nested objects, '=' values are evaluated last with
    ``self`` bound, '*', '-' and '!' columns leave the preprocessor alone."""
    f = _write(tmp_path, "n radius mat.tanPhi note !EXEC\n20 =self.n*0.5 pi/10 * foo\n")
    with _Batch(f, 2):
        S = batch.runPreprocessor(_Pre())
    n, r, tp, note, checked = S.tags["made"]
    assert (n, r, note, checked) == (20, 10.0, "x", True) and abs(tp - np.pi / 10) < 1e-15
    assert S.tags["line"] == "l2" and S.tags["title"] == "n=20,radius==self.n*0.5,mat.tanPhi=pi_10,EXEC=foo"
    f2 = _write(tmp_path, "nope\n1\n", "bad.txt")
    with _Batch(f2, 2):
        with pytest.raises(AttributeError, match="nope"):
            batch.runPreprocessor(_Pre())
    S = batch.runPreprocessor(_Pre(), preFile="p.py")
    assert S.tags["line"] == "default" and S.tags["title"] == "p.py"


def test_results_database(tmp_path):
    """writeResults / dbReadResults (py/batch.py:50-164, 172-243) on SQLite: one row per call,
    the batch table and line recorded, misc and series as JSON, the format version checked."""
    import woodem_gb300 as woo
    db = str(tmp_path / "res.sqlite")
    S = woo.Scene()
    S.tags["title"] = "first"
    batch.writeResults(S, defaultDb=db, quiet=True, series={"t": np.arange(3.0)}, Ek=1.5, n=np.int64(4))
    with _Batch("tab.txt", 7):
        batch.options.batchResults = db
        S.tags["title"] = "second"
        batch.writeResults(S, quiet=True, vec=np.array([1.0, 2.0]))
        batch.options.batchResults = ""
    rows = batch.dbReadResults(db)
    assert [r["title"] for r in rows] == ["first", "second"]
    assert rows[0]["batchtable"] == "" and rows[0]["batchTableLine"] == -1
    assert rows[1]["batchtable"] == "tab.txt" and rows[1]["batchTableLine"] == 7
    assert rows[0]["misc"] == {"Ek": 1.5, "n": 4} and rows[1]["misc"] == {"vec": [1.0, 2.0]}
    assert np.array_equal(rows[0]["series"]["t"], [0.0, 1.0, 2.0])
    assert rows[0]["formatVersion"] == batch.dbFormatVersion and rows[0]["sceneId"] == S.tags["id"]
    assert rows[0]["tags"]["title"] == "first"
    assert batch.dbReadResults(db, basicTypes=True)[0]["series"] == {"t": [0.0, 1.0, 2.0]}
    conn = sqlite3.connect(db)
    with conn:
        conn.execute("update batch set formatVersion=2")
    conn.close()
    with pytest.raises(RuntimeError, match="format mismatch"):
        batch.writeResults(S, defaultDb=db, quiet=True)
    with pytest.raises(NotImplementedError, match="h5py"):
        batch.writeResults(S, defaultDb=str(tmp_path / "r.hdf5"), quiet=True)
    with pytest.raises(ValueError, match="extension"):
        batch.writeResults(S, defaultDb=str(tmp_path / "r.txt"), quiet=True)
    with pytest.raises(ValueError, match="not a sequence"):
        batch.writeResults(S, defaultDb=str(tmp_path / "r2.sqlite"), quiet=True, series={"x": 3.0})


STUDY = """# box settles of a parametric study
n radius young! tanPhi! damping precision stopAtStep
300 3e-3 1e7 0.5 0.2 'fp64' 40
400 = 3e7 0.3 0.1 = =
350 4e-3 1e6 * 0 = 60
250 = = 0.4 = 'fp32' 40
300 3e-3 1e7 0.5 0.2 'fp64' 40
"""


def test_plan_groups_lines(tmp_path):
    """Lines of one precision and one step count share a Batch, up to the particle budget; the
    step count comes from each scene's stopAtStep unless given."""
    f = _write(tmp_path, STUDY)
    plan = batch.runTable(f, scenes.BoxSettle(), dryRun=True)
    assert plan == [("batch", 40, [3, 4, 7]), ("batch", 60, [5]), ("batch", 40, [6])]
    plan = batch.runTable(f, scenes.BoxSettle(), steps=10, lines="3-5,7", dryRun=True, max_particles=800)
    assert plan == [("batch", 10, [3, 4]), ("batch", 10, [5, 7])]
    S = {l: s for l, s in [(l, _table.buildLine(scenes.BoxSettle(), f, l)) for l in (3, 7)]}
    assert S[3].tags["title"] == "young=1e7,tanPhi=0.5" and S[7].tags["title"] == "young=1e7,tanPhi=0.5__line=7__"
    assert len(S[3].dem.par) == 306 and S[3].gpu.precision == "fp64" and S[3].stopAtStep == 40
    assert not _table.inBatch()


def test_cli_dry_run(tmp_path, capsys):
    f = _write(tmp_path, STUDY)
    assert _table.main([f, "woodem_gb300.scenes:BoxSettle", "-l", "3,5", "--dry-run"]) == 0
    out = capsys.readouterr().out.split("\n")
    assert out[0] == "batch 40 steps: lines 3" and out[1] == "batch 60 steps: lines 5"
    sim = tmp_path / "sim.py"
    sim.write_text("from woodem_gb300.scenes import BoxSettle\npre = BoxSettle(n=100)\n")
    assert isinstance(_table.loadSimulation(str(sim)), scenes.BoxSettle)


def test_spread_and_json(tmp_path):
    """dbToSpread (CSV) and dbToJSON of a results database (py/batch.py:245-370)."""
    import woodem_gb300 as woo
    db = str(tmp_path / "r.sqlite")
    for k in range(3):
        S = woo.Scene()
        S.tags["title"] = "t%d" % k
        batch.writeResults(S, defaultDb=db, quiet=True, Ek=float(k), nest={"a": [k, k + 1]})
    txt = batch.dbToSpread(db)
    cols = {line.split(",")[0]: line.split(",")[1:] for line in txt.strip().splitlines()}
    assert txt.splitlines()[0].startswith("title,") and cols["title"] == ["t0", "t1", "t2"]
    assert cols["misc.Ek"] == ["0.0", "1.0", "2.0"] and cols["misc.nest.a.1"] == ["1", "2", "3"]
    assert not any(k.startswith("tags") for k in cols)
    txt = batch.dbToSpread(db, rows=True, selector=lambda r: r["title"] != "t1")
    lines = txt.strip().splitlines()
    assert len(lines) == 3 and lines[0].split(",")[0] == "title"
    with pytest.raises(NotImplementedError):
        batch.dbToSpread(db, out=str(tmp_path / "x.xls"))
    import json
    assert [r["title"] for r in json.loads(batch.dbToJSON(db))] == ["t0", "t1", "t2"]


def test_deprecated_utils_aliases(tmp_path):
    import warnings
    from woodem_gb300 import utils
    import woodem_gb300 as woo
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        assert utils.runningInBatch() is False and utils.waitIfBatch() is None
        S = woo.Scene()
        utils.readParamsFromTable(S, a=1)
        assert S.lab.table.a == 1
    assert sum(issubclass(x.category, DeprecationWarning) for x in w) == 3


def test_reference_batch_results(tmp_path):
    """py/tests/batch.py:12-40 (TestBatchResults, SQLite): misc values and a Woo object in misc,
    grouped series, read back; the CSV spreadsheet written."""
    import math
    import woodem_gb300 as woo
    misc = dict(a="a", pi=math.pi, sphere=woo.dem.Sphere(radius=2.3))
    series = dict(random=np.random.default_rng(0).random(100), ones=np.ones(10))
    series["group1/item1"] = np.ones(10)
    series["group1/item2"] = 2 * np.ones(10)
    series["group2/item1"] = 3 * np.ones(10)
    S = woo.core.Scene(fields=[woo.dem.DemField()])
    db = str(tmp_path / "res.sqlite")
    batch.writeResults(S, defaultDb=db, syncXls=False, quiet=True, series=series, **misc)
    r = batch.dbReadResults(db)[0]
    assert r["misc"]["a"] == "a" and r["misc"]["pi"] == math.pi
    assert isinstance(r["misc"]["sphere"], woo.dem.Sphere) and r["misc"]["sphere"].radius == 2.3
    assert r["series"]["ones"][2] == 1 and r["series"]["group1/item2"][0] == 2
    assert batch.dbReadResults(db, basicTypes=True)[0]["misc"]["sphere"]["__class__"] == "woo.dem.Sphere"
    batch.dbToSpread(db, str(tmp_path / "res.csv"), series=False)
    assert "misc.sphere.radius" in open(str(tmp_path / "res.csv")).read()
