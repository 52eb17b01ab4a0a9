"""Scene.labels / Scene.lab (core/LabelMapper.cpp), restating py/tests/labels.py for the objects
of the path (Leapfrog stands in for the reference's PyRunner)."""
import pytest

import woodem_gb300 as woo
from woodem_gb300.core import LabelMapper, Object, Scene
from woodem_gb300.dem import DemField, Leapfrog


@pytest.fixture
def S():
    return Scene(fields=[DemField()])


def test_access(S):
    S.labels["abc"] = 123
    assert S.lab.abc == 123
    assert S.labels._whereIs("abc") == LabelMapper.inPy
    S.lab.ghi = 456
    assert S.labels["ghi"] == 456


def test_del(S):
    S.labels["foo"] = 123
    assert S.lab.foo == 123
    del S.lab.foo
    assert S.labels._whereIs("foo") == LabelMapper.nowhere


def test_seq(S):
    o1, o2, o3 = Object(), Object(), Object()
    S.lab.objs = [None, o1, o2, o3]
    assert S.lab.objs[1] == o1
    assert S.labels._whereIs("objs") == LabelMapper.inWooSeq
    S.lab.objs2 = (None, o1, o2, o3)
    assert S.lab.objs2[1] == o1
    assert S.labels._whereIs("objs2") == LabelMapper.inWooSeq
    S.labels["objs3[2]"] = o2
    assert S.lab.objs3[0] is None
    assert S.lab.objs3[2] == o2
    assert len(S.lab.objs3) == 3
    assert S.labels["objs3[2]"] is o2


def test_mixed_seq(S):
    o1, o2 = Object(), Object()
    with pytest.raises(ValueError):
        setattr(S.lab, "ll", [o1, o2, 12])
    with pytest.raises(ValueError):
        setattr(S.lab, "ll", (12, 23, o1))
    S.lab.ll1 = []
    S.lab.ll2 = ()
    S.lab.ll3 = [None, None]
    S.lab.mm = [o1, None]
    setattr(S.lab, "ll4[0]", [])
    assert S.labels._whereIs("mm") == LabelMapper.inWooSeq
    S.lab.nn = [231, None]
    assert S.labels._whereIs("nn") == LabelMapper.inPy


def test_shared(S):
    S.engines = [Leapfrog()]
    S.lab.someEngine = S.engines[0]
    assert S.labels._whereIs("someEngine") == LabelMapper.inWoo
    S2 = S.deepcopy()
    assert S2.lab.someEngine is S2.engines[0]


def test_auto_label(S):
    ee = Leapfrog(label="abc")
    S.engines = [ee]
    assert S.lab.abc == ee
    assert S.labels._whereIs("abc") == LabelMapper.inWoo
    S.engines = woo.utils.defaultEngines(dynDtPeriod=0)
    S.engines[2].lawDisp[0].label = "law"
    assert S.lab.law is S.engines[2].lawDisp[0]


def test_pseudo_modules(S):
    with pytest.raises(AttributeError):
        S.lab.abc
    with pytest.raises(NameError):
        setattr(S.lab, "abc.defg", 1)
    S.lab._newModule("abc")
    assert S.lab._whereIs("abc") == LabelMapper.inMod
    S.lab.abc.a1 = 1
    with pytest.raises(AttributeError):
        S.lab.abc._newModule("a1")
    with pytest.raises(ValueError):
        S.lab._newModule("abc")
    S.lab._newModule("foo.bar")
    assert S.lab._whereIs("foo") == LabelMapper.inMod
    S.lab.foo.bar.bb = 1
    assert S.lab.foo.bar.bb == 1
    S.labels["foo.bar.baz[0]"] = 1
    with pytest.raises(ValueError):
        S.labels["abc"]
    with pytest.raises(NameError):
        S.labels["abc"] = 3


def test_writable(S, caplog):
    S.lab.if_overwriting_this_causes_warning_it_is_a_bug = 3
    S.lab._setWritable("if_overwriting_this_causes_warning_it_is_a_bug")
    with caplog.at_level("WARNING", logger="woo.core"):
        S.lab.if_overwriting_this_causes_warning_it_is_a_bug = 4
        assert not caplog.records
        S.lab.other = 1
        S.lab.other = 2
        assert len(caplog.records) == 1


def test_dir_and_hasattr(S):
    S.lab._newModule("foo")
    S.lab.foo.bar = 1
    S.lab.foo2 = 1
    assert "bar" in S.lab.foo.__dir__()
    assert hasattr(S.lab.foo, "bar") and not hasattr(S.lab.foo, "baz")
    assert {"foo", "foo2"} <= set(dir(S.lab))


def test_labels_survive_save_load(S, tmp_path):
    S.lab._newModule("table")
    S.lab.table.radius = 2e-3
    S.lab.lf = Leapfrog()
    S.engines = [S.lab.lf]
    path = str(tmp_path / "s.bin")
    S.save(path)
    S2 = Scene.load(path)
    assert S2.lab.table.radius == 2e-3 and S2.lab.lf is S2.engines[0]


def test_expand_tags(S):
    S.tags["title"] = "drum"
    assert S.expandTags("/tmp/{title}-{id}.{unknown}") == "/tmp/drum-%s.{unknown}" % S.tags["id"]
    assert S.expandTags("plain") == "plain"
