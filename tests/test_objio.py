"""Object.dump/dumps/load/loads (lib/object/ObjectIO.hpp; py/tests/io.py TestFormatsAndDetection):
engines and a particle of a defaultEngines scene through each format, the type preserved and
checked on loading, unknown formats refused."""
import math

import numpy as np
import pytest

import woodem_gb300 as woo
from woodem_gb300 import utils
from woodem_gb300.core import Object
from woodem_gb300.dem import DemField, Node


def _scene():
    S = woo.core.Scene(fields=[DemField()])
    S.engines = utils.defaultEngines()
    S.dem.par.add(utils.sphere((0, 0, 0), radius=1))
    return S


@pytest.mark.parametrize("fmt,ext", [("expr", ".expr"), ("json", ".json"), ("pickle", ".pickle"), ("auto", ".bin"),
                                     ("auto", ".bin.gz"), ("auto", ".json")])
def test_dump_load_engines(fmt, ext, tmp_path):
    S = _scene()
    for k, o in enumerate(S.engines):
        out = str(tmp_path / ("e%d%s" % (k, ext)))
        o.dump(out, format=fmt)
        o2 = Object.load(out, format="auto")
        assert type(o2) == type(o)
        o3 = type(o).load(out, format="auto")
        assert type(o3) == type(o)
        with pytest.raises(TypeError):
            Node.load(out)
    lf = S.engines[0]
    o2 = Object.loads(lf.dumps(format="json"))
    assert o2.damping == lf.damping and o2.reset == lf.reset
    cl = Object.loads(S.engines[2].dumps(format="expr"))
    assert [type(f).__name__ for f in cl.lawDisp] == [type(f).__name__ for f in S.engines[2].lawDisp]
    dyn = Object.loads(S.engines[3].dumps(format="expr"))
    assert dyn.stepPeriod == 100 and math.isnan(dyn.dt)


def test_dump_particle_and_formats(tmp_path):
    S = _scene()
    p = S.dem.par[0]
    out = str(tmp_path / "p.pickle")
    p.dump(out)
    assert type(Object.load(out)) == type(p)
    with pytest.raises(IOError):
        p.dumps(format="json")  # its nodes belong to the field: pickle only
    assert "<table>" in S.engines[0].dumps(format="html")
    with pytest.raises(IOError):
        S.engines[0].dumps(format="bogus")
    mat = Object.loads(utils.defaultMaterial().dumps(format="json"))
    assert mat.young == 1e7 and mat.tanPhi == pytest.approx(math.tan(0.5))
