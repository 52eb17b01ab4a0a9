"""The VtkExport engine on the GPU path: the queued steps are cut where it is due, it writes the
state of that step (equal, bit for bit, to the oracle's after as many steps), and the run itself
is unchanged by the exports."""
import numpy as np
import pytest

from woodem_gb300 import _plan, scenes
from woodem_gb300.dem import VtkExport

from test_vtk import _arrays

pytestmark = pytest.mark.gpu


def test_export_engine(tmp_path, gpu_lib):
    S = scenes.hertz_drum(n=800, seed=1, diameter=0.2, length=0.08, div=17, axDiv=4, fill_fraction=0.3)
    A = _plan.compile_scene(S)
    from oracle.oracle import Oracle
    O = Oracle(A, threads=4)
    e = VtkExport(stepPeriod=40, out=str(tmp_path / "drum."), what=VtkExport.spheres | VtkExport.con)
    S.engines = list(S.engines) + [e]
    S.run(130)
    assert e.outSteps == [0, 40, 80, 120] and len(e.outFiles["spheres"]) == 4 and e.nDone == 4
    O.run(121)  # the export of step 120 holds the state after that step
    sph = np.nonzero(A.particles["shape"] == 0)[0]
    sp = _arrays(e.outFiles["spheres"][-1])
    assert np.array_equal(sp["Points"], O.nodes()["pos"][A.particles["nodes"][sph, 0]])
    cn = _arrays(e.outFiles["con"][-1])
    assert int(cn["_piece"]["NumberOfLines"]) == int(np.count_nonzero(O.contacts()["real"]))
    O.run(9)
    S.sync()
    for k in ("pos", "vel", "angVel"):
        assert np.array_equal(S.dem._nodes.soa.col(k), O.nodes()[k])
