"""VTK export (VtkExport, pkg/dem/VtkExport.cpp) on the CPU: the files written from a state and a
contact listing of the oracle, parsed back: sphere points and data, the particle stress of
DemFuncs::particleStress, facet and wall triangles, one line per real contact (two for a contact
across a periodic boundary, each as short as the contact), and the PeriodicEngine activation
rule the host engines use."""
import math
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from woodem_gb300 import _plan, scenes, vtk
from woodem_gb300.dem import VtkExport


def _oracle_state(S, steps):
    from oracle.oracle import Oracle
    O = Oracle(_plan.compile_scene(S), threads=4)
    O.run(steps)
    nd = S.dem._nodes.soa
    for k, v in O.nodes().items():
        nd.col(k)[:] = v
    S.step = steps
    return O.contacts()


def _arrays(path):
    root = ET.parse(path).getroot()
    piece = root[0][0]
    out = {"_piece": piece.attrib}
    for da in piece.iter("DataArray"):
        t = da.attrib["type"]
        vals = np.array((da.text or "").split(), dtype=float if t.startswith("Float") else np.int64)
        nc = int(da.attrib.get("NumberOfComponents", 1))
        out[da.attrib["Name"]] = vals.reshape(-1, nc) if nc > 1 else vals
    return out


def test_drum_export(tmp_path, oracle_lib):
    S = scenes.hertz_drum(n=800, seed=1, diameter=0.2, length=0.08, div=17, axDiv=4, fill_fraction=0.3)
    con = _oracle_state(S, 60)
    A = _plan.compile_scene(S)
    out = str(tmp_path / "d.")
    with pytest.raises(RuntimeError, match="glAB"):
        vtk.export(S, con, out=out)
    files = vtk.export(S, con, out=out, infError=False)
    sp = _arrays(files["spheres"])
    sph = np.nonzero(A.particles["shape"] == 0)[0]
    assert int(sp["_piece"]["NumberOfPoints"]) == len(sph)
    assert np.array_equal(sp["Points"], A.nodes["pos"][A.particles["nodes"][sph, 0]])
    assert np.array_equal(sp["radius"], A.particles["radius"][sph]) and np.array_equal(sp["id"], sph)
    # particleStress of one sphere, from the listing
    real = con["real"] != 0
    p = int(sph[np.argmax(np.bincount(np.concatenate([con["id_lo"][real], con["id_hi"][real]]), minlength=len(A.particles["shape"]))[sph])])
    want = np.zeros(3)
    for k in np.nonzero(real & ((con["id_lo"] == p) | (con["id_hi"] == p)))[0]:
        a, b = con["id_lo"][k], con["id_hi"][k]
        r = [A.particles["radius"][q] if A.particles["shape"][q] == 0 else -1 for q in (a, b)]
        rr = min(r) if min(r) > 0 else max(r)
        want += np.asarray(con["trsf"][k]).reshape(3, 3)[:, 0] * con["local"][k][0] / (math.pi * rr * rr)
    got = sp["sigN"][np.nonzero(sph == p)[0][0]]
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    me = _arrays(files["mesh"])
    nfac = int(np.sum(A.particles["shape"] == 2))
    assert int(me["_piece"]["NumberOfCells"]) == nfac and len(me["types"]) == nfac and np.all(me["types"] == 5)
    cn = _arrays(files["con"])
    assert int(cn["_piece"]["NumberOfLines"]) == int(real.sum()) and len(cn["Fn"]) == int(real.sum())
    # walls with glAB: two triangles each
    for q in S.dem.par:
        if type(q.shape).__name__ == "Wall":
            q.shape.glAB = ((-0.1, -0.1), (0.1, 0.1))
    me = _arrays(vtk.export(S, con, out=out, what=VtkExport.mesh)["mesh"])
    assert int(me["_piece"]["NumberOfCells"]) == nfac + 2 * int(np.sum(A.particles["shape"] == 1))


def test_periodic_contacts_drawn_short(tmp_path, oracle_lib):
    S = scenes.periodic_shear(n=500, seed=3, fill_fraction=0.4, shear_rate=0.0)
    g = -30.0 * np.eye(3)
    g[0, 2] = 40.0
    S.cell.nextGradV = g
    from oracle.oracle import Oracle
    O = Oracle(_plan.compile_scene(S), threads=4)
    O.run(400)
    nd = S.dem._nodes.soa
    for k, v in O.nodes().items():
        nd.col(k)[:] = v
    hs, tr, gv = O.cell()
    S.cell.hSize = hs
    con = O.contacts()
    real = con["real"] != 0
    assert np.any(np.abs(con["cell_dist"][real]).sum(axis=1) > 0)  # some contacts cross the boundary
    files = vtk.export(S, con, out=str(tmp_path / "p."), what=VtkExport.spheres | VtkExport.con, step=400)
    sp = _arrays(files["spheres"])
    frac = np.linalg.solve(hs, sp["Points"].T).T
    assert np.all(frac >= -1e-12) and np.all(frac < 1 + 1e-12)  # wrapped into the cell
    cn = _arrays(files["con"])
    pts = cn["Points"]
    conn = cn["connectivity"].reshape(-1, 2)
    lengths = np.linalg.norm(pts[conn[:, 0]] - pts[conn[:, 1]], axis=1)
    rmax = float(np.max(S.dem.par.soa.col("radius")))
    assert len(conn) > int(real.sum()) and np.all(lengths < 2.01 * rmax)


def test_periodic_engine_rule():
    """_isActivated follows core/Engine.cpp:169-194 (stepModulo, initRun, nDo, virtPeriod)."""
    from test_dyndt_oracle import _activation
    for kw, start in ((dict(stepPeriod=10), 0), (dict(stepPeriod=10, initRun=False), 0), (dict(stepPeriod=10), 7),
                      (dict(stepPeriod=10, stepModulo=False), 7), (dict(stepPeriod=6, nDo=3), 0),
                      (dict(stepPeriod=0, virtPeriod=7.5e-3), 0)):
        e = VtkExport(**kw)
        ran = [s for s in range(start, start + 40) if e._isActivated(s, (s - start) * 1e-3, 0.0)]
        n_done, last, prev, want = _activation(40, start, 1e-3, period=kw.get("stepPeriod", 1),
                                               modulo=kw.get("stepModulo", True), init_run=kw.get("initRun", True),
                                               n_do=kw.get("nDo", -1), virt=kw.get("virtPeriod", 0.0))
        assert ran == want and (e.nDone, e.stepLast, e.stepPrev) == (n_done, last, prev), kw
    with pytest.raises(NotImplementedError, match="host"):
        from woodem_gb300.batch import Batch
        S = scenes.box_settle_small(n=50, seed=0)
        S.engines = list(S.engines) + [VtkExport(stepPeriod=10)]
        Batch([S])
