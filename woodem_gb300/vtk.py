"""VTK export of a scene's state (VtkExport, pkg/dem/VtkExport.cpp:123-620).

``export(S, contacts, ...)`` writes, for Scene S at its current state, the reference's three
files as VTK XML (ASCII data):

* ``{out}spheres.{step}.vtu`` — one vertex per sphere (periodic cells: wrapped into the cell,
  Cell::canonicalizePt) with
  point data radius, mass, id, mask, color, vel, angVel, matId and cell data sigN, sigT (the
  contact forces over the contact area, DemFuncs::particleStress, pkg/dem/Funcs.cpp:227-240);
* ``{out}mesh.{step}.vtu`` — triangles of facets (closed flat edges when halfThick > 0) and walls
  (the rectangle Wall.glAB; a wall without it raises with infError, else is skipped) with cell
  data color, matState, matId, vel, angVel, |sigma|;
* ``{out}con.{step}.vtp`` — one line per real contact between the particles' positions (the
  contact point for a non-sphere end) with cell data Fn and |Ft|; a contact crossing a periodic
  boundary is drawn twice, from each end's displayed position to the image of the other end.

``contacts`` is a contact listing (``Simulation.contacts()`` of the device simulation, or the
oracle's listing of the same layout). The ``VtkExport`` engine (woodem_gb300.dem) calls this
between queued steps when it is due.
"""
import math
import os

import numpy as np

WHAT_SPHERES, WHAT_MESH, WHAT_CON, WHAT_TRI = 1, 2, 4, 8
WHAT_ALL = WHAT_SPHERES | WHAT_MESH | WHAT_CON | WHAT_TRI


def _fmt(a):
    a = np.asarray(a, dtype=float).ravel()
    return " ".join(repr(float(x)) for x in a)


def _ifmt(a):
    return " ".join(str(int(x)) for x in np.asarray(a).ravel())


def _array(name, data, ncomp, kind="Float64"):
    body = _ifmt(data) if kind.startswith(("Int", "UInt")) else _fmt(data)
    return '<DataArray type="%s" Name="%s" NumberOfComponents="%d" format="ascii">%s</DataArray>\n' % (kind, name, ncomp, body)


def _write_ugrid(path, points, cells, cell_type, point_data, cell_data, nan_value):
    """Unstructured grid: ``cells`` a list of point-index tuples of one VTK cell type."""
    pts = np.asarray(points, dtype=float).reshape(-1, 3)
    conn = [i for c in cells for i in c]
    offs = np.cumsum([len(c) for c in cells]) if cells else np.zeros(0)
    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian">\n<UnstructuredGrid>\n')
        f.write('<Piece NumberOfPoints="%d" NumberOfCells="%d">\n' % (len(pts), len(cells)))
        f.write("<PointData>\n")
        for name, (data, nc, kind) in point_data.items():
            f.write(_array(name, np.nan_to_num(np.asarray(data, float), nan=nan_value) if kind == "Float64" else data, nc, kind))
        f.write("</PointData>\n<CellData>\n")
        for name, (data, nc, kind) in cell_data.items():
            f.write(_array(name, np.nan_to_num(np.asarray(data, float), nan=nan_value) if kind == "Float64" else data, nc, kind))
        f.write("</CellData>\n<Points>\n")
        f.write(_array("Points", np.nan_to_num(pts, nan=nan_value), 3))
        f.write("</Points>\n<Cells>\n")
        f.write(_array("connectivity", conn, 1, "Int64"))
        f.write(_array("offsets", offs, 1, "Int64"))
        f.write(_array("types", [cell_type] * len(cells), 1, "UInt8"))
        f.write("</Cells>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n")


def _write_lines(path, points, lines, cell_data, nan_value):
    pts = np.asarray(points, dtype=float).reshape(-1, 3)
    conn = [i for l in lines for i in l]
    offs = [2 * (k + 1) for k in range(len(lines))]
    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian">\n<PolyData>\n')
        f.write('<Piece NumberOfPoints="%d" NumberOfVerts="0" NumberOfLines="%d" NumberOfStrips="0" NumberOfPolys="0">\n'
                % (len(pts), len(lines)))
        f.write("<CellData>\n")
        for name, data in cell_data.items():
            f.write(_array(name, np.nan_to_num(np.asarray(data, float), nan=nan_value), 1))
        f.write("</CellData>\n<Points>\n")
        f.write(_array("Points", np.nan_to_num(pts, nan=nan_value), 3))
        f.write("</Points>\n<Lines>\n")
        f.write(_array("connectivity", conn, 1, "Int64"))
        f.write(_array("offsets", offs, 1, "Int64"))
        f.write("</Lines>\n</Piece>\n</PolyData>\n</VTKFile>\n")


def _qrot(q, v):
    """Rotate v by the unit quaternion q = (w, x, y, z)."""
    w, x, y, z = q
    u = np.array([x, y, z])
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def export(S, contacts, out="", what=WHAT_ALL, mask=0, sphereSphereOnly=False, infError=True, nanValue=0.0,
           step=None):
    """Write the files of one export of scene S (host containers current); returns {kind: path}.
    Shapes carry no colour here: the colour arrays are 0."""
    if what > WHAT_ALL or what < 0:
        raise ValueError("VtkExport.what=%d, but should be at most %d." % (what, WHAT_ALL))
    step = int(S.step if step is None else step)
    out = S.expandTags(out)
    d = os.path.dirname(out)
    if d:
        os.makedirs(d, exist_ok=True)
    ps, ns = S.dem.par.soa, S.dem._nodes.soa
    shape = np.asarray(ps.col("shape"))
    pnodes = np.asarray(ps.col("nodes"))
    radius, pmask, pmat = np.asarray(ps.col("radius")), np.asarray(ps.col("mask")), np.asarray(ps.col("mat"))
    npos, nvel, nang = np.asarray(ns.col("pos")), np.asarray(ns.col("vel")), np.asarray(ns.col("angVel"))
    n = len(shape)
    is_sphere = shape == 0
    node0 = np.maximum(pnodes[:, 0], 0)
    xsp = npos[node0]  # spatial position of each particle's first node
    pos = xsp.copy()
    cds = np.zeros((n, 3), int)
    H = np.asarray(S.cell.hSize, float) if S.isPeriodic else None
    if S.isPeriodic:
        frac = np.linalg.solve(H, xsp.T).T
        cds = np.floor(frac).astype(int)
        pos = xsp - cds @ H.T
    c = contacts
    real = np.asarray(c["real"]) != 0
    lo, hi = np.asarray(c["id_lo"]), np.asarray(c["id_hi"])
    ida = np.asarray(c["id_a"])
    trsf = np.asarray(c["trsf"], float).reshape(-1, 3, 3)
    loc = np.asarray(c["local"], float).reshape(-1, 3)
    cpt = np.asarray(c["cpt"], float).reshape(-1, 3)
    cdist = np.asarray(c["cell_dist"]).reshape(-1, 3)
    selm = (pmask & mask) != 0 if mask else np.ones(n, bool)
    files = {}
    if what & WHAT_SPHERES:
        # DemFuncs::particleStress: per real contact, (1/contA)*ori*(Fn,0,0) and (1/contA)*ori*(0,Ft1,Ft2)
        # to each of its particles; contA = pi*min(r1,r2)^2 (the sphere's radius against a wall or facet)
        k = np.nonzero(real)[0]
        ra = np.where(is_sphere[lo[k]], radius[lo[k]], -1.0)
        rb = np.where(is_sphere[hi[k]], radius[hi[k]], -1.0)
        rr = np.where((ra > 0) & (rb > 0), np.minimum(ra, rb), np.where(ra > 0, ra, rb))
        contA = math.pi * rr * rr
        fn = trsf[k][:, :, 0] * loc[k, 0:1]
        ft = trsf[k][:, :, 1] * loc[k, 1:2] + trsf[k][:, :, 2] * loc[k, 2:3]
        sigN = np.zeros((n, 3))
        sigT = np.zeros((n, 3))
        for ends in (lo[k], hi[k]):
            np.add.at(sigN, ends, fn / contA[:, None])
            np.add.at(sigT, ends, ft / contA[:, None])
        sel = np.nonzero(is_sphere & selm)[0]
        pdata = {
            "radius": (radius[sel], 1, "Float64"),
            "mass": (np.asarray(ns.col("mass"))[node0[sel]], 1, "Float64"),
            "id": (sel, 1, "Int32"),
            "mask": (pmask[sel], 1, "Int32"),
            "color": (np.zeros(len(sel)), 1, "Float64"),
            "vel": (nvel[node0[sel]], 3, "Float64"),
            "angVel": (nang[node0[sel]], 3, "Float64"),
            "matId": (pmat[sel], 1, "Int32"),
        }
        cdata = {"sigT": (sigT[sel], 3, "Float64"), "sigN": (sigN[sel], 3, "Float64")}
        path = "%sspheres.%d.vtu" % (out, step)
        _write_ugrid(path, pos[sel], [(q,) for q in range(len(sel))], 1, pdata, cdata, nanValue)
        files["spheres"] = path
    if what & WHAT_MESH:
        pts, tris, cd = [], [], {"matId": [], "vel": [], "angVel": []}

        def add(vertices, conn, i):
            base = len(pts)
            pts.extend(vertices)
            for t in conn:
                tris.append(tuple(base + q for q in t))
                cd["matId"].append(pmat[i])
                cd["vel"].append(nvel[node0[i]])
                cd["angVel"].append(nang[node0[i]])
        ori = np.asarray(ns.col("ori"))
        for i in np.nonzero((shape != 0) & selm)[0]:
            if shape[i] == 2:  # facet
                A, B, C = npos[pnodes[i, 0]], npos[pnodes[i, 1]], npos[pnodes[i, 2]]
                ht = float(np.asarray(ps.col("halfThick"))[i])
                if ht == 0:
                    add([A, B, C], [(0, 1, 2)], i)
                else:
                    nrm = np.cross(B - A, C - A)
                    dz = nrm / np.linalg.norm(nrm) * ht
                    add([A + dz, B + dz, C + dz, A - dz, B - dz, C - dz],
                        [(0, 1, 2), (3, 4, 5), (0, 1, 3), (3, 1, 4), (1, 2, 4), (4, 2, 5), (2, 0, 5), (5, 0, 3)], i)
            elif shape[i] == 1:  # wall: the rectangle glAB in the wall's plane
                ab = S.dem.par[int(i)].shape.glAB
                if ab is None or not np.all(np.isfinite(np.asarray(ab, float))):
                    if infError:
                        raise RuntimeError("Wall #%d does not have Wall.glAB set and cannot be exported to VTK with "
                                           "VtkExport.infError=True." % i)
                    continue
                (l0, l1), (h0, h1) = np.asarray(ab, float)
                ax0 = int(np.asarray(ps.col("axis"))[i])
                ax1, ax2 = (ax0 + 1) % 3, (ax0 + 2) % 3
                corners = []
                for u, v in ((l0, l1), (l0, h1), (h0, l1), (h0, h1)):  # A, B, C, D
                    x = np.zeros(3)
                    x[ax1], x[ax2] = u, v
                    corners.append(npos[node0[i]] + _qrot(ori[node0[i]], x))
                add(corners, [(0, 1, 3), (0, 3, 2)], i)
        m = len(tris)
        path = "%smesh.%d.vtu" % (out, step)
        _write_ugrid(path, pts if pts else np.zeros((0, 3)), tris, 5, {},
                     {"color": (np.zeros(m), 1, "Float64"), "matState": (np.zeros(m), 1, "Float64"),
                      "matId": (cd["matId"], 1, "Int32"), "vel": (np.reshape(cd["vel"], (-1, 3)), 3, "Float64"),
                      "angVel": (np.reshape(cd["angVel"], (-1, 3)), 3, "Float64"), "|sigma|": (np.zeros(m), 1, "Float64")},
                     nanValue)
        files["mesh"] = path
    if what & WHAT_CON:
        pts = [q for q in pos]
        lines, fn, ft = [], [], []
        for k in np.nonzero(real)[0]:
            a = int(ida[k])
            b = int(hi[k]) if a == int(lo[k]) else int(lo[k])
            if mask and (not selm[a] or not selm[b]):
                continue
            if sphereSphereOnly and not (is_sphere[a] and is_sphere[b]):
                continue
            cd_ab = cdist[k] * (1 if a == int(lo[k]) else -1)  # pB's image is at pB + H*cd_ab
            segs = []
            if not S.isPeriodic or np.array_equal(cd_ab, cds[a] - cds[b]):
                # both ends where they are displayed; a non-sphere end is the contact point
                shift = (cds[a] @ H.T) if S.isPeriodic else 0.0
                ea = a if is_sphere[a] else (pts.append(cpt[k] - shift) or len(pts) - 1)
                eb = b if is_sphere[b] else (pts.append(cpt[k] - shift) or len(pts) - 1)
                segs.append((ea, eb))
            else:
                # across the periodic boundary: from each end's displayed position to the image
                # of the other end seen from it
                xa, xb = xsp[a], xsp[b] + cd_ab @ H.T
                for me, here, there in ((a, xa, xb), (b, xb, xa)):
                    pts.append(pos[me] + (there - here))
                    fake = len(pts) - 1
                    if is_sphere[me]:
                        start_id = me
                    else:
                        pts.append(pos[me] + (cpt[k] - here))
                        start_id = len(pts) - 1
                    segs.append((start_id, fake))
            for sgm in segs:
                lines.append(sgm)
                fn.append(loc[k, 0])
                ft.append(math.hypot(loc[k, 1], loc[k, 2]))
        path = "%scon.%d.vtp" % (out, step)
        _write_lines(path, pts if pts else np.zeros((0, 3)), lines, {"Fn": fn, "|Ft|": ft}, nanValue)
        files["con"] = path
    return files
