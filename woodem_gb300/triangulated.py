"""``woo.triangulated`` counterparts: ``cylinder`` (py/triangulated.py:10-69) and
``quadrilateral`` (py/triangulated.py:70-83).

The reference builds the mantle through GTS (un-vendored here): rings of ``div``
points (the last one coinciding with the first and merged) at ``axDiv+1`` axial
stations, two triangles per quad. This module builds the same triangulation
directly, with facet vertices shared between neighbouring facets and the facet
normal pointing away from the axis, so that ``fakeVel = -radius*angVel*n x axis``
moves the surface in the sense of the caps' angular velocity.
"""
import math

import numpy as np

from . import utils
from .dem import Node


def cylinder(A, B, radius, div=20, axDiv=1, capA=False, capB=False, masks=None, wallCaps=False, angVel=0, fixed=True, **kw):
    A = np.asarray(A, dtype=float)
    B = np.asarray(B, dtype=float)
    cylLen = float(np.linalg.norm(B - A))
    ax = (B - A) / cylLen
    if axDiv < 0:
        circum = 2 * radius * math.pi
        axDiv = int(abs(axDiv) * cylLen / (circum / div))
    # orthonormal frame (ax, e1, e2)
    tmp = np.array([0.0, 1.0, 0.0]) if abs(ax[1]) < 0.9 else np.array([0.0, 0.0, 1.0])
    e1 = np.cross(ax, tmp)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(ax, e1)
    thetas = np.linspace(0, 2 * math.pi, num=div, endpoint=True)[:-1]  # seam point merged
    xx = np.linspace(0, cylLen, num=max(axDiv + 1, 2))
    caps = []
    if wallCaps:
        cAx = -1
        for i in (0, 1, 2):
            if abs(ax[i]) > (1 - 1e-6):
                cAx = i
        if cAx < 0:
            raise ValueError("With wallCaps=True, cylinder axis must be aligned with some global axis")
        sign = int(math.copysign(1, ax[cAx]))
        wk = {k: v for k, v in kw.items() if k in ("mat", "mask", "color", "visible")}
        if capA:
            caps.append(utils.wall(A, axis=cAx, sense=sign, **wk))
            if angVel != 0:
                w = np.zeros(3)
                w[cAx] = sign * angVel
                caps[-1].shape.nodes[0].dem.angVel = w
        if capB:
            caps.append(utils.wall(B, axis=cAx, sense=-sign, **wk))
            if angVel != 0:
                w = np.zeros(3)
                w[cAx] = sign * angVel
                caps[-1].shape.nodes[0].dem.angVel = w
    elif capA or capB:
        raise NotImplementedError("triangulated caps: use wallCaps=True")
    nodes = [[Node(pos=A + x * ax + radius * (math.cos(t) * e1 + math.sin(t) * e2)) for t in thetas] for x in xx]
    nt = len(thetas)
    fk = {k: v for k, v in kw.items() if k in ("mat", "mask", "color", "visible", "halfThick", "wire")}
    ff = []
    for i in range(len(xx) - 1):
        for j in range(nt):
            a, b = nodes[i][j], nodes[i][(j + 1) % nt]
            c, d = nodes[i + 1][j], nodes[i + 1][(j + 1) % nt]
            # vertex order giving an outward normal ((b-a) x (c-a) points away from the axis)
            for tri in ((a, c, b), (b, c, d)):
                f = utils.facet(list(tri), fixed=fixed, **fk)
                n = f.shape.getNormal()
                mid = np.mean([np.asarray(t.pos) for t in tri], axis=0)
                radial = (mid - A) - np.dot(mid - A, ax) * ax
                if np.dot(n, radial) < 0:
                    f.shape.nodes = [tri[0], tri[2], tri[1]]
                ff.append(f)
    if angVel != 0:
        for f in ff:
            f.shape.fakeVel = -radius * angVel * np.cross(f.shape.getNormal(), ax)
    if masks:
        for f in ff:
            f.mask = masks[0]
        if wallCaps:
            if capA:
                caps[0].mask = masks[1]
            if capB:
                caps[-1].mask = masks[2]
    return caps + ff


def quadrilateral(A, B, C, D, size=0, div=(0, 0), **kw):
    """Triangulated quadrilateral ABDC (a skew one when the points are not coplanar),
    py/triangulated.py:70-83: ``div`` subdivisions along AB (and CD) and along AC (and BD), or
    subdivisions of at most ``size`` (at least 2 each), 2x2 by default; two facets per cell of
    the bilinear grid A + ac*(C-A) + ab*((B + ac*(D-B)) - (A + ac*(C-A))), vertices shared. (The
    reference normalises the AB-CD direction of that grid, which gives the same points only for
    sides of unit length.) ``kw`` go to utils.facet."""
    A, B, C, D = (np.asarray(x, dtype=float) for x in (A, B, C, D))
    div = tuple(int(x) for x in div)
    if sum(div) > 0:
        if min(div) < 1:
            raise ValueError("Both components of div must be positive")
        if size > 0:
            raise ValueError("only one of *div* or *size* may be given (not both)")
    else:
        l1 = min(np.linalg.norm(A - C), np.linalg.norm(D - B))
        l2 = min(np.linalg.norm(A - B), np.linalg.norm(C - D))
        div = (int(max(2, math.ceil(l1 / size))), int(max(2, math.ceil(l2 / size)))) if size != 0 else (2, 2)
    AC, BD = C - A, D - B
    aabb, aacc = np.linspace(0, 1, div[0] + 1), np.linspace(0, 1, div[1] + 1)
    nodes = [[Node(pos=(A + ac * AC) + ab * ((B + ac * BD) - (A + ac * AC))) for ac in aacc] for ab in aabb]
    out = []
    for i in range(div[0]):
        for j in range(div[1]):
            a, b, c, d = nodes[i][j], nodes[i + 1][j], nodes[i + 1][j + 1], nodes[i][j + 1]
            out.append(utils.facet([a, b, c], **kw))
            out.append(utils.facet([a, c, d], **kw))
    return out
