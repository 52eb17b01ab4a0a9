"""``woo.triangulated.cylinder`` counterpart (py/triangulated.py:10-69).

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
