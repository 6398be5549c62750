"""Oracle of boundary facets and surface traction loads (TEST INFRASTRUCTURE).

Restates:
* scikit-fem boundary facets (faces of exactly one element) with the
  midpoint tagging of ``Mesh.with_boundaries``, by brute-force counting;
* ``assemble_surface_forces`` sktopt/mesh/task_elastic.py:15-81: per facet
  group the total area A = int 1 dGamma, the traction value / A along one
  component, and F = int traction v dGamma.  Quadrature here: 3x3 Gauss on
  the bilinear map of a hexahedron face and the edge-midpoint rule on a
  triangle (both exact for these integrands; the product uses other rules).
"""
from __future__ import annotations

import numpy as np

from .mesh import HEX_OFFSETS

HEX_FACES = [[a for a in range(8) if HEX_OFFSETS[a][f // 2] == f % 2] for f in range(6)]
TET_FACES = [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]]


def faces_of(kind):
    return HEX_FACES if kind == "hex" else TET_FACES


def boundary_facets(m, pred=None):
    count = {}
    owner = {}
    for e in range(m.nelements):
        for f, loc in enumerate(faces_of(m.kind)):
            key = tuple(sorted(int(x) for x in m.t[loc, e]))
            count[key] = count.get(key, 0) + 1
            owner.setdefault(key, (e, f))
    rows = sorted(owner[k] for k, c in count.items() if c == 1)
    out = []
    for e, f in rows:
        mid = m.p[:, m.t[faces_of(m.kind)[f], e]].mean(axis=1)
        if pred is None or bool(pred(mid[:, None])[0]):
            out.append((e, f))
    return np.asarray(out, dtype=np.int64).reshape(-1, 2)


def _facet_rule(m, e, f):
    loc = faces_of(m.kind)[f]
    X = m.p[:, m.t[loc, e]]
    if m.kind == "tet":
        a = 0.5 * np.linalg.norm(np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]))
        # edge midpoints, weights 1/3: exact for quadratics
        pts = [(0.5, 0.5, 0.0), (0.0, 0.5, 0.5), (0.5, 0.0, 0.5)]
        return loc, a, sum(np.array(p) * a / 3.0 for p in pts)
    ax = [d for d in range(3) if d != f // 2]
    uv = HEX_OFFSETS[loc][:, ax]
    xg, wg = np.polynomial.legendre.leggauss(3)
    xg = 0.5 * (xg + 1.0)
    wg = 0.5 * wg
    area = 0.0
    integ = np.zeros(4)
    for s, ws in zip(xg, wg):
        for t, wt in zip(xg, wg):
            N = np.array([(s if o[0] else 1 - s) * (t if o[1] else 1 - t) for o in uv])
            dS = np.array([(1.0 if o[0] else -1.0) * (t if o[1] else 1 - t) for o in uv])
            dT = np.array([(s if o[0] else 1 - s) * (1.0 if o[1] else -1.0) for o in uv])
            jac = np.linalg.norm(np.cross(X @ dS, X @ dT))
            area += ws * wt * jac
            integ += ws * wt * jac * N
    return loc, area, integ


def surface_forces(m, facets_list, dirs, values):
    """task_elastic.py:15-81, one load vector per group."""
    out = []
    for fac, d, v in zip(facets_list, dirs, values):
        comp = int(d[2:]) - 1
        rules = [_facet_rule(m, e, f) for e, f in fac]
        A = sum(r[1] for r in rules)
        F = np.zeros(3 * m.nnodes)
        for (e, f), (loc, _, integ) in zip(fac, rules):
            for a, val in zip(loc, integ):
                F[3 * m.t[a, e] + comp] += float(v) / A * val
        out.append(F)
    return out
