"""Meshes on a logical cell grid: structured hexahedra or 6-tet splits.

Node and element numbering follow scikit-fem's ``MeshHex.init_tensor`` (used
by sktopt/mesh/toy_problem.py:10-37): node (ix, iy, iz) has index
``iy + (ny+1)*(ix + (nx+1)*iz)`` and cell (ex, ey, ez) index
``ey + ny*(ex + nx*ez)``; the eight local hex nodes are the offsets
(0,0,0) (0,1,0) (1,0,0) (0,0,1) (1,1,0) (0,1,1) (1,0,1) (1,1,1).  The logical
coordinates are kept so the multigrid preconditioner can coarsen the grid.
"""
from __future__ import annotations

import numpy as np

HEX_OFFSETS = np.array([[0, 0, 0], [0, 1, 0], [1, 0, 0], [0, 0, 1],
                        [1, 1, 0], [0, 1, 1], [1, 0, 1], [1, 1, 1]], dtype=np.int64)

# Freudenthal split of a cell into 6 tets, one per axis order of the path
# (0,0,0) -> (1,1,1); conforming between neighbouring cells.
TET_AXIS_ORDERS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


class GridMesh:
    """skfem-shaped mesh: ``p`` (3, n_nodes), ``t`` (nloc, n_elem).

    Meshes read from files carry no logical grid (``shape`` None): they are
    solved without the geometric multigrid.  ``boundaries`` (name -> facets,
    rows (element, local face)) and ``subdomains`` (name -> elements) hold
    the tags of a mesh file."""

    def __init__(self, p, t, kind, shape=None, node_ijk=None, cell_of_elem=None,
                 boundaries=None, subdomains=None):
        self.p = np.ascontiguousarray(p, dtype=np.float64)
        self.t = np.ascontiguousarray(t, dtype=np.int64)
        self.kind = kind
        self.shape = tuple(int(s) for s in shape) if shape is not None else None
        self.node_ijk = np.ascontiguousarray(node_ijk, dtype=np.int64) \
            if node_ijk is not None else None
        self.cell_of_elem = np.ascontiguousarray(cell_of_elem, dtype=np.int64) \
            if cell_of_elem is not None else None
        self.boundaries = dict(boundaries or {})
        self.subdomains = dict(subdomains or {})

    @property
    def has_grid(self) -> bool:
        return self.shape is not None and self.node_ijk is not None

    @property
    def nnodes(self) -> int:
        return self.p.shape[1]

    @property
    def nelements(self) -> int:
        return self.t.shape[1]

    @property
    def nvertices(self) -> int:
        return self.p.shape[1]


def _node_ijk(nx, ny, nz):
    n = np.arange((nx + 1) * (ny + 1) * (nz + 1), dtype=np.int64)
    iy = n % (ny + 1)
    ix = (n // (ny + 1)) % (nx + 1)
    iz = n // ((ny + 1) * (nx + 1))
    return np.vstack([ix, iy, iz])


def _cell_ijk(nx, ny, nz):
    c = np.arange(nx * ny * nz, dtype=np.int64)
    ey = c % ny
    ex = (c // ny) % nx
    ez = c // (ny * nx)
    return ex, ey, ez


def _nid(ix, iy, iz, nx, ny):
    return iy + (ny + 1) * (ix + (nx + 1) * iz)


def _orient_hex(t, p):
    """sktopt/mesh/utils.py:18-54: swap local nodes 1 and 3 on negative orientation."""
    c = p[:, t]
    det = np.einsum("ij,ij->j", np.cross((c[:, 1] - c[:, 0]).T, (c[:, 3] - c[:, 0]).T).T,
                    c[:, 4] - c[:, 0])
    bad = det < 0
    if np.any(bad):
        t = t.copy()
        a = t[1, bad].copy()
        t[1, bad] = t[3, bad]
        t[3, bad] = a
    return t


def _orient_tet(t, p):
    """sktopt/mesh/utils.py:57-91: swap local nodes 1 and 2 on negative volume."""
    c = p[:, t]
    vol = np.einsum("ij,ij->j", np.cross((c[:, 1] - c[:, 0]).T, (c[:, 2] - c[:, 0]).T).T,
                    c[:, 3] - c[:, 0])
    bad = vol < 0
    if np.any(bad):
        t = t.copy()
        a = t[1, bad].copy()
        t[1, bad] = t[2, bad]
        t[2, bad] = a
    return t


def structured_hex(x, y, z) -> GridMesh:
    """Hex mesh on the tensor grid of node coordinates x, y, z."""
    x, y, z = (np.asarray(v, dtype=np.float64) for v in (x, y, z))
    nx, ny, nz = len(x) - 1, len(y) - 1, len(z) - 1
    ijk = _node_ijk(nx, ny, nz)
    p = np.vstack([x[ijk[0]], y[ijk[1]], z[ijk[2]]])
    ex, ey, ez = _cell_ijk(nx, ny, nz)
    t = np.empty((8, ex.size), dtype=np.int64)
    for a, (ox, oy, oz) in enumerate(HEX_OFFSETS):
        t[a] = _nid(ex + ox, ey + oy, ez + oz, nx, ny)
    t = _orient_hex(t, p)
    return GridMesh(p, t, "hex", (nx, ny, nz), ijk, np.arange(ex.size))


def create_box_hex(nx, ny, nz, hx=1.0, hy=1.0, hz=1.0) -> GridMesh:
    return structured_hex(np.arange(nx + 1) * float(hx), np.arange(ny + 1) * float(hy),
                          np.arange(nz + 1) * float(hz))


def create_box_hex_jittered(nx, ny, nz, lx, ly, lz, jitter=0.2, seed=0) -> GridMesh:
    """Hex mesh of the nx x ny x nz grid on [0,lx]x[0,ly]x[0,lz] with every
    interior node coordinate moved by U(-jitter*h, jitter*h) per axis
    (``numpy.random.default_rng(seed)``); boundary coordinates stay on their
    faces.  The cells are general trilinear hexahedra (the boundary faces
    stay planar); the logical grid is kept for the multigrid hierarchy."""
    m = structured_hex(np.linspace(0.0, lx, nx + 1), np.linspace(0.0, ly, ny + 1),
                       np.linspace(0.0, lz, nz + 1))
    ijk = m.node_ijk
    d = np.random.default_rng(seed).uniform(-1.0, 1.0, size=m.p.shape)
    h = np.array([lx / nx, ly / ny, lz / nz])[:, None]
    inside = (ijk > 0) & (ijk < np.array([nx, ny, nz])[:, None])
    p = m.p + np.where(inside, d * jitter * h, 0.0)
    return GridMesh(p, m.t, "hex", m.shape, ijk, m.cell_of_elem)


def create_box_hex_len(x_len, y_len, z_len, mesh_size) -> GridMesh:
    """sktopt/mesh/toy_problem.py:10-37."""
    n = [int(np.ceil(v / mesh_size)) for v in (x_len, y_len, z_len)]
    return structured_hex(np.linspace(0, x_len, n[0] + 1), np.linspace(0, y_len, n[1] + 1),
                          np.linspace(0, z_len, n[2] + 1))


def create_box_tet(nx, ny, nz, lx, ly, lz, jitter=0.0, seed=0) -> GridMesh:
    """6-tet split of an nx x ny x nz grid on [0,lx]x[0,ly]x[0,lz].

    Interior node coordinates move by U(-jitter*h, jitter*h) per axis
    (``numpy.random.default_rng(seed)``); boundary coordinates stay on their
    faces.
    """
    hx, hy, hz = lx / nx, ly / ny, lz / nz
    ijk = _node_ijk(nx, ny, nz)
    p = np.vstack([ijk[0] * hx, ijk[1] * hy, ijk[2] * hz]).astype(np.float64)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-1.0, 1.0, size=p.shape)
        h = np.array([hx, hy, hz])[:, None]
        n = np.array([nx, ny, nz])[:, None]
        inside = (ijk > 0) & (ijk < n)
        p = p + np.where(inside, d * jitter * h, 0.0)
    ex, ey, ez = _cell_ijk(nx, ny, nz)
    nc = ex.size
    t = np.empty((4, 6 * nc), dtype=np.int64)
    for k, order in enumerate(TET_AXIS_ORDERS):
        off = [0, 0, 0]
        t[0, k::6] = _nid(ex, ey, ez, nx, ny)
        for a, ax in enumerate(order):
            off[ax] += 1
            t[a + 1, k::6] = _nid(ex + off[0], ey + off[1], ez + off[2], nx, ny)
    t = _orient_tet(t, p)
    return GridMesh(p, t, "tet", (nx, ny, nz), ijk, np.repeat(np.arange(nc), 6))


def elements_volume(mesh: GridMesh) -> np.ndarray:
    """sktopt/fea/composer.py:164-180 (tet) and 191-248 (hex, six |tet| volumes)."""
    c = mesh.p[:, mesh.t]

    def tet(a, b, cc, d, signed=False):
        v = np.einsum("ij,ij->j", np.cross((c[:, b] - c[:, a]).T, (c[:, cc] - c[:, a]).T).T,
                      c[:, d] - c[:, a]) / 6.0
        return v if signed else np.abs(v)

    if mesh.kind == "tet":
        v = tet(0, 1, 2, 3, signed=True)
        if np.any(v < -1e-12):
            raise ValueError("negative tet volume")
        return v
    out = np.zeros(mesh.nelements)
    for q in ((0, 1, 3, 4), (1, 2, 3, 6), (1, 5, 6, 4), (3, 6, 7, 4), (1, 3, 6, 4),
              (1, 6, 5, 4)):
        out += tet(*q)
    return out


def element_centers(mesh: GridMesh) -> np.ndarray:
    """sktopt/filters/spacial.py:13-16."""
    return np.mean(mesh.p[:, mesh.t], axis=1)


def get_elements_by_nodes(mesh: GridMesh, target_nodes) -> np.ndarray:
    """sktopt/mesh/utils.py:180-228: sorted elements touching any target node."""
    if isinstance(target_nodes, np.ndarray):
        nodes = np.unique(target_nodes)
    else:
        nodes = np.unique(np.concatenate([np.asarray(n).ravel() for n in target_nodes]))
    hit = np.zeros(mesh.nnodes, dtype=bool)
    hit[nodes.astype(np.int64)] = True
    return np.nonzero(hit[mesh.t].any(axis=0))[0].astype(np.int32)


def setdiff1d(a, b):
    """sktopt/mesh/task_common.py:18-21."""
    a = np.asarray(a)
    return np.ascontiguousarray(a[~np.isin(a, b)])


def get_points_in_range(x_rng, y_rng, z_rng):
    """sktopt/mesh/utils.py:8-15: closed-box test on points (3, n)."""
    def in_range(x):
        return ((x[0] >= x_rng[0]) & (x[0] <= x_rng[1]) & (x[1] >= y_rng[0]) &
                (x[1] <= y_rng[1]) & (x[2] >= z_rng[0]) & (x[2] <= z_rng[1]))
    return in_range


def hex_face_local_nodes(axis: int, side: int) -> list:
    """Local nodes (MeshHex order) of the hexahedron face normal to ``axis``
    at offset ``side`` (0 or 1)."""
    return [a for a in range(8) if HEX_OFFSETS[a][axis] == side]


def boundary_faces(mesh: GridMesh, predicate) -> np.ndarray:
    """Boundary faces of a structured hex grid whose midpoints satisfy
    ``predicate`` (scikit-fem ``Mesh.with_boundaries`` over boundary facets,
    the tagging of sktopt's ``from_mesh_tags`` tasks, task_heat.py:252-321).
    Rows (element, axis, side), grouped by face plane."""
    if mesh.kind != "hex":
        raise ValueError("boundary_faces needs a structured hex mesh")
    n = mesh.shape
    e = np.arange(mesh.nelements)
    cell = (((e // n[1]) % n[0]), e % n[1], e // (n[1] * n[0]))
    rows = []
    for axis in range(3):
        for side in (0, 1):
            sel = e[cell[axis] == (0 if side == 0 else n[axis] - 1)]
            loc = hex_face_local_nodes(axis, side)
            mid = mesh.p[:, mesh.t[loc][:, sel]].mean(axis=1)
            keep = sel[np.asarray(predicate(mid), dtype=bool)]
            rows.append(np.stack([keep, np.full(keep.size, axis), np.full(keep.size, side)], 1))
    return np.concatenate(rows).astype(np.int64)


def face_nodes(mesh: GridMesh, faces: np.ndarray) -> np.ndarray:
    """Sorted unique nodes of the faces (element, axis, side)."""
    if len(faces) == 0:
        return np.array([], dtype=np.int64)
    return np.unique(np.concatenate([mesh.t[hex_face_local_nodes(a, s), e]
                                     for e, a, s in faces]))


# Local faces: hexahedron face f = 2 axis + side (the face normal to ``axis``
# at offset ``side``); tetrahedron face f = the face opposite local node f.
HEX_FACES = [[a for a in range(8) if HEX_OFFSETS[a][f // 2] == f % 2] for f in range(6)]
TET_FACES = [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]]


def element_faces(kind: str) -> list:
    return HEX_FACES if kind == "hex" else TET_FACES


def facet_nodes_of(mesh: GridMesh, facets: np.ndarray) -> np.ndarray:
    """(n, k) nodes of facets given as rows (element, local face)."""
    faces = element_faces(mesh.kind)
    facets = np.asarray(facets, dtype=np.int64).reshape(-1, 2)
    if facets.shape[0] == 0:
        return np.zeros((0, len(faces[0])), dtype=np.int64)
    loc = np.asarray(faces)[facets[:, 1]]                       # (n, k)
    return mesh.t[loc, facets[:, 0][:, None]]


def boundary_facets(mesh: GridMesh, predicate=None) -> np.ndarray:
    """Boundary facets (faces of exactly one element) as rows (element, local
    face), in element order; with ``predicate`` only those whose midpoints
    satisfy it (scikit-fem ``Mesh.with_boundaries`` semantics)."""
    faces = element_faces(mesh.kind)
    ne = mesh.nelements
    keys, owner = [], []
    for f, loc in enumerate(faces):
        keys.append(np.sort(mesh.t[loc].T, axis=1))
        owner.append(np.stack([np.arange(ne), np.full(ne, f)], 1))
    keys = np.concatenate(keys)
    owner = np.concatenate(owner)
    _, inv, cnt = np.unique(keys, axis=0, return_inverse=True, return_counts=True)
    bnd = owner[cnt[inv.reshape(-1)] == 1]
    order = np.lexsort((bnd[:, 1], bnd[:, 0]))
    bnd = bnd[order]
    if predicate is not None:
        mid = mesh.p[:, facet_nodes_of(mesh, bnd)].mean(axis=2)
        bnd = bnd[np.asarray(predicate(mid), dtype=bool)]
    return bnd.astype(np.int64)


def all_facets(mesh: GridMesh):
    """Every facet once, as rows (element, local face) of its first owner in
    element order, with a flag per row: True for boundary facets (faces of
    exactly one element)."""
    faces = element_faces(mesh.kind)
    ne = mesh.nelements
    keys, owner = [], []
    for f, loc in enumerate(faces):
        keys.append(np.sort(mesh.t[loc].T, axis=1))
        owner.append(np.stack([np.arange(ne), np.full(ne, f)], 1))
    keys = np.concatenate(keys)
    owner = np.concatenate(owner)
    order = np.lexsort((owner[:, 1], owner[:, 0]))
    keys, owner = keys[order], owner[order]
    _, first, cnt = np.unique(keys, axis=0, return_index=True, return_counts=True)
    first_sorted = np.sort(first)
    uniq_cnt = cnt[np.argsort(first)]
    return owner[first_sorted].astype(np.int64), uniq_cnt == 1


def facets_satisfying(mesh: GridMesh, predicate, boundaries_only: bool = False) -> np.ndarray:
    """scikit-fem ``Mesh.facets_satisfying`` (used at toy_problem.py:66-73):
    every facet, interior facets once, whose midpoint satisfies the
    predicate, as rows (element, local face); ``boundaries_only`` keeps the
    boundary facets (``Mesh.with_boundaries``)."""
    fac, bnd = all_facets(mesh)
    if boundaries_only:
        fac = fac[bnd]
    mid = mesh.p[:, facet_nodes_of(mesh, fac)].mean(axis=2)
    return fac[np.asarray(predicate(mid), dtype=bool)]


def elements_satisfying(mesh: GridMesh, predicate) -> np.ndarray:
    """scikit-fem ``Mesh.elements_satisfying`` (toy_problem.py:76-79):
    elements whose midpoints (the mean of their nodes) satisfy it."""
    return np.nonzero(np.asarray(predicate(element_centers(mesh)), dtype=bool))[0]


def with_boundaries(mesh: GridMesh, boundaries: dict) -> GridMesh:
    """scikit-fem ``Mesh.with_boundaries`` (toy_problem.py:127): named
    boundary-facet groups from predicates on the facet midpoints (or facet
    arrays given as they are); returns a mesh with them added."""
    out = GridMesh(mesh.p, mesh.t, mesh.kind, mesh.shape, mesh.node_ijk, mesh.cell_of_elem,
                   mesh.boundaries, mesh.subdomains)
    for name, b in boundaries.items():
        out.boundaries[name] = facets_satisfying(mesh, b, boundaries_only=True) \
            if callable(b) else np.asarray(b, dtype=np.int64).reshape(-1, 2)
    return out


def with_subdomains(mesh: GridMesh, subdomains: dict) -> GridMesh:
    """scikit-fem ``Mesh.with_subdomains`` (toy_problem.py:129): named element
    sets (arrays, or predicates on the element midpoints)."""
    out = GridMesh(mesh.p, mesh.t, mesh.kind, mesh.shape, mesh.node_ijk, mesh.cell_of_elem,
                   mesh.boundaries, mesh.subdomains)
    for name, e in subdomains.items():
        out.subdomains[name] = elements_satisfying(mesh, e) if callable(e) \
            else np.asarray(e, dtype=np.int64)
    return out


def facets_to_faces(facets: np.ndarray) -> np.ndarray:
    """Hexahedron facets (element, f) as (element, axis, side) rows."""
    facets = np.asarray(facets, dtype=np.int64).reshape(-1, 2)
    return np.stack([facets[:, 0], facets[:, 1] // 2, facets[:, 1] % 2], 1)
