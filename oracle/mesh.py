"""Oracle meshes, element volumes and boundary sets (TEST INFRASTRUCTURE).

Restates:
* scikit-fem 11.x ``MeshHex.init_tensor`` numbering (third party, called at
  scikit-topt/sktopt/mesh/toy_problem.py:34): nodes are numbered
  ``iy + npy*(ix + npx*iz)`` (meshgrid 'xy' flattened in Fortran order) and
  elements ``ey + (npy-1)*(ex + (npx-1)*ez)``; the eight local nodes are the
  offsets (0,0,0) (0,1,0) (1,0,0) (0,0,1) (1,1,0) (0,1,1) (1,0,1) (1,1,1).
* ``fix_hexahedron_orientation`` scikit-topt/sktopt/mesh/utils.py:18-54 and
  ``fix_tetrahedron_orientation`` utils.py:57-91.
* element volumes, composer.py:164-180 (tet) and 191-248 (hex, sum of six
  |tet| volumes in a fixed node pattern).
* ``get_elements_by_nodes`` utils.py:180-228 and the design-set rules of
  ``FEMDomain.from_nodes`` task_common.py:105-270.

Parity unpinned: scikit-fem cannot be imported here to confirm the numbering.
"""
from __future__ import annotations

import numpy as np

# local node offsets of the hexahedron, in scikit-fem's MeshHex order
HEX_OFFSETS = np.array(
    [[0, 0, 0], [0, 1, 0], [1, 0, 0], [0, 0, 1],
     [1, 1, 0], [0, 1, 1], [1, 0, 1], [1, 1, 1]], dtype=np.int64)


class GridMesh:
    """Mesh on a logical (nx, ny, nz) cell grid: hex cells or 6-tet splits."""

    def __init__(self, p, t, kind, shape, node_ijk, cell_of_elem):
        self.p = p                    # (3, n_nodes) float64
        self.t = t                    # (nloc, n_elem) int64
        self.kind = kind              # "hex" | "tet"
        self.shape = shape            # (nx, ny, nz) cells
        self.node_ijk = node_ijk      # (3, n_nodes) logical coordinates
        self.cell_of_elem = cell_of_elem  # (n_elem,) logical cell id

    @property
    def nnodes(self):
        return self.p.shape[1]

    @property
    def nelements(self):
        return self.t.shape[1]


def node_index(ix, iy, iz, npx, npy):
    return iy + npy * (ix + npx * iz)


def grid_nodes(x, y, z):
    """Node coordinates in MeshHex.init_tensor order."""
    npx, npy, npz = len(x), len(y), len(z)
    n = np.arange(npx * npy * npz, dtype=np.int64)
    iy = n % npy
    ix = (n // npy) % npx
    iz = n // (npy * npx)
    p = np.vstack([np.asarray(x, float)[ix], np.asarray(y, float)[iy],
                   np.asarray(z, float)[iz]])
    ijk = np.vstack([ix, iy, iz]).astype(np.int64)
    return p, ijk


def grid_cells(nx, ny, nz):
    """(ex, ey, ez) of every cell in element order ey + ny*(ex + nx*ez)."""
    ez, ex, ey = np.meshgrid(np.arange(nz), np.arange(nx), np.arange(ny),
                             indexing="ij")
    return ex.reshape(-1), ey.reshape(-1), ez.reshape(-1)


def fix_hexahedron_orientation(t, p):
    """utils.py:18-54: swap local nodes 1 and 3 where det(p1-p0, p3-p0, p4-p0) < 0."""
    t = np.array(t, copy=True)
    c = p[:, t]
    v1 = c[:, 1] - c[:, 0]
    v2 = c[:, 3] - c[:, 0]
    v3 = c[:, 4] - c[:, 0]
    det = np.einsum("ij,ij->j", np.cross(v1.T, v2.T).T, v3)
    neg = det < 0
    t[1, neg], t[3, neg] = t[3, neg].copy(), t[1, neg].copy()
    return t


def fix_tetrahedron_orientation(t, p):
    """utils.py:57-91: swap local nodes 1 and 2 where the signed volume < 0."""
    t = np.array(t, copy=True)
    c = p[:, t]
    v1 = c[:, 1] - c[:, 0]
    v2 = c[:, 2] - c[:, 0]
    v3 = c[:, 3] - c[:, 0]
    vol = np.einsum("ij,ij->j", np.cross(v1.T, v2.T).T, v3) / 6.0
    neg = vol < 0
    t[1, neg], t[2, neg] = t[2, neg].copy(), t[1, neg].copy()
    return t


def create_box_hex(nx, ny, nz, hx=1.0, hy=1.0, hz=1.0):
    """Structured hex box of nx*ny*nz cells (toy_problem.py:10-37 for unit boxes)."""
    x = np.arange(nx + 1) * float(hx)
    y = np.arange(ny + 1) * float(hy)
    z = np.arange(nz + 1) * float(hz)
    p, ijk = grid_nodes(x, y, z)
    ex, ey, ez = grid_cells(nx, ny, nz)
    t = np.empty((8, ex.size), dtype=np.int64)
    for a, (ox, oy, oz) in enumerate(HEX_OFFSETS):
        t[a] = node_index(ex + ox, ey + oy, ez + oz, nx + 1, ny + 1)
    t = fix_hexahedron_orientation(t, p)
    return GridMesh(p, t, "hex", (nx, ny, nz), ijk, np.arange(ex.size))


def create_box_hex_len(x_len, y_len, z_len, mesh_size):
    """toy_problem.py:10-37 (ceil of length / mesh_size cells, linspace nodes)."""
    nx = int(np.ceil(x_len / mesh_size))
    ny = int(np.ceil(y_len / mesh_size))
    nz = int(np.ceil(z_len / mesh_size))
    x = np.linspace(0, x_len, nx + 1)
    y = np.linspace(0, y_len, ny + 1)
    z = np.linspace(0, z_len, nz + 1)
    p, ijk = grid_nodes(x, y, z)
    ex, ey, ez = grid_cells(nx, ny, nz)
    t = np.empty((8, ex.size), dtype=np.int64)
    for a, (ox, oy, oz) in enumerate(HEX_OFFSETS):
        t[a] = node_index(ex + ox, ey + oy, ez + oz, nx + 1, ny + 1)
    t = fix_hexahedron_orientation(t, p)
    return GridMesh(p, t, "hex", (nx, ny, nz), ijk, np.arange(ex.size))


# Freudenthal split of the unit cube into 6 tets along the (0,0,0)-(1,1,1)
# diagonal: one tet per axis permutation; conforming across cells.
_TET_PATHS = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def create_box_tet(nx, ny, nz, lx, ly, lz, jitter=0.0, seed=0):
    """6-tet split of an nx*ny*nz grid on [0,lx]x[0,ly]x[0,lz].

    Interior node coordinates are jittered by U(-jitter*h, jitter*h) per axis
    with ``numpy.random.default_rng(seed)``; a node on a boundary plane keeps
    that coordinate, so no node leaves its face.
    """
    hx, hy, hz = lx / nx, ly / ny, lz / nz
    x = np.arange(nx + 1) * hx
    y = np.arange(ny + 1) * hy
    z = np.arange(nz + 1) * hz
    p, ijk = grid_nodes(x, y, z)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-1.0, 1.0, size=p.shape)
        h = np.array([hx, hy, hz])[:, None]
        n = np.array([nx, ny, nz])[:, None]
        interior = (ijk > 0) & (ijk < n)
        p = p + np.where(interior, d * jitter * h, 0.0)
    ex, ey, ez = grid_cells(nx, ny, nz)
    ncell = ex.size
    t = np.empty((4, 6 * ncell), dtype=np.int64)
    cell = np.repeat(np.arange(ncell), 6)
    for k, perm in enumerate(_TET_PATHS):
        off = np.zeros(3, dtype=np.int64)
        verts = [off.copy()]
        for ax in perm:
            off[ax] += 1
            verts.append(off.copy())
        for a, (ox, oy, oz) in enumerate(verts):
            t[a, k::6] = node_index(ex + ox, ey + oy, ez + oz, nx + 1, ny + 1)
    t = fix_tetrahedron_orientation(t, p)
    return GridMesh(p, t, "tet", (nx, ny, nz), ijk, cell)


def _tet_volume_abs(p0, p1, p2, p3):
    """composer.py:183-188."""
    v1 = p1 - p0
    v2 = p2 - p0
    v3 = p3 - p0
    return np.abs(np.einsum("ij,ij->j", np.cross(v1.T, v2.T).T, v3)) / 6.0


def elements_volume(mesh: GridMesh):
    """composer.py:314-322; hex: six-tet pattern of composer.py:191-248."""
    c = mesh.p[:, mesh.t]
    if mesh.kind == "tet":
        v1 = c[:, 1] - c[:, 0]
        v2 = c[:, 2] - c[:, 0]
        v3 = c[:, 3] - c[:, 0]
        vol = np.einsum("ij,ij->j", np.cross(v1.T, v2.T).T, v3) / 6.0
        if np.any(vol < -1e-12):
            raise ValueError("negative tet volume")
        return vol
    pat = [(0, 1, 3, 4), (1, 2, 3, 6), (1, 5, 6, 4),
           (3, 6, 7, 4), (1, 3, 6, 4), (1, 6, 5, 4)]
    vol = np.zeros(mesh.nelements)
    for a, b, cc, d in pat:
        vol += _tet_volume_abs(c[:, a], c[:, b], c[:, cc], c[:, d])
    return vol


def element_centers(mesh: GridMesh):
    """spacial.py:13-16: mean of the element's node coordinates."""
    return np.mean(mesh.p[:, mesh.t], axis=1)


def get_elements_by_nodes(mesh: GridMesh, nodes_list):
    """utils.py:180-228: sorted unique elements touching any of the nodes."""
    nodes = np.unique(np.concatenate([np.asarray(n).ravel() for n in nodes_list]))
    mark = np.zeros(mesh.nnodes, dtype=bool)
    mark[nodes.astype(np.int64)] = True
    hit = mark[mesh.t].any(axis=0)
    return np.nonzero(hit)[0].astype(np.int32)


def setdiff1d(a, b):
    """task_common.py:18-21 (order-preserving set difference)."""
    a = np.asarray(a)
    mask = ~np.isin(a, b)
    return np.ascontiguousarray(a[mask])
