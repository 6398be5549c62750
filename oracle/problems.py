"""Oracle problem set-ups for the benchmark workloads (TEST INFRASTRUCTURE).

Cantilever (60x20x20 and 240x80x80 hex workloads): unit hex grid, all DOFs of
the nodes on x = 0 clamped, a downward unit load split evenly over the nodes
of the bottom edge at x = L (x = nx, z = 0), built as a nodal load through
``FEMDomain.from_nodes`` rules (task_common.py:105-270): elements touching
the Dirichlet or load nodes leave the design set and are held at 1
(common_density.py:740-744, 1130-1134).

Heat (100x50x50 workload): T = 0 on the nodes of a centred patch of
10x10 elements on z = 0, uniform volumetric source.
"""
from __future__ import annotations

import numpy as np

from . import mesh as M
from . import fem
from .filters import SpacialFilter


def cantilever_sets(m, load_frac=None):
    nx, ny, nz = m.shape
    ijk = m.node_ijk
    dir_nodes = np.nonzero(ijk[0] == 0)[0]
    edge = (ijk[0] == nx) & (ijk[2] == 0)
    if load_frac is None:
        load_nodes = np.nonzero(edge)[0]
    else:
        iy = int(round(load_frac * ny))
        load_nodes = np.nonzero(edge & (ijk[1] == iy))[0]
    return dir_nodes, load_nodes


def cantilever(nx, ny, nz, nu=0.3, E0=1.0, load_frac=None):
    m = M.create_box_hex(nx, ny, nz)
    dir_nodes, load_nodes = cantilever_sets(m, load_frac)
    f = np.zeros(3 * m.nnodes)
    f[3 * load_nodes + 2] = -1.0 / load_nodes.size
    pb = fem.ElasticProblem(m, dir_nodes, [f], E0=E0, nu=nu)
    dir_el = M.get_elements_by_nodes(m, [dir_nodes])
    neu_el = M.get_elements_by_nodes(m, [load_nodes])
    all_el = np.arange(m.nelements)
    design = M.setdiff1d(all_el, neu_el)          # task_common.py:211-227
    design = M.setdiff1d(design, dir_el)          # task_common.py:398-401
    fixed_one = np.concatenate([dir_el, neu_el]).astype(np.int64)
    vol = M.elements_volume(m)
    return m, pb, design, fixed_one, vol


def heat_patch_nodes(m, patch=10):
    nx, ny, nz = m.shape
    ijk = m.node_ijk
    x0 = (nx - patch) // 2
    y0 = (ny - patch) // 2
    sel = (ijk[2] == 0) & (ijk[0] >= x0) & (ijk[0] <= x0 + patch) & \
        (ijk[1] >= y0) & (ijk[1] <= y0 + patch)
    return np.nonzero(sel)[0]


def heat_box(nx, ny, nz, patch=10, source=1.0, k0=1.0):
    m = M.create_box_hex(nx, ny, nz)
    dn = heat_patch_nodes(m, min(patch, nx, ny))
    pb = fem.HeatProblem(m, dn, source=source, k0=k0)
    dir_el = M.get_elements_by_nodes(m, [dn])
    design = M.setdiff1d(np.arange(m.nelements), dir_el)
    vol = M.elements_volume(m)
    return m, pb, design, dir_el.astype(np.int64), vol


def gaussian_filter_for(m, design, radius):
    mask = np.zeros(m.nelements, dtype=bool)
    mask[design] = True
    return SpacialFilter(m, radius, mask)


def in_range(x_rng, y_rng, z_rng):
    """sktopt/mesh/utils.py:8-15 (closed box test on points (3, n))."""
    def f(x):
        return ((x[0] >= x_rng[0]) & (x[0] <= x_rng[1]) & (x[1] >= y_rng[0]) &
                (x[1] <= y_rng[1]) & (x[2] >= z_rng[0]) & (x[2] <= z_rng[1]))
    return f


def boundary_faces(m, pred):
    """Boundary faces of a structured hex box whose midpoints satisfy pred
    (scikit-fem ``Mesh.with_boundaries`` on boundary facets, as the heat task
    of tests/test_global_flow.py:84-91 tags them).  Rows (element, axis, side)."""
    from .heat_robin import hex_face_nodes
    nx, ny, nz = m.shape
    n = (nx, ny, nz)
    e = np.arange(m.nelements)
    ey = e % ny
    ex = (e // ny) % nx
    ez = e // (ny * nx)
    cell = (ex, ey, ez)
    rows = []
    for axis in range(3):
        for side in (0, 1):
            sel = e[cell[axis] == (0 if side == 0 else n[axis] - 1)]
            loc = hex_face_nodes(axis, side)
            mid = m.p[:, m.t[loc][:, sel]].mean(axis=1)
            keep = sel[pred(mid)]
            rows.append(np.stack([keep, np.full(keep.size, axis), np.full(keep.size, side)], 1))
    return np.concatenate(rows).astype(np.int64)


def face_nodes(m, faces):
    from .heat_robin import hex_face_nodes
    out = [m.t[hex_face_nodes(a, s), e] for e, a, s in faces]
    return np.unique(np.concatenate(out)) if out else np.array([], np.int64)


def box_hex_lengths(nx, ny, nz, lx, ly, lz):
    """nx x ny x nz cells on [0,lx]x[0,ly]x[0,lz] with linspace nodes
    (toy_problem.py:10-37 node placement)."""
    p, ijk = M.grid_nodes(np.linspace(0, lx, nx + 1), np.linspace(0, ly, ny + 1),
                          np.linspace(0, lz, nz + 1))
    ex, ey, ez = M.grid_cells(nx, ny, nz)
    t = np.empty((8, ex.size), dtype=np.int64)
    for a, (ox, oy, oz) in enumerate(M.HEX_OFFSETS):
        t[a] = M.node_index(ex + ox, ey + oy, ez + oz, nx + 1, ny + 1)
    t = M.fix_hexahedron_orientation(t, p)
    return M.GridMesh(p, t, "hex", (nx, ny, nz), ijk, np.arange(ex.size))


def heat_plate(nx=40, ny=40, nz=5, objective="compliance", avg_temp_weight=0.0,
               dirichlet_values=600.0, robin=True, pairing="reference"):
    """The heat task of tests/test_global_flow.py:53-104: 8 x 8 x 1 plate,
    Robin (h = 4e-5, T_env = 300) on x = 0 and y = 8, T = 600 on the boundary
    facets near the corner (7.6..8, 0..0.4), k = 10, all elements design."""
    from .heat_robin import HeatRobinProblem
    lx, ly, lz = 8.0, 8.0, 1.0
    m = box_hex_lengths(nx, ny, nz, lx, ly, lz)
    rob = [boundary_faces(m, in_range((0.0, 0.0), (0.0, ly), (0.0, lz))),
           boundary_faces(m, in_range((0.0, lx), (ly, ly), (0.0, lz)))]
    dfaces = boundary_faces(m, in_range((lx - lx / 20, lx), (0.0, ly / 20), (0.0, lz)))
    dn = face_nodes(m, dfaces)
    pb = HeatRobinProblem(m, dn, dirichlet_values, k0=10.0,
                          robin_faces=rob if robin else None,
                          robin_coefficient=4.0e-5 if robin else None,
                          robin_bc_value=300.0 if robin else None,
                          objective=objective, avg_temp_weight=avg_temp_weight,
                          pairing=pairing)
    dir_el = M.get_elements_by_nodes(m, [dn])
    design = M.setdiff1d(np.arange(m.nelements), dir_el)
    vol = M.elements_volume(m)
    return m, pb, design, dir_el.astype(np.int64), vol
