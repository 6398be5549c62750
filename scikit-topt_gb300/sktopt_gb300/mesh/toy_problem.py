"""Benchmark problem set-ups (structured grids, nodal loads).

Cantilever (60x20x20 and 240x80x80 hex workloads): unit hexahedra, all DOFs
of the nodes on x = 0 clamped, a downward unit load split evenly over the
nodes of the bottom edge at x = L (x = nx, z = 0) -- or, with ``load_frac``,
on the single edge node nearest to y = load_frac * ny.  Built through the
``FEMDomain.from_nodes`` rules (sktopt/mesh/task_common.py:105-270).

Heat box (100x50x50 workload): T = 0 on the nodes of a centred patch of
``patch`` x ``patch`` elements on z = 0 and a uniform volumetric source.

``toy_base`` / ``toy_test`` / ``toy1`` / ``toy1_fine`` / ``toy2``: the
reference's own toy problems (sktopt/mesh/toy_problem.py:51-144), facets
and elements selected by their midpoints as scikit-fem does.
"""
from __future__ import annotations

import numpy as np

from .grid import (create_box_hex, create_box_hex_len, create_box_tet, elements_satisfying,
                   facets_satisfying, get_points_in_range, with_boundaries, with_subdomains)
from .task import LinearElasticity, LinearHeatConduction


def cantilever(nx, ny, nz, E=1.0, nu=0.3, load_frac=None):
    mesh = create_box_hex(nx, ny, nz)
    ijk = mesh.node_ijk
    dn = np.nonzero(ijk[0] == 0)[0]
    edge = (ijk[0] == nx) & (ijk[2] == 0)
    if load_frac is None:
        ln = np.nonzero(edge)[0]
    else:
        ln = np.nonzero(edge & (ijk[1] == int(round(load_frac * ny))))[0]
    f = np.zeros(3 * mesh.nnodes)
    f[3 * ln + 2] = -1.0 / ln.size
    tsk = LinearElasticity.from_nodes(mesh, dn, "all", ln, [f], np.arange(mesh.nelements),
                                      E, nu)
    return tsk


def heat_box(nx, ny, nz, patch=10, source=1.0, k=1.0):
    from ..fea.composer import source_vector
    mesh = create_box_hex(nx, ny, nz)
    ijk = mesh.node_ijk
    pw = min(patch, nx, ny)
    x0, y0 = (nx - pw) // 2, (ny - pw) // 2
    sel = (ijk[2] == 0) & (ijk[0] >= x0) & (ijk[0] <= x0 + pw) & \
        (ijk[1] >= y0) & (ijk[1] <= y0 + pw)
    dn = np.nonzero(sel)[0]
    return LinearHeatConduction.from_nodes(mesh, dn, source_vector(mesh, source),
                                           np.arange(mesh.nelements), k=k)


def heat_plate(nx=40, ny=40, nz=5, objective="compliance", avg_temp_weight=0.0,
               dirichlet_values=600.0, robin=True, jitter=0.0, seed=0):
    """The heat task of sktopt's tests/test_global_flow.py:53-104 on an
    nx x ny x nz grid: 8 x 8 x 1 plate (the reference meshes it at 0.2, i.e.
    40 x 40 x 5), Robin h = 4e-5, T_env = 300 on x = 0 and y = 8, T = 600 on
    the boundary facets with midpoints in [7.6, 8] x [0, 0.4] x [0, 1],
    k = 10, every element designable (design_robin_boundary=True).  With
    jitter > 0 the interior nodes move by U(-jitter h, jitter h) (seeded):
    general hexahedra with the same boundary faces."""
    from .grid import create_box_hex_jittered, get_points_in_range as rng, structured_hex
    lx, ly, lz = 8.0, 8.0, 1.0
    if jitter > 0.0:
        mesh = create_box_hex_jittered(nx, ny, nz, lx, ly, lz, jitter=jitter, seed=seed)
    else:
        mesh = structured_hex(np.linspace(0, lx, nx + 1), np.linspace(0, ly, ny + 1),
                              np.linspace(0, lz, nz + 1))
    return LinearHeatConduction.from_boundaries(
        mesh, rng((lx - lx / 20, lx), (0.0, ly / 20), (0.0, lz)), dirichlet_values,
        [rng((0.0, 0.0), (0.0, ly), (0.0, lz)), rng((0.0, lx), (ly, ly), (0.0, lz))]
        if robin else None,
        4.0e-5 if robin else None, 300.0 if robin else None, True, 10.0,
        objective=objective, avg_temp_weight=avg_temp_weight)


def heat_plate_tet(nx=40, ny=40, nz=5, objective="compliance", avg_temp_weight=0.0,
                   dirichlet_values=600.0, robin=True, jitter=0.2, seed=0):
    """The heat plate of ``heat_plate`` meshed with P1 tetrahedra: the
    nx x ny x nz grid split into 6 tetrahedra per cell, interior nodes
    jittered by U(-jitter h, jitter h) (seeded), Robin on the x = 0 and y = 8
    boundary facets, T = 600 on the boundary facets near the corner."""
    from .grid import get_points_in_range as rng
    lx, ly, lz = 8.0, 8.0, 1.0
    mesh = create_box_tet(nx, ny, nz, lx, ly, lz, jitter=jitter, seed=seed)
    return LinearHeatConduction.from_boundaries(
        mesh, rng((lx - lx / 20, lx), (0.0, ly / 20), (0.0, lz)), dirichlet_values,
        [rng((0.0, 0.0), (0.0, ly), (0.0, lz)), rng((0.0, lx), (ly, ly), (0.0, lz))]
        if robin else None,
        4.0e-5 if robin else None, 300.0 if robin else None, True, 10.0,
        objective=objective, avg_temp_weight=avg_temp_weight)


def multi_load_tet(nx=160, ny=80, nz=40, lx=2.0, ly=1.0, lz=1.0, jitter=0.2, seed=0,
                   E=1.0, nu=0.3):
    """Box meshed with jittered P1 tets, bottom face clamped, 4 point-load cases."""
    mesh = create_box_tet(nx, ny, nz, lx, ly, lz, jitter=jitter, seed=seed)
    ijk = mesh.node_ijk
    dn = np.nonzero(ijk[2] == 0)[0]
    top = np.nonzero(ijk[2] == nz)[0]
    rng = np.random.default_rng(seed + 1)
    picks = rng.choice(top, size=2, replace=False)
    loads, nodes = [], []
    for node, comp, sign in ((picks[0], 0, 1.0), (picks[0], 1, 1.0), (picks[0], 2, -1.0),
                             (picks[1], 2, -1.0)):
        f = np.zeros(3 * mesh.nnodes)
        f[3 * node + comp] = sign
        loads.append(f)
        nodes.append(np.array([node]))
    return LinearElasticity.from_nodes(mesh, dn, "all", nodes, loads,
                                       np.arange(mesh.nelements), E, nu)


def batched_cantilever_specs(n=256, seed=0):
    """The batched-designs configuration: n cantilevers with nx ~ U{16..64},
    ny, nz ~ U{8..32}, volume fraction ~ U(0.2, 0.5) and the load at a
    position ~ U(0, 1) along the x = L bottom edge (snapped to the nearest
    node), all from one seeded generator.  Returns (nx, ny, nz, vf, load_frac)
    tuples."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.integers(16, 65))
        ny = int(rng.integers(8, 33))
        nz = int(rng.integers(8, 33))
        vf = float(rng.uniform(0.2, 0.5))
        lf = float(rng.uniform(0.0, 1.0))
        out.append((nx, ny, nz, vf, lf))
    return out


def toy_base(mesh_size: float, intorder: int = 2):
    """toy_problem.py:51-91: an 8 x 6 x 4 box of hexahedra of size
    `mesh_size`; all DOFs fixed on the facets with midpoints at x <= 0.03; a
    total force -100 along u^3 spread uniformly over the facets (interior ones
    included) with midpoints in x in [8 - 1.2, 8.1], y in [2.4, 3.6],
    z in [4 - 1.2, 4]; E0 = 210e3, nu = 0.3; every element in the design
    set (less those the loads and supports touch, as from_facets does)."""
    x_len, y_len, z_len, eps = 8.0, 6.0, 4.0, 1.2
    mesh = create_box_hex_len(x_len, y_len, z_len, mesh_size)
    dirichlet_facets = facets_satisfying(
        mesh, get_points_in_range((0.0, 0.03), (0.0, y_len), (0.0, z_len)))
    force_facets = facets_satisfying(
        mesh, get_points_in_range((x_len - eps, x_len + 0.1), (y_len * 2 / 5, y_len * 3 / 5),
                                  (z_len - eps, z_len)))
    design_elements = elements_satisfying(
        mesh, get_points_in_range((0.0, x_len), (0.0, y_len), (0.0, z_len)))
    return LinearElasticity.from_facets(mesh, dirichlet_facets, "all", force_facets, "u^3",
                                        -100.0, design_elements, 210e3, 0.30)


def toy_test():
    """toy_problem.py:94-95."""
    return toy_base(1.0)


def toy1():
    """toy_problem.py:98-99."""
    return toy_base(0.3)


def toy1_fine():
    """toy_problem.py:102-103."""
    return toy_base(0.2)


def toy2():
    """toy_problem.py:106-144: an 8 x 8 x 1 plate of hexahedra of size 0.3
    (27 x 27 x 4), all DOFs fixed on the boundary facets with x <= 0.05, two
    load cases along u^2 (-1 and +1) on the x = 8 boundary facets with
    y >= 8 - 0.3 and y <= 0.3, from the mesh tags; E0 = 210e3, nu = 0.3."""
    x_len, y_len, z_len, mesh_size = 8.0, 8.0, 1.0, 0.3
    mesh = create_box_hex_len(x_len, y_len, z_len, mesh_size)
    eps = mesh_size
    mesh = with_boundaries(mesh, {
        "dirichlet": get_points_in_range((0.0, 0.05), (0.0, y_len), (0.0, z_len)),
        "neumann_0": get_points_in_range((x_len, x_len), (y_len - eps, y_len), (0, z_len)),
        "neumann_1": get_points_in_range((x_len, x_len), (0, eps), (0, z_len)),
    })
    mesh = with_subdomains(mesh, {"design": np.arange(mesh.nelements)})
    return LinearElasticity.from_mesh_tags(mesh, "all", ["u^2", "u^2"], [-1.0, 1.0], 210e3,
                                           0.30)
