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
