"""Oracle density filters and Heaviside projection (TEST INFRASTRUCTURE).

Restates:
* ``make_kernel('gaussian')`` spacial.py:37-45 (sigma = r/3, support 3*sigma),
  ``build_filter_matrix`` spacial.py:51-103 (cKDTree ball query, design
  columns only, row normalisation), ``SpacialFilter.forward/gradient``
  spacial.py:135-166.
* ``HelmholtzFilterNodal`` helmholtz_filter_nodal.py:26-233: volume-weighted
  element->node average (non-design value 1 forward, 0 gradient), the nodal
  system (M + r^2 K) solved with the non-design nodes condensed to 1
  (forward) or as a pure Neumann problem (gradient), node->element mean, and
  the gradient's clamp to <= 0.
* ``heaviside_projection`` / derivative projection.py:27-118.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
from scipy.spatial import cKDTree

from .mesh import element_centers
from . import fem


def gaussian_filter_matrix(centers, radius, design_mask):
    """spacial.py:51-103 with the gaussian kernel of spacial.py:37-45."""
    s = radius / 3.0
    support = 3.0 * s
    n_all = centers.shape[1]
    if design_mask is None:
        design_mask = np.ones(n_all, dtype=bool)
    design_ids = np.nonzero(design_mask)[0]
    tree = cKDTree(centers.T)
    nbrs = tree.query_ball_point(centers[:, design_ids].T, support)
    rows, cols, data = [], [], []
    for row_idx, (i, js_all) in enumerate(zip(design_ids, nbrs)):
        js_all = np.asarray(js_all, dtype=int)
        js = js_all[design_mask[js_all]]
        if js.size == 0:
            continue
        dij = np.linalg.norm(centers[:, js] - centers[:, [i]], axis=0)
        w = np.exp(-0.5 * (dij / s) ** 2)
        rows.append(np.full(js.size, row_idx))
        cols.append(np.searchsorted(design_ids, js))
        data.append(w)
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    data = np.concatenate(data)
    nd = design_ids.size
    W = sp.coo_matrix((data, (rows, cols)), shape=(nd, nd)).tocsr()
    row_sum = np.array(W.sum(axis=1)).ravel()
    row_sum[row_sum == 0.0] = 1.0
    W = sp.diags(1.0 / row_sum) @ W
    W = W.tocsr()
    W.sort_indices()
    return W


class SpacialFilter:
    """spacial.py:106-166 (the matrix is rebuilt per radius, not per call)."""

    def __init__(self, mesh, radius, design_mask):
        self.centers = element_centers(mesh)
        self.design_mask = design_mask
        self.radius = None
        self.update_radius(radius)

    def update_radius(self, radius):
        if radius != self.radius:
            self.radius = radius
            self.W = gaussian_filter_matrix(self.centers, radius,
                                            self.design_mask)

    def forward(self, rho):
        out = np.copy(rho)
        out[self.design_mask] = self.W @ rho[self.design_mask]
        return out

    def gradient(self, v):
        out = np.zeros_like(v)
        out[self.design_mask] = self.W.T @ v[self.design_mask]
        return out


def element_to_node_average(mesh, vol, rho, design_mask, fixed_value):
    """helmholtz_filter_nodal.py:30-56 (weighted=True)."""
    val = np.where(design_mask, rho, fixed_value)
    num = np.zeros(mesh.nnodes)
    wsum = np.zeros(mesh.nnodes)
    for a in range(mesh.t.shape[0]):
        np.add.at(num, mesh.t[a], vol * val)
        np.add.at(wsum, mesh.t[a], vol)
    wsum[wsum == 0.0] = 1.0
    return num / wsum


def node_to_element_mean(mesh, x):
    """helmholtz_filter_nodal.py:26-27."""
    return np.mean(x[mesh.t], axis=0)


class HelmholtzFilterNodal:
    """helmholtz_filter_nodal.py:160-233."""

    def __init__(self, mesh, elements_volume, radius, design_mask):
        self.mesh = mesh
        self.vol = elements_volume
        self.design_mask = design_mask
        if mesh.kind == "hex":
            c = mesh.p[:, mesh.t[:, 0]]
            _, Kh = fem.hex_element_matrices(c, 0.3)
            M = fem.hex_mass_matrix(c)
            self.Kloc, self.Mloc = Kh, M
        else:
            _, Kh, M = fem.element_matrices(mesh, 0.3)
            self.Kloc, self.Mloc = Kh, M
        ones = np.ones(mesh.nelements)
        self.M = fem.assemble(mesh.t, self.Mloc, ones, mesh.nnodes, 1)
        self.K = fem.assemble(mesh.t, self.Kloc, ones, mesh.nnodes, 1)
        self.fixed_nodes = np.unique(mesh.t[:, ~design_mask].ravel())
        self.radius = radius

    def update_radius(self, radius):
        self.radius = radius

    def _A(self):
        return (self.M + (self.radius ** 2) * self.K).tocsr()

    def solve(self, rho_node, condense):
        """solve_helmholtz helmholtz_filter_nodal.py:121-157."""
        A = self._A()
        b = self.M @ rho_node
        if condense and self.fixed_nodes.size > 0:
            D = self.fixed_nodes
            I = np.setdiff1d(np.arange(A.shape[0]), D)
            x = np.zeros(A.shape[0])
            x[D] = 1.0
            rhs = b[I] - A[I][:, D] @ x[D]
            x[I] = spla.spsolve(A[I][:, I].tocsc(), rhs)
            return x
        return spla.spsolve(A.tocsc(), b)

    def forward(self, rho):
        rn = element_to_node_average(self.mesh, self.vol, rho,
                                     self.design_mask, 1.0)
        return node_to_element_mean(self.mesh, self.solve(rn, True))

    def gradient(self, v):
        vn = element_to_node_average(self.mesh, self.vol, v,
                                     self.design_mask, 0.0)
        out = node_to_element_mean(self.mesh, self.solve(vn, False))
        return np.minimum(out, 0.0)


def heaviside_projection(rho, beta, eta=0.5):
    """projection.py:27-77."""
    num = np.tanh(beta * eta) + np.tanh(beta * (rho - eta))
    den = np.tanh(beta * eta) + np.tanh(beta * (1.0 - eta)) + 1e-12
    return num / den


def heaviside_projection_derivative(rho, beta, eta=0.5):
    """projection.py:80-118: beta * sech^2(beta (rho - eta)) / denominator."""
    c = np.cosh(beta * (rho - eta))
    den = np.tanh(beta * eta) + np.tanh(beta * (1.0 - eta)) + 1e-12
    return (1.0 / (c * c)) * beta / den
