"""Oracle of the heat plugin's Robin terms and heat objectives (TEST INFRASTRUCTURE).

Only ``tests/``, the smoke entry and the bench's CPU legs use this module, as
the checker.  It restates, on hexahedral meshes with the 2x2x2 Gauss rule of
the element matrices (basis intorder=2) and on P1 tetrahedra with the
4-point degree-2 rule (intorder=2: barycentric points (a, b, b, b),
a = (5 + 3 sqrt 5) / 20, b = (5 - sqrt 5) / 20, weights 1/4 of the volume)
for every volume form:

* ``_element_to_nodal_average`` sktopt/fea/solver_heat.py:600-613 and the
  same average inside ``objectives_multi_load`` 730-737: ``np.add.at`` over
  ``t.ravel()`` with ``np.repeat(rho, nloc)``, divided by max(count, 1).
  ``t`` is (nloc, n_elem), so ``t.ravel()`` runs over the local index first
  and ``np.repeat`` over the elements first: the entry ``t[a, e]`` receives
  ``rho[(a * n_elem + e) // nloc]``.  ``pairing="reference"`` keeps that;
  ``pairing="element"`` gives node ``t[a, e]`` the density of element e.
* ``get_robin_virtual`` solver_heat.py:552-572: K += h rho^p (1-rho)^q
  |grad rho| u v and f += the same times T_env v, rho the interpolated
  nodal average.
* ``assemble_surface_robin`` sktopt/mesh/task_heat.py:60-139: K += h u v and
  f += h T_env v on the Robin facets (its density-weighted branch never runs:
  ``rho_field`` stays None there).
* ``solve_multi_load`` / ``solve_heat_system_multi`` solver_heat.py:136-253:
  K = conduction + Robin terms; every Dirichlet value gives one column with
  T = value on the Dirichlet nodes (``skfem.enforce`` with x = value).
* ``objectives_multi_load`` solver_heat.py:705-895: compliance T^T K T with
  K before enforcement; heat exchange J_num / J_den (306-321, 382-390,
  411-440) with the adjoint K_e lam = dJ/dT (392-408, 823-843; the Dirichlet
  value is enforced on the adjoint too), zero when J_den <= 1e-16 (803-809);
  averaged temperature sum(T) with K_e lam = 1 (876-890); the
  ``avg_temp_weight`` combination 845-874.
* ``energy_multi_load`` 897-926: 1/2 k |grad T|^2, or grad T . grad lam
  (324-379, 529-550) per element.
* ``compliance_sensitivity_multi_load`` 928-980: ``dC_drho_simp`` of the
  conduction energy (SIMP derivative whatever the interpolation), plus, for
  the compliance objective with Robin data, the explicit term
  ``_robin_compliance_explicit_grad_`` 575-597 mapped to elements by
  ``_nodal_gradient_to_element_gradient`` 616-625.

Parity unpinned at the scikit-fem boundary (scikit-fem is absent here); the
analytic checks of tests/test_cpu_heat_robin.py pin the quadrature.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import fem
from .fem import GAUSS2, GAUSS2_W, hex_shape_grads_ref, hex_shape_vals_ref
from .mesh import HEX_OFFSETS


def hex_quadrature(mesh):
    """Shape values N (nq, 8), physical gradients dN (ne, nq, 8, 3) and
    weights w*detJ (ne, nq) at the 2x2x2 Gauss points of every hexahedron."""
    pts = []
    for i, xi in enumerate(GAUSS2):
        for j, eta in enumerate(GAUSS2):
            for k, zeta in enumerate(GAUSS2):
                pts.append(((xi, eta, zeta), GAUSS2_W[i] * GAUSS2_W[j] * GAUSS2_W[k]))
    N = np.array([hex_shape_vals_ref(x) for x, _ in pts])            # (nq, 8)
    gr = np.array([hex_shape_grads_ref(x) for x, _ in pts])          # (nq, 8, 3)
    c = mesh.p[:, mesh.t]                                            # (3, 8, ne)
    J = np.einsum("dae,qak->eqdk", c, gr)                            # dx_d / dxi_k
    det = np.linalg.det(J)
    Jinv = np.linalg.inv(J)
    dN = np.einsum("qak,eqkd->eqad", gr, Jinv)
    w = np.array([wq for _, wq in pts])
    return N, dN, w[None, :] * det


_TA = (5.0 + 3.0 * np.sqrt(5.0)) / 20.0
_TB = (5.0 - np.sqrt(5.0)) / 20.0


def tet_quadrature(mesh):
    """Shape values N (4, 4) at the 4-point degree-2 rule, the constant
    physical gradients dN (ne, 4, 4, 3) and weights w*detJ (ne, 4) of every
    P1 tetrahedron."""
    N = np.full((4, 4), _TB)
    np.fill_diagonal(N, _TA)                                       # point q: (a at node q)
    c = mesh.p[:, mesh.t]                                          # (3, 4, ne)
    J = np.stack([c[:, 1] - c[:, 0], c[:, 2] - c[:, 0], c[:, 3] - c[:, 0]], axis=2)  # (3, ne, 3)
    J = np.transpose(J, (1, 0, 2))                                 # (ne, 3, 3): dx_d / dxi_k
    det = np.linalg.det(J)
    Jinv = np.linalg.inv(J)
    gr = np.array([[-1.0, -1.0, -1.0], [1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0]])  # dN/dxi
    g = np.einsum("ak,ekd->ead", gr, Jinv)                         # (ne, 4, 3)
    dN = np.broadcast_to(g[:, None], (g.shape[0], 4, 4, 3)).copy()
    wd = np.repeat((np.abs(det) / 24.0)[:, None], 4, axis=1)
    return N, dN, wd


def element_quadrature(mesh):
    return hex_quadrature(mesh) if mesh.kind == "hex" else tet_quadrature(mesh)


def nodal_average(mesh, rho, pairing="reference"):
    """solver_heat.py:600-613.  Returns (rho_nodal, count)."""
    t = mesh.t
    nloc, ne = t.shape
    nv = mesh.nnodes
    vals = np.repeat(rho, nloc) if pairing == "reference" else np.tile(rho, nloc)
    rn = np.zeros(nv)
    cnt = np.zeros(nv)
    np.add.at(rn, t.ravel(), vals)
    np.add.at(cnt, t.ravel(), 1.0)
    rn /= np.maximum(cnt, 1.0)
    return rn, cnt


def _at_qp(N, dN, mesh, x_nodal):
    xe = x_nodal[mesh.t]                                             # (8, ne)
    val = np.einsum("qa,ae->eq", N, xe)
    grad = np.einsum("eqad,ae->eqd", dN, xe)
    return val, grad


def _scatter_vec(mesh, fe):
    """Sum element vectors fe (ne, 8) into a nodal vector."""
    out = np.zeros(mesh.nnodes)
    np.add.at(out, mesh.t.T.ravel(), fe.ravel())
    return out


def _assemble_mats(mesh, Me):
    t = mesh.t
    nloc, ne = t.shape
    rows = np.broadcast_to(t.T[:, :, None], (ne, nloc, nloc)).reshape(-1)
    cols = np.broadcast_to(t.T[:, None, :], (ne, nloc, nloc)).reshape(-1)
    n = mesh.nnodes
    K = sp.coo_matrix((Me.reshape(-1), (rows, cols)), shape=(n, n)).tocsr()
    K.sum_duplicates()
    K.sort_indices()
    return K


def virtual_robin(mesh, Q, rho_n, h, t_env, p, q):
    """get_robin_virtual solver_heat.py:552-572: element matrices (ne, 8, 8)
    and element load vectors (ne, 8)."""
    N, dN, wd = Q
    r, g = _at_qp(N, dN, mesh, rho_n)
    iface = np.sqrt(np.sum(g ** 2, axis=2))
    heff = h * r ** p * (1.0 - r) ** q
    c = wd * heff * iface                                            # (ne, nq)
    Me = np.einsum("eq,qa,qb->eab", c, N, N)
    fe = np.einsum("eq,qa->ea", c * t_env, N)
    return Me, fe


# local faces of the hexahedron: (axis, side) -> the 4 local nodes
def hex_face_nodes(axis, side):
    return [a for a in range(8) if HEX_OFFSETS[a][axis] == side]


TET_FACES = [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]]


def surface_robin_tet(mesh, faces, h, t_env):
    """assemble_surface_robin task_heat.py:60-139 on triangle facets, rows
    (element, local face): h int N_a N_b = h A / 12 (1 + delta_ab) and
    h T_env int N_a = h T_env A / 3 (exact)."""
    nf = faces.shape[0]
    Me = np.zeros((nf, 4, 4))
    load = np.zeros(mesh.nnodes)
    for k, (e, f) in enumerate(faces):
        loc = TET_FACES[f]
        X = mesh.p[:, mesh.t[loc, e]]
        A = 0.5 * np.linalg.norm(np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]))
        for i, a in enumerate(loc):
            for j, b in enumerate(loc):
                Me[k, a, b] = h * A / 12.0 * (2.0 if i == j else 1.0)
        np.add.at(load, mesh.t[loc, e], h * t_env * A / 3.0)
    return Me, load


def surface_robin(mesh, faces, h, t_env):
    """assemble_surface_robin task_heat.py:60-139 for one facet group.

    faces: (nf, 3) rows (element, axis, side) on hexahedra, (nf, 2) rows
    (element, local face) on tetrahedra.  Returns per-face element matrices
    (nf, nloc, nloc) (zero outside the face's nodes) and the nodal load.
    Hexahedra: 2x2 Gauss on the bilinear face map (exact for these
    polynomial forms)."""
    if mesh.kind != "hex":
        return surface_robin_tet(mesh, faces, h, t_env)
    nf = faces.shape[0]
    Me = np.zeros((nf, 8, 8))
    load = np.zeros(mesh.nnodes)
    for k, (e, axis, side) in enumerate(faces):
        loc = hex_face_nodes(axis, side)
        ax = [d for d in range(3) if d != axis]
        X = mesh.p[:, mesh.t[loc, e]]                               # (3, 4)
        uv = HEX_OFFSETS[loc][:, ax]                                # (4, 2)
        m = np.zeros((4, 4))
        f = np.zeros(4)
        for i, s in enumerate(GAUSS2):
            for j, tt in enumerate(GAUSS2):
                w = GAUSS2_W[i] * GAUSS2_W[j]
                Nf = np.array([(s if o[0] else 1 - s) * (tt if o[1] else 1 - tt) for o in uv])
                dS = np.array([(1.0 if o[0] else -1.0) * (tt if o[1] else 1 - tt) for o in uv])
                dT = np.array([(s if o[0] else 1 - s) * (1.0 if o[1] else -1.0) for o in uv])
                jac = np.linalg.norm(np.cross(X @ dS, X @ dT))
                m += w * jac * np.outer(Nf, Nf)
                f += w * jac * Nf
        for i, a in enumerate(loc):
            for j, b in enumerate(loc):
                Me[k, a, b] = h * m[i, j]
        np.add.at(load, mesh.t[loc, e], h * t_env * f)
    return Me, load


def hx_den(mesh, Q, rho_n):
    """_hx_den_density_ solver_heat.py:382-390 summed over elements."""
    N, dN, wd = Q
    _, g = _at_qp(N, dN, mesh, rho_n)
    return float(np.sum(wd * np.sqrt(np.sum(g ** 2, axis=2))))


def hx_num(mesh, Q, rho_n, T, h, t_env):
    """_hx_num_density_ solver_heat.py:306-321 summed (h the scalar coefficient)."""
    N, dN, wd = Q
    _, g = _at_qp(N, dN, mesh, rho_n)
    Tq, _ = _at_qp(N, dN, mesh, T)
    iface = np.sqrt(np.sum(g ** 2, axis=2))
    return float(np.sum(wd * (-t_env * h * (Tq - t_env) * iface)))


def hx_adj_rhs(mesh, Q, rho_n, h, t_env, p, q):
    """_hx_adj_rhs_ solver_heat.py:392-408 with h_eff the interpolated nodal
    h rho^p (1 - rho)^q (825-830), before the division by J_den."""
    N, dN, wd = Q
    _, g = _at_qp(N, dN, mesh, rho_n)
    heff_n = h * rho_n ** p * (1.0 - rho_n) ** q
    hq, _ = _at_qp(N, dN, mesh, heff_n)
    iface = np.sqrt(np.sum(g ** 2, axis=2))
    fe = np.einsum("eq,qa->ea", wd * (-t_env * hq * iface), N)
    return _scatter_vec(mesh, fe)


def robin_explicit_grad(mesh, Q, rho_n, T, h, t_env, p, q):
    """_robin_compliance_explicit_grad_ solver_heat.py:575-597 (nodal vector)."""
    N, dN, wd = Q
    r, g = _at_qp(N, dN, mesh, rho_n)
    Tq, _ = _at_qp(N, dN, mesh, T)
    iface = np.sqrt(np.sum(g ** 2, axis=2))
    safe = np.maximum(iface, 1e-12)
    a = r ** p * (1.0 - r) ** q
    da = p * r ** (p - 1.0) * (1.0 - r) ** q - q * r ** p * (1.0 - r) ** (q - 1.0)
    phi = 2.0 * t_env * Tq - Tq * Tq
    term1 = np.einsum("eq,qa->ea", wd * h * da * iface * phi, N)
    nrm = g / safe[:, :, None]
    term2 = np.einsum("eq,eqd,eqad->ea", wd * h * a * phi, nrm, dN)
    return _scatter_vec(mesh, term1 + term2)


def nodal_to_element(mesh, nodal, count):
    """_nodal_gradient_to_element_gradient solver_heat.py:616-625."""
    out = np.zeros(mesh.nelements)
    for local_nodes in mesh.t:
        out += nodal[local_nodes] / np.maximum(count[local_nodes], 1.0)
    return out


def _solve_enforced(K, f, D, value):
    """skfem.enforce with x = value on D, then a direct solve.  The solve
    runs on x - value (same solution): the constant field carries the
    prescribed value, so rounding acts on the small deviation only."""
    n = K.shape[0]
    g = np.full(n, float(value))
    rhs = f - K @ g
    Ke, fe = fem.enforce(K, rhs, D)
    d = spla.spsolve(Ke.tocsc(), fe)
    d[D] = 0.0
    return g + d


def grad_dot(mesh, Q, X, Y):
    """Per element int grad X . grad Y with the gradients at the quadrature
    points (the skfem form of solver_heat.py:256-262, 324-338, 529-533)."""
    N, dN, wd = Q
    _, gx = _at_qp(N, dN, mesh, X)
    _, gy = _at_qp(N, dN, mesh, Y)
    return np.sum(wd * np.sum(gx * gy, axis=2), axis=1)


class HeatRobinProblem:
    """FEM_SimpLinearHeatConduction (solver_heat.py:628-980) on a hex or P1
    tet mesh."""

    def __init__(self, mesh, dirichlet_nodes, dirichlet_values, k0=1.0,
                 robin_faces=None, robin_coefficient=None, robin_bc_value=None,
                 objective="compliance", avg_temp_weight=0.0, q=4.0, emit=None,
                 pairing="reference"):
        self.mesh = mesh
        self.E0 = k0
        self.bs = 1
        self.n_dof = mesh.nnodes
        self.D = np.sort(np.asarray(dirichlet_nodes, np.int64))
        vals = dirichlet_values if isinstance(dirichlet_values, (list, tuple)) \
            else [dirichlet_values]
        self.values = [float(v) for v in vals]
        if mesh.kind == "hex" and fem._is_uniform_box(mesh):
            c = mesh.p[:, mesh.t[:, 0]]
            _, self.Kloc = fem.hex_element_matrices(c, 0.3)
        else:   # tetrahedra and general hexahedra: per-element matrices
            _, self.Kloc, _ = fem.element_matrices(mesh, 0.3)
        self.dofs = fem.element_dofs(mesh.t, 1)
        self.h = robin_coefficient
        self.t_env = robin_bc_value
        self.objective = objective
        self.avg_w = float(avg_temp_weight)
        self.q = float(q)
        self.pairing = pairing
        self.emit = np.zeros(mesh.nnodes) if emit is None else np.asarray(emit, float)
        self.Q = element_quadrature(mesh)
        # surface Robin terms (rho independent)
        self.surf_K = sp.csr_matrix((mesh.nnodes, mesh.nnodes))
        self.surf_f = np.zeros(mesh.nnodes)
        if robin_faces is not None:
            groups = robin_faces if isinstance(robin_faces, list) else [robin_faces]
            hs = self.h if isinstance(self.h, list) else [self.h] * len(groups)
            ts = self.t_env if isinstance(self.t_env, list) else [self.t_env] * len(groups)
            for faces, hh, tt in zip(groups, hs, ts):
                Me, load = surface_robin(mesh, np.asarray(faces), hh, tt)
                if len(faces):
                    nloc = mesh.t.shape[0]
                    sub = np.zeros((mesh.nelements, nloc, nloc))
                    np.add.at(sub, np.asarray(faces)[:, 0], Me)
                    self.surf_K = self.surf_K + _assemble_mats(mesh, sub)
                self.surf_f += load
        self.lam = None

    def operator(self, rho, p, kmin):
        """K (before enforcement) and f of solve_multi_load solver_heat.py:198-253."""
        k = fem.material(getattr(self, "interp", "SIMP"))(rho, self.E0, kmin, p)
        K = fem.assemble(self.mesh.t, self.Kloc, k, self.mesh.nnodes, 1) + self.surf_K
        f = self.emit + self.surf_f
        rho_n = None
        if self.h is not None:
            rho_n, _ = nodal_average(self.mesh, rho, self.pairing)
            Me, fe = virtual_robin(self.mesh, self.Q, rho_n, self.h, self.t_env, p, self.q)
            K = K + _assemble_mats(self.mesh, Me)
            f = f + _scatter_vec(self.mesh, fe)
        return K.tocsr(), f, rho_n

    def objectives(self, rho, p, kmin, solver="spsolve", rtol=1e-8):
        K, f, rho_n = self.operator(rho, p, kmin)
        nl = len(self.values)
        T = np.column_stack([_solve_enforced(K, f, self.D, v) for v in self.values])
        obj = self.objective
        if obj == "compliance":
            J = np.array([T[:, i] @ (K @ T[:, i]) for i in range(nl)])
            self.lam = -2.0 * T
        elif obj == "heat_exchange":
            if rho_n is None:
                raise RuntimeError("heat_exchange objective requires Robin boundary data.")
            den = hx_den(self.mesh, self.Q, rho_n)
            if den <= 1e-16:
                self.lam = np.zeros_like(T)
                return np.zeros(nl), T
            J = np.array([hx_num(self.mesh, self.Q, rho_n, T[:, i], self.h, self.t_env) / den
                          for i in range(nl)])
            rhs = hx_adj_rhs(self.mesh, self.Q, rho_n, self.h, self.t_env, p, self.q) / den
            lam = np.column_stack([_solve_enforced(K, rhs, self.D, v) for v in self.values])
            if self.avg_w != 0.0:
                avg = T.sum(axis=0)
                lam_avg = np.column_stack([_solve_enforced(K, np.ones(self.n_dof), self.D, v)
                                           for v in self.values])
                if nl > 1:
                    hs = max(float(np.mean(np.abs(J))), 1e-12)
                    as_ = max(float(np.mean(np.abs(avg))), 1e-12)
                    J = J / hs + self.avg_w * (avg / as_)
                    lam = lam / hs + (self.avg_w / as_) * lam_avg
                else:
                    J = J + self.avg_w * avg
                    lam = lam + self.avg_w * lam_avg
            self.lam = lam
        elif obj == "averaged_temp":
            J = T.sum(axis=0)
            self.lam = np.column_stack([_solve_enforced(K, np.ones(self.n_dof), self.D, v)
                                        for v in self.values])
        else:
            raise ValueError(f"Unknown objective: {obj}")
        return J, T

    def conduction_energy(self, rho, p, kmin, U):
        """heat_energy_skfem_multi solver_heat.py:282-303: 1/2 k |grad T|^2
        integrated with the gradients at the quadrature points."""
        k = fem.material(getattr(self, "interp", "SIMP"))(rho, self.E0, kmin, p)
        return np.column_stack([0.5 * k * grad_dot(self.mesh, self.Q, U[:, i], U[:, i])
                                for i in range(U.shape[1])])

    def energy(self, rho, p, kmin, U):
        """energy_multi_load solver_heat.py:897-926."""
        if self.objective == "compliance":
            return self.conduction_energy(rho, p, kmin, U)
        return np.column_stack([grad_dot(self.mesh, self.Q, U[:, i], self.lam[:, i])
                                for i in range(U.shape[1])])

    def custom_sensitivity(self, rho, p, kmin, U):
        """compliance_sensitivity_multi_load solver_heat.py:928-980."""
        en = self.conduction_energy(rho, p, kmin, U)
        grad = np.column_stack([fem.dC_drho_simp(rho, en[:, i], self.E0, kmin, p)
                                for i in range(U.shape[1])])
        if self.objective != "compliance" or self.h is None:
            return grad
        rho_n, cnt = nodal_average(self.mesh, rho, self.pairing)
        hs = self.h if isinstance(self.h, list) else [self.h]
        ts = self.t_env if isinstance(self.t_env, list) else [self.t_env]
        for hh, tt in zip(hs, ts):
            for i in range(U.shape[1]):
                ng = robin_explicit_grad(self.mesh, self.Q, rho_n, U[:, i], float(hh), tt,
                                         float(p), self.q)
                grad[:, i] += nodal_to_element(self.mesh, ng, cnt)
        return grad
