"""Oracle FEA: element matrices, assembly, enforce, solve, energy, sensitivity.

TEST INFRASTRUCTURE (see ``oracle/__init__.py``).  Restates:
* SIMP interpolation composer.py:19-22 and Lame parameters composer.py:82-83.
* ``assemble_stiffness_matrix`` composer.py:53-101 and
  ``assemble_conduction_matrix`` composer.py:104-145 (scikit-fem ``asm`` with
  ``ElementVector(ElementHex1)`` / ``ElementTetP1``, interleaved DOFs
  ``3*node + comp``, Gauss quadrature exact for affine cells, COO -> CSR with
  duplicates summed).
* ``skfem.enforce`` as used at solver_elastic.py:211 (rows and columns of the
  Dirichlet DOFs zeroed, unit diagonal, prescribed value in the RHS).
* ``solve_u`` solver_elastic.py:61-143 (spsolve, cg_jacobi, cg_pyamg), the maxiter rule
  solver_elastic.py:201-204, compliance solver_elastic.py:236 and 465.
* element strain energy solver_elastic.py:470-537 (1/2 u_e^T K_e(rho) u_e),
  heat energy solver_heat.py:256-303, ``dC_drho_simp`` derivatives.py:25-52.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .mesh import HEX_OFFSETS, GridMesh

_G = 0.5 / np.sqrt(3.0)
GAUSS2 = np.array([0.5 - _G, 0.5 + _G])   # 2-point Gauss on [0, 1]
GAUSS2_W = np.array([0.5, 0.5])


def simp_interpolation(rho, E0, Emin, p):
    """composer.py:19-22."""
    return Emin + (E0 - Emin) * (rho ** p)


def ramp_interpolation(rho, E0, Emin, p):
    """composer.py:25-39: Emin + (E0 - Emin) rho / (1 + p (1 - rho))."""
    return Emin + (E0 - Emin) * (rho / (1.0 + p * (1.0 - rho)))


def material(kind):
    """E(rho) of the interpolation named in DensityMethodConfig.interpolation."""
    return {"SIMP": simp_interpolation, "RAMP": ramp_interpolation}[kind]


def lame(E, nu):
    """composer.py:82-83."""
    lam = (nu * E) / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))
    return lam, mu


def hex_shape_grads_ref(xi):
    """d N_a / d xi for the trilinear hex on [0,1]^3 in MeshHex local order."""
    g = np.empty((8, 3))
    for a, o in enumerate(HEX_OFFSETS):
        f = [xi[d] if o[d] else 1.0 - xi[d] for d in range(3)]
        df = [1.0 if o[d] else -1.0 for d in range(3)]
        g[a, 0] = df[0] * f[1] * f[2]
        g[a, 1] = f[0] * df[1] * f[2]
        g[a, 2] = f[0] * f[1] * df[2]
    return g


def hex_shape_vals_ref(xi):
    v = np.empty(8)
    for a, o in enumerate(HEX_OFFSETS):
        v[a] = np.prod([xi[d] if o[d] else 1.0 - xi[d] for d in range(3)])
    return v


def _elastic_D(nu, E=1.0):
    lam, mu = lame(E, nu)
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] += 2.0 * mu
    D[3:, 3:] = np.eye(3) * mu
    return D


def _B_from_grads(g):
    """Engineering strain matrix (6 x 3n) for interleaved DOFs 3a+c."""
    n = g.shape[0]
    B = np.zeros((6, 3 * n))
    for a in range(n):
        gx, gy, gz = g[a]
        c = 3 * a
        B[0, c] = gx
        B[1, c + 1] = gy
        B[2, c + 2] = gz
        B[3, c] = gy; B[3, c + 1] = gx
        B[4, c + 1] = gz; B[4, c + 2] = gy
        B[5, c] = gz; B[5, c + 2] = gx
    return B


def hex_element_matrices(coords, nu):
    """Unit-modulus elastic (24x24) and unit-conductivity (8x8) matrices of one hex.

    ``coords`` is (3, 8) in MeshHex local order; 2x2x2 Gauss (intorder=2,
    toy_problem.py:80) with the isoparametric Jacobian.
    """
    D = _elastic_D(nu)
    Ke = np.zeros((24, 24))
    Kh = np.zeros((8, 8))
    for i, xi in enumerate(GAUSS2):
        for j, eta in enumerate(GAUSS2):
            for k, zeta in enumerate(GAUSS2):
                w = GAUSS2_W[i] * GAUSS2_W[j] * GAUSS2_W[k]
                gr = hex_shape_grads_ref((xi, eta, zeta))
                J = coords @ gr                    # (3,3): dx/dxi
                detJ = np.linalg.det(J)
                g = gr @ np.linalg.inv(J)          # (8,3): dN/dx
                B = _B_from_grads(g)
                Ke += w * detJ * (B.T @ D @ B)
                Kh += w * detJ * (g @ g.T)
    return Ke, Kh


def hex_mass_matrix(coords):
    """Consistent scalar mass matrix of one hex (Helmholtz filter)."""
    M = np.zeros((8, 8))
    for i, xi in enumerate(GAUSS2):
        for j, eta in enumerate(GAUSS2):
            for k, zeta in enumerate(GAUSS2):
                w = GAUSS2_W[i] * GAUSS2_W[j] * GAUSS2_W[k]
                gr = hex_shape_grads_ref((xi, eta, zeta))
                detJ = np.linalg.det(coords @ gr)
                N = hex_shape_vals_ref((xi, eta, zeta))
                M += w * detJ * np.outer(N, N)
    return M


def tet_element_matrices(coords, nu):
    """Unit-modulus elastic (12x12), conduction (4x4) and mass (4x4) of one P1 tet."""
    X = coords.T                                    # (4, 3)
    A = np.hstack([np.ones((4, 1)), X])             # rows [1 x y z]
    C = np.linalg.inv(A)                            # N_a = C[:, a] . [1 x y z]
    g = C[1:, :].T                                  # (4, 3)
    V = abs(np.linalg.det(A)) / 6.0
    B = _B_from_grads(g)
    Ke = V * (B.T @ _elastic_D(nu) @ B)
    Kh = V * (g @ g.T)
    M = V / 20.0 * (np.ones((4, 4)) + np.eye(4))
    return Ke, Kh, M


def element_matrices(mesh: GridMesh, nu):
    """Per-element unit matrices (n_e, ndof, ndof) for elasticity and heat."""
    ne = mesh.nelements
    nloc = mesh.t.shape[0]
    Ke = np.empty((ne, 3 * nloc, 3 * nloc))
    Kh = np.empty((ne, nloc, nloc))
    M = np.empty((ne, nloc, nloc))
    for e in range(ne):
        c = mesh.p[:, mesh.t[:, e]]
        if mesh.kind == "hex":
            Ke[e], Kh[e] = hex_element_matrices(c, nu)
            M[e] = hex_mass_matrix(c)
        else:
            Ke[e], Kh[e], M[e] = tet_element_matrices(c, nu)
    return Ke, Kh, M


def element_dofs(t, bs):
    """(bs*nloc, n_e) global DOFs, interleaved ``bs*node + comp``."""
    nloc, ne = t.shape
    d = np.empty((bs * nloc, ne), dtype=np.int64)
    for a in range(nloc):
        for c in range(bs):
            d[bs * a + c] = bs * t[a] + c
    return d


def assemble(t, Kloc, scale, n_nodes, bs):
    """Sum_e scale_e * Kloc_e into a canonical CSR (scikit-fem ``asm``)."""
    dofs = element_dofs(t, bs)
    n = dofs.shape[0]
    ne = t.shape[1]
    rows = np.broadcast_to(dofs.T[:, :, None], (ne, n, n)).reshape(-1)
    cols = np.broadcast_to(dofs.T[:, None, :], (ne, n, n)).reshape(-1)
    if Kloc.ndim == 2:
        vals = (scale[:, None, None] * Kloc[None, :, :]).reshape(-1)
    else:
        vals = (scale[:, None, None] * Kloc).reshape(-1)
    N = bs * n_nodes
    K = sp.coo_matrix((vals, (rows, cols)), shape=(N, N)).tocsr()
    K.sum_duplicates()
    K.sort_indices()
    return K


def enforce(K, f, D):
    """``skfem.enforce`` with x = 0 on D: zero rows and columns, unit diagonal."""
    K = K.tocsr(copy=True)
    N = K.shape[0]
    mask = np.zeros(N, dtype=bool)
    mask[D] = True
    rows = np.repeat(np.arange(N), np.diff(K.indptr))
    kill = mask[rows] | mask[K.indices]
    K.data[kill] = 0.0
    diag = (rows == K.indices) & mask[rows]
    K.data[diag] = 1.0
    fe = np.array(f, dtype=float, copy=True)
    if fe.ndim == 1:
        fe[D] = 0.0
    else:
        fe[D, :] = 0.0
    return K, fe


def default_maxiter(n_dof, maxiter=None):
    """solver_elastic.py:201-204."""
    return min(1000, max(300, n_dof // 5)) if maxiter is None else maxiter


def solve(Ke, Fe, solver="spsolve", rtol=1e-8, maxiter=None):
    """solver_elastic.py:61-143 for 'spsolve', 'cg_jacobi' and 'cg_pyamg'
    (the smoothed-aggregation preconditioner of ``oracle/amg.py``)."""
    if solver == "spsolve":
        if Fe.ndim == 2:
            lu = spla.splu(Ke.tocsc())
            return lu.solve(Fe)
        return spla.spsolve(Ke.tocsc(), Fe)
    if solver == "spsolve_mmd":
        # the same direct solve with SuperLU's minimum-degree ordering of
        # A^T + A: less fill on these symmetric 3-D systems, several times
        # faster at 60x20x20, the same solution to rounding
        lu = spla.splu(Ke.tocsc(), permc_spec="MMD_AT_PLUS_A")
        return lu.solve(Fe)
    if solver == "cg_pyamg":
        from .amg import cg_pyamg
        mi = default_maxiter(Ke.shape[0], maxiter)
        if Fe.ndim == 2:
            return np.stack([cg_pyamg(Ke, Fe[:, j], rtol, mi) for j in range(Fe.shape[1])],
                            axis=1)
        return cg_pyamg(Ke, Fe, rtol, mi)
    if solver == "cg_jacobi":
        Minv = 1.0 / Ke.diagonal()
        M = spla.LinearOperator(Ke.shape, matvec=lambda x: Minv * x)
        u, info = spla.cg(Ke, Fe, M=M, rtol=rtol,
                          maxiter=default_maxiter(Ke.shape[0], maxiter))
        return u
    raise ValueError(f"Unknown solver: {solver}")


def element_quadratic(u, dofs, Kloc):
    """u_e^T Kloc_e u_e for every element (Kloc shared (n,n) or (n_e,n,n))."""
    ue = u[dofs]                       # (n, n_e)
    if Kloc.ndim == 2:
        return np.einsum("ie,ij,je->e", ue, Kloc, ue)
    return np.einsum("ie,eij,je->e", ue, Kloc, ue)


def dE_drho_simp(rho, E0, Emin, p):
    """derivatives.py:34-39."""
    return p * (E0 - Emin) * np.maximum(rho, 1e-6) ** (p - 1)


def E_simp(rho, E0, Emin, p):
    """derivatives.py:25-26."""
    return Emin + (E0 - Emin) * np.maximum(rho, 1e-6) ** p


def dC_drho_simp(rho, strain_energy, E0, Emin, p):
    """derivatives.py:42-52: -(dE/drho) * 2 U_e / E."""
    dE = dE_drho_simp(rho, E0, Emin, p)
    E = E_simp(rho, E0, Emin, p)
    return -2.0 * strain_energy * dE / np.maximum(E, 1e-12)


def dC_drho_ramp(rho, strain_energy, E0, Emin, p):
    """derivatives.py:56-72 (dE_drho_ramp, _E_ramp)."""
    den = 1.0 + p * (1.0 - rho)
    dE = (E0 - Emin) * (den - p * rho) / (den ** 2)
    E = Emin + (E0 - Emin) * (rho / den)
    return -2.0 * strain_energy * dE / np.maximum(E, 1e-12)


def sensitivity(kind):
    """dC/drho of the interpolation named in DensityMethodConfig.interpolation."""
    return {"SIMP": dC_drho_simp, "RAMP": dC_drho_ramp}[kind]


class ElasticProblem:
    """Linear elasticity on a GridMesh with nodal loads (task_elastic.py:85-147)."""

    def __init__(self, mesh, dirichlet_nodes, forces, E0=1.0, nu=0.3,
                 Kloc=None):
        self.mesh = mesh
        self.E0 = E0
        self.nu = nu
        self.bs = 3
        self.n_dof = 3 * mesh.nnodes
        dn = np.asarray(dirichlet_nodes, dtype=np.int64)
        self.dirichlet_dofs = np.sort(
            (3 * dn[:, None] + np.arange(3)[None, :]).reshape(-1))
        self.forces = [np.asarray(f, float) for f in forces]
        if Kloc is None:
            if mesh.kind == "hex" and _is_uniform_box(mesh):
                c = mesh.p[:, mesh.t[:, 0]]
                Kloc, _ = hex_element_matrices(c, nu)
            else:
                Kloc = element_matrices(mesh, nu)[0]
        self.Kloc = Kloc
        self.dofs = element_dofs(mesh.t, 3)

    def stiffness(self, rho, p, Emin):
        E = material(getattr(self, "interp", "SIMP"))(rho, self.E0, Emin, p)
        return assemble(self.mesh.t, self.Kloc, E, self.mesh.nnodes, 3)

    def objectives(self, rho, p, Emin, solver="spsolve", rtol=1e-8,
                   force_scale=1.0):
        """compute_compliance_basis(_multi_load) solver_elastic.py:146-467."""
        K = self.stiffness(rho, p, Emin)
        F = np.column_stack([f * force_scale for f in self.forces])
        Ke, Fe = enforce(K, F, self.dirichlet_dofs)
        free = np.setdiff1d(np.arange(self.n_dof), self.dirichlet_dofs)
        if F.shape[1] == 1:
            u = solve(Ke, Fe[:, 0], solver, rtol)[:, None]
            comp = np.array([Fe[free, 0] @ u[free, 0]])
        else:
            u = solve(Ke, Fe, "spsolve")
            comp = np.einsum("ij,ij->j", Fe, u)
        return comp, u

    def energy(self, rho, p, Emin, U):
        """strain_energy_skfem_multi solver_elastic.py:507-537."""
        E = material(getattr(self, "interp", "SIMP"))(rho, self.E0, Emin, p)
        out = np.empty((rho.size, U.shape[1]))
        for i in range(U.shape[1]):
            out[:, i] = 0.5 * E * element_quadratic(U[:, i], self.dofs, self.Kloc)
        return out


class HeatProblem:
    """Steady conduction with Dirichlet T=0 and a volumetric source."""

    def __init__(self, mesh, dirichlet_nodes, source=1.0, k0=1.0, Kloc=None,
                 emit=None):
        self.mesh = mesh
        self.E0 = k0
        self.bs = 1
        self.n_dof = mesh.nnodes
        self.dirichlet_dofs = np.sort(np.asarray(dirichlet_nodes, np.int64))
        if Kloc is None:
            if mesh.kind == "hex" and _is_uniform_box(mesh):
                c = mesh.p[:, mesh.t[:, 0]]
                _, Kloc = hex_element_matrices(c, 0.3)
            else:
                Kloc = element_matrices(mesh, 0.3)[1]
        self.Kloc = Kloc
        self.dofs = element_dofs(mesh.t, 1)
        if emit is None:
            emit = source_vector(mesh, source)
        self.emit = emit

    def stiffness(self, rho, p, kmin):
        k = simp_interpolation(rho, self.E0, kmin, p)
        return assemble(self.mesh.t, self.Kloc, k, self.mesh.nnodes, 1)

    def objectives(self, rho, p, kmin, solver="spsolve", rtol=1e-8):
        """solver_heat.py:198-253 and compliance T^T K T at 785-789."""
        K = self.stiffness(rho, p, kmin)
        Ke, fe = enforce(K, self.emit, self.dirichlet_dofs)
        T = solve(Ke, fe, solver, rtol)
        return np.array([T @ (K @ T)]), T[:, None]

    def energy(self, rho, p, kmin, U):
        """heat_energy_skfem_multi solver_heat.py:282-303 (1/2 k |grad T|^2)."""
        k = simp_interpolation(rho, self.E0, kmin, p)
        return (0.5 * k * element_quadratic(U[:, 0], self.dofs, self.Kloc))[:, None]


def source_vector(mesh, s):
    """Load of a uniform volumetric source s: f_a = s * integral of N_a."""
    f = np.zeros(mesh.nnodes)
    if mesh.kind == "hex":
        for e in range(mesh.nelements):
            c = mesh.p[:, mesh.t[:, e]]
            fe = np.zeros(8)
            for xi in GAUSS2:
                for eta in GAUSS2:
                    for zeta in GAUSS2:
                        gr = hex_shape_grads_ref((xi, eta, zeta))
                        fe += 0.125 * np.linalg.det(c @ gr) * \
                            hex_shape_vals_ref((xi, eta, zeta))
            np.add.at(f, mesh.t[:, e], s * fe)
    else:
        c = mesh.p[:, mesh.t]
        v1 = c[:, 1] - c[:, 0]
        v2 = c[:, 2] - c[:, 0]
        v3 = c[:, 3] - c[:, 0]
        vol = np.abs(np.einsum("ij,ij->j", np.cross(v1.T, v2.T).T, v3)) / 6.0
        for a in range(4):
            np.add.at(f, mesh.t[a], s * vol / 4.0)
    return f


def _is_uniform_box(mesh):
    """True when every hex is a translate of the first one."""
    c = mesh.p[:, mesh.t]
    rel = c - c[:, :1, :]
    return np.allclose(rel, rel[:, :, :1], rtol=0, atol=1e-12)
