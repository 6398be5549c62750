"""Element matrices and material interpolation (set-up, host side).

Mirrors sktopt/fea/composer.py: SIMP and RAMP interpolation (19-39), Lame parameters
(82-83), and the bilinear forms assembled by ``assemble_stiffness_matrix``
(53-101: lambda tr(eps(u)) tr(eps(v)) + 2 mu eps(u):eps(v)) and
``assemble_conduction_matrix`` (104-145: grad u . grad v) for the
``ElementHex1`` (2x2x2 Gauss, intorder=2 as in toy_problem.py:80) and
``ElementTetP1`` bases, with interleaved DOFs ``3*node + comp``.  The GPU
assembles sum_e coef_e Ke from these unit-modulus matrices.
"""
from __future__ import annotations

import numpy as np

from ..mesh.grid import HEX_OFFSETS, GridMesh


def simp_interpolation(rho, E0, Emin, p):
    """composer.py:19-22."""
    return Emin + (E0 - Emin) * (rho ** p)


def ramp_interpolation(rho, E0, Emin, p):
    """composer.py:25-39: Emin + (E0 - Emin) rho / (1 + p (1 - rho))."""
    return Emin + (E0 - Emin) * (rho / (1.0 + p * (1.0 - rho)))


def interpolation_kind(fn) -> int:
    """Kernel code of a material interpolation: 0 SIMP, 1 RAMP."""
    name = getattr(fn, "__name__", "")
    if fn is simp_interpolation or name == "simp_interpolation":
        return 0
    if fn is ramp_interpolation or name == "ramp_interpolation":
        return 1
    raise NotImplementedError("the GPU path implements SIMP and RAMP interpolation")


def lame_parameters(E, nu):
    """composer.py:82-83."""
    return (nu * E) / ((1.0 + nu) * (1.0 - 2.0 * nu)), E / (2.0 * (1.0 + nu))


def _gauss2():
    g = 0.5 / np.sqrt(3.0)
    pts = np.array([0.5 - g, 0.5 + g])
    X = np.array([[a, b, c] for c in pts for b in pts for a in pts])   # (8, 3)
    return X, np.full(8, 0.125)


def _hex_ref_grads(X):
    """(nq, 8, 3) reference gradients of the trilinear shape functions on [0,1]^3."""
    o = HEX_OFFSETS.astype(np.float64)                     # (8, 3)
    f = np.where(o[None] == 1.0, X[:, None, :], 1.0 - X[:, None, :])   # (nq, 8, 3)
    s = np.where(o == 1.0, 1.0, -1.0)[None]                # (1, 8, 3)
    g = np.empty_like(f)
    g[..., 0] = s[..., 0] * f[..., 1] * f[..., 2]
    g[..., 1] = f[..., 0] * s[..., 1] * f[..., 2]
    g[..., 2] = f[..., 0] * f[..., 1] * s[..., 2]
    vals = f[..., 0] * f[..., 1] * f[..., 2]
    return g, vals


def _strain_operator(G):
    """G (..., n, 3) physical gradients -> B (..., 6, 3n), engineering strains."""
    n = G.shape[-2]
    B = np.zeros(G.shape[:-2] + (6, 3 * n))
    gx, gy, gz = G[..., 0], G[..., 1], G[..., 2]
    B[..., 0, 0::3] = gx
    B[..., 1, 1::3] = gy
    B[..., 2, 2::3] = gz
    B[..., 3, 0::3] = gy
    B[..., 3, 1::3] = gx
    B[..., 4, 1::3] = gz
    B[..., 4, 2::3] = gy
    B[..., 5, 0::3] = gz
    B[..., 5, 2::3] = gx
    return B


def _elastic_D(nu):
    lam, mu = lame_parameters(1.0, nu)
    D = np.diag([2 * mu, 2 * mu, 2 * mu, mu, mu, mu]).astype(np.float64)
    D[:3, :3] += lam
    return D


def hex_matrices(coords, nu):
    """coords (n_e, 3, 8) -> elastic (n_e,24,24), conduction (n_e,8,8), mass (n_e,8,8)."""
    X, w = _gauss2()
    g, vals = _hex_ref_grads(X)                            # (q,8,3), (q,8)
    J = np.einsum("eda,qak->eqdk", coords, g)              # dx_d/dxi_k
    detJ = np.linalg.det(J)                                # (e,q)
    Jinv = np.linalg.inv(J)                                # (e,q,k,d)
    G = np.einsum("qak,eqkd->eqad", g, Jinv)               # dN_a/dx_d
    wd = detJ * w[None]                                    # (e,q)
    B = _strain_operator(G)                                # (e,q,6,24)
    D = _elastic_D(nu)
    Ke = np.einsum("eq,eqik,ij,eqjl->ekl", wd, B, D, B, optimize=True)
    Kh = np.einsum("eq,eqad,eqbd->eab", wd, G, G, optimize=True)
    M = np.einsum("eq,qa,qb->eab", wd, vals, vals, optimize=True)
    return Ke, Kh, M


def tet_matrices(coords, nu):
    """coords (n_e, 3, 4) -> elastic (n_e,12,12), conduction (n_e,4,4), mass (n_e,4,4)."""
    ne = coords.shape[0]
    A = np.concatenate([np.ones((ne, 4, 1)), np.transpose(coords, (0, 2, 1))], axis=2)
    Ainv = np.linalg.inv(A)                                # rows: [1 x y z] coefficients
    G = np.transpose(Ainv[:, 1:, :], (0, 2, 1))            # (e, 4, 3)
    V = np.abs(np.linalg.det(A)) / 6.0
    B = _strain_operator(G)                                # (e, 6, 12)
    # B^T D B and G G^T as batched matrix products (BLAS), not einsum loops
    Ke = V[:, None, None] * np.matmul(np.transpose(B, (0, 2, 1)),
                                      np.matmul(_elastic_D(nu)[None], B))
    Kh = V[:, None, None] * np.matmul(G, np.transpose(G, (0, 2, 1)))
    M = (V / 20.0)[:, None, None] * (np.ones((4, 4)) + np.eye(4))[None]
    return Ke, Kh, M


def element_matrices(mesh: GridMesh, nu=0.3, shared_if_uniform=True):
    """Unit element matrices; a single shared copy when all cells are translates."""
    coords = np.transpose(mesh.p[:, mesh.t], (2, 0, 1))    # (n_e, 3, nloc)
    if shared_if_uniform and mesh.kind == "hex":
        rel = coords - coords[:, :, :1]
        if np.allclose(rel, rel[:1], rtol=0.0, atol=1e-12):
            Ke, Kh, M = hex_matrices(coords[:1], nu)
            return Ke, Kh, M
    if mesh.kind == "hex":
        return hex_matrices(coords, nu)
    return tet_matrices(coords, nu)


def source_vector(mesh: GridMesh, s: float) -> np.ndarray:
    """Load of a uniform volumetric source: f_a = s * integral of N_a."""
    coords = np.transpose(mesh.p[:, mesh.t], (2, 0, 1))
    if mesh.kind == "hex":
        X, w = _gauss2()
        g, vals = _hex_ref_grads(X)
        detJ = np.linalg.det(np.einsum("eda,qak->eqdk", coords, g))
        fe = s * np.einsum("eq,q,qa->ea", detJ, w, vals)
    else:
        A = np.concatenate([np.ones((coords.shape[0], 4, 1)),
                            np.transpose(coords, (0, 2, 1))], axis=2)
        fe = s * np.repeat((np.abs(np.linalg.det(A)) / 24.0)[:, None], 4, axis=1)
    f = np.zeros(mesh.nnodes)
    for a in range(mesh.t.shape[0]):
        f += np.bincount(mesh.t[a], weights=fe[:, a], minlength=mesh.nnodes)
    return f
