"""Smoothed-aggregation AMG preconditioner of the reference's ``cg_pyamg``
solver option (TEST INFRASTRUCTURE; see ``oracle/__init__.py``).

The reference builds ``pyamg.smoothed_aggregation_solver(K_cond)`` and runs
SciPy CG with ``ml.aspreconditioner()`` (solver_elastic.py:94-103).  PyAMG is
a third-party dependency pinned at ``pyamg >=5.2.1,<6.0.0``
(pyproject.toml:23) and absent from the reference tree; this module restates
the published algorithm of its SA solver with the 5.x defaults the reference
takes (no keyword arguments are passed):

* strength of connection: symmetric, theta = 0 (every stored entry connects);
* aggregation: "standard" greedy three-pass aggregation (serial, in
  ``csrc/amg.c``);
* near-null-space candidates B = ones, improved at the finest level by four
  symmetric Gauss-Seidel sweeps on A B = 0;
* tentative prolongator T: per aggregate, B restricted to the aggregate and
  normalised (one candidate, so the per-aggregate QR is a normalisation);
  coarse candidates = the norms;
* smoothed prolongator P = (I - omega / rho(D^-1 A) D^-1 A) T, omega = 4/3,
  rho estimated by 15 Arnoldi steps;
* Galerkin coarse operator R A P with R = P^T (symmetric problem);
* levels until n <= max_coarse = 10 or max_levels = 10; coarsest level
  solved with the pseudo-inverse;
* V-cycle with one symmetric Gauss-Seidel sweep (forward then backward)
  before and after the coarse correction; as a preconditioner one V-cycle
  from a zero guess.

Random-vector details of PyAMG's spectral-radius estimate are not restated
(a seeded start vector is used), so hierarchies agree with PyAMG's in
structure and up to that estimate; parity of the solve is on its solution
(the preconditioned CG stops at the same relative residual).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "csrc", "amg.c")
_LIB_DIR = os.path.join(_HERE, "_build")
_LIB = os.path.join(_LIB_DIR, "liboracle_amg.so")
_lib = None


def build_lib(force=False):
    """Compile ``csrc/amg.c`` into ``_build/liboracle_amg.so`` (gcc)."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        os.makedirs(_LIB_DIR, exist_ok=True)
        tmp = _LIB + f".{os.getpid()}.tmp"
        subprocess.check_call(["gcc", "-O2", "-std=c99", "-shared", "-fPIC", "-o", tmp, _SRC])
        os.replace(tmp, _LIB)
    return _LIB


def _c():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build_lib())
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        lib.oracle_standard_aggregation.restype = ctypes.c_int64
        lib.oracle_standard_aggregation.argtypes = [ctypes.c_int64, i64p, i64p, i64p, i64p]
        lib.oracle_gauss_seidel.restype = None
        lib.oracle_gauss_seidel.argtypes = [i64p, i64p, f64p, f64p, f64p, ctypes.c_int64,
                                            ctypes.c_int64, ctypes.c_int64]
        _lib = lib
    return _lib


class _Csr:
    """int64 / float64 CSR arrays of a SciPy matrix for the C kernels."""

    def __init__(self, A):
        A = sp.csr_matrix(A)
        A.sort_indices()
        self.A = A
        self.n = A.shape[0]
        self.p = np.ascontiguousarray(A.indptr, dtype=np.int64)
        self.j = np.ascontiguousarray(A.indices, dtype=np.int64)
        self.x = np.ascontiguousarray(A.data, dtype=np.float64)


def symmetric_strength(A, theta=0.0):
    """Entries with |a_ij|^2 >= theta^2 |a_ii a_jj| (diagonal kept)."""
    A = sp.csr_matrix(A)
    if theta == 0.0:
        return A
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    d = np.abs(A.diagonal())
    keep = (np.abs(A.data) ** 2 >= theta * theta * d[rows] * d[A.indices]) | \
        (rows == A.indices)
    S = sp.csr_matrix((A.data[keep], (rows[keep], A.indices[keep])), shape=A.shape)
    return S


def standard_aggregation(S):
    """Aggregate index of every node (-1: isolated) and the aggregate count."""
    c = _Csr(S)
    agg = np.empty(c.n, dtype=np.int64)
    roots = np.empty(c.n, dtype=np.int64)
    na = _c().oracle_standard_aggregation(c.n, c.p, c.j, agg, roots)
    return agg, int(na)


def gauss_seidel(c: _Csr, x, b, sweep="symmetric", iterations=1):
    """In-place Gauss-Seidel sweeps on A x = b (``c`` from ``_Csr(A)``)."""
    lib = _c()
    for _ in range(iterations):
        if sweep in ("forward", "symmetric"):
            lib.oracle_gauss_seidel(c.p, c.j, c.x, x, b, 0, c.n, 1)
        if sweep in ("backward", "symmetric"):
            lib.oracle_gauss_seidel(c.p, c.j, c.x, x, b, c.n - 1, -1, -1)
    return x


def fit_candidates(agg, n_agg, B):
    """Tentative prolongator for one candidate column: T[i, agg(i)] = B_i /
    ||B restricted to agg(i)||, and the coarse candidates (the norms)."""
    n = agg.size
    ok = agg >= 0
    nrm2 = np.bincount(agg[ok], weights=B[ok] ** 2, minlength=n_agg)
    nrm = np.sqrt(nrm2)
    vals = np.zeros(n)
    vals[ok] = B[ok] / np.where(nrm[agg[ok]] > 0, nrm[agg[ok]], 1.0)
    rows = np.arange(n)[ok]
    T = sp.csr_matrix((vals[ok], (rows, agg[ok])), shape=(n, n_agg))
    return T, nrm


def spectral_radius(A, steps=15, seed=0):
    """Largest |eigenvalue| of the Hessenberg matrix of `steps` Arnoldi steps
    from a seeded random start."""
    n = A.shape[0]
    m = min(steps, n)
    rng = np.random.default_rng(seed)
    V = np.zeros((m + 1, n))
    H = np.zeros((m + 1, m))
    v = rng.random(n)
    V[0] = v / np.linalg.norm(v)
    k_used = m
    for k in range(m):
        w = A @ V[k]
        for i in range(k + 1):
            H[i, k] = np.dot(V[i], w)
            w = w - H[i, k] * V[i]
        H[k + 1, k] = np.linalg.norm(w)
        if H[k + 1, k] < 1e-14:
            k_used = k + 1
            break
        V[k + 1] = w / H[k + 1, k]
    ev = np.linalg.eigvals(H[:k_used, :k_used])
    return float(np.max(np.abs(ev)))


def jacobi_prolongation(A, T, omega=4.0 / 3.0):
    """P = T - omega / rho(D^-1 A) * D^-1 A T."""
    d = A.diagonal()
    dinv = np.where(d != 0.0, 1.0 / np.where(d != 0.0, d, 1.0), 0.0)
    DA = sp.diags(dinv) @ A
    rho = spectral_radius(DA)
    return sp.csr_matrix(T - (omega / rho) * (DA @ T))


class Level:
    def __init__(self, A):
        self.A = sp.csr_matrix(A)
        self.c = _Csr(self.A)
        self.P = None
        self.R = None


class SmoothedAggregationSolver:
    """The hierarchy and V-cycle described in the module docstring."""

    def __init__(self, A, theta=0.0, omega=4.0 / 3.0, max_levels=10, max_coarse=10,
                 improve_iterations=4):
        A = sp.csr_matrix(A, dtype=np.float64)
        self.levels = [Level(A)]
        B = np.ones(A.shape[0])
        while len(self.levels) < max_levels and self.levels[-1].A.shape[0] > max_coarse:
            L = self.levels[-1]
            if len(self.levels) == 1 and improve_iterations:
                B = gauss_seidel(L.c, B.copy(), np.zeros_like(B), "symmetric",
                                 improve_iterations)
            S = symmetric_strength(L.A, theta)
            agg, na = standard_aggregation(S)
            if na == 0 or na >= L.A.shape[0]:
                break
            T, B = fit_candidates(agg, na, B)
            P = jacobi_prolongation(L.A, T, omega)
            L.P = P
            L.R = sp.csr_matrix(P.T)
            self.levels.append(Level(L.R @ L.A @ P))
        last = self.levels[-1]
        self.coarse_pinv = sla.pinv(last.A.toarray())

    def _cycle(self, lvl, x, b):
        L = self.levels[lvl]
        if lvl == len(self.levels) - 1:
            x[:] = self.coarse_pinv @ b
            return x
        gauss_seidel(L.c, x, b, "symmetric", 1)
        r = b - L.A @ x
        bc = L.R @ r
        xc = np.zeros_like(bc)
        self._cycle(lvl + 1, xc, bc)
        x += L.P @ xc
        gauss_seidel(L.c, x, b, "symmetric", 1)
        return x

    def vcycle(self, b):
        """One V-cycle from x = 0 (the preconditioner's application)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        return self._cycle(0, np.zeros_like(b), b)

    def aspreconditioner(self):
        n = self.levels[0].A.shape[0]
        return spla.LinearOperator((n, n), matvec=self.vcycle, dtype=np.float64)

    def operator_complexity(self):
        return sum(L.A.nnz for L in self.levels) / self.levels[0].A.nnz

    def shapes(self):
        return [L.A.shape[0] for L in self.levels]


def cg_pyamg(Ke, Fe, rtol=1e-8, maxiter=None, stats=None):
    """solver_elastic.py:94-103: SA hierarchy of the enforced matrix, one
    V-cycle per CG step as the preconditioner, SciPy CG to ``rtol``."""
    ml = SmoothedAggregationSolver(Ke)
    M = ml.aspreconditioner()
    count = [0]

    def cb(_):
        count[0] += 1
    u, info = spla.cg(Ke, Fe, M=M, rtol=rtol, maxiter=maxiter, callback=cb)
    if stats is not None:
        stats.update(iters=count[0], info=int(info), levels=ml.shapes(),
                     complexity=ml.operator_complexity())
    return u


def sa_transfer_from_aggregates(A, agg, cnt_f, bs, lmax, omega=4.0 / 3.0):
    """The block smoothed-aggregation transfer of the GPU hierarchy, restated
    for checking it: candidates = the bs per-component translations (zero on
    fixed DOFs), tentative T(i, a)_cc = sqrt(cnt_f[i, c] / cnt_c[a, c]),
    P = T - omega / lmax * Dinv A T with the block-diagonal inverse Dinv,
    coarse operator P^T A P with a unit diagonal on empty coarse DOFs.
    ``cnt_f``: free finest-level DOFs below each DOF (1 / 0 at level 0).
    Returns (P, coarse operator, cnt_c)."""
    A = sp.csr_matrix(A)
    n = agg.size
    nc = int(agg.max()) + 1
    cnt_f = np.asarray(cnt_f, dtype=np.int64).reshape(n, bs)
    cnt_c = np.zeros((nc, bs), dtype=np.int64)
    np.add.at(cnt_c, agg, cnt_f)
    w = np.where(cnt_f > 0, np.sqrt(cnt_f / np.maximum(cnt_c[agg], 1)), 0.0)
    rows = (np.arange(n)[:, None] * bs + np.arange(bs)[None, :]).ravel()
    cols = (agg[:, None] * bs + np.arange(bs)[None, :]).ravel()
    T = sp.csr_matrix((w.ravel(), (rows, cols)), shape=(n * bs, nc * bs))
    blocks = np.zeros((n, bs, bs))
    Acoo = A.tocoo()
    same = (Acoo.row // bs) == (Acoo.col // bs)
    blocks[Acoo.row[same] // bs, Acoo.row[same] % bs, Acoo.col[same] % bs] = Acoo.data[same]
    inv = np.zeros_like(blocks)
    for i in range(n):
        if abs(np.linalg.det(blocks[i])) > 0:
            inv[i] = np.linalg.inv(blocks[i])
    Dinv = sp.block_diag([sp.csr_matrix(b) for b in inv], format="csr")
    P = sp.csr_matrix(T - (omega / lmax) * (Dinv @ (A @ T)))
    Ac = (P.T @ A @ P).toarray()
    d = np.diag(Ac).copy()
    d[d == 0.0] = 1.0
    np.fill_diagonal(Ac, d)
    return P, Ac, cnt_c.ravel()
