"""Python handle around the native FEM engine (topt_fem_* in include/topt.h)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from .. import _native as N
from .._device import as_device, default_device, stream_handle
from ..mesh.grid import GridMesh


@dataclass
class SolveStats:
    status: int
    iters: int
    outer: int
    relres: float

    @property
    def status_name(self) -> str:
        return N.STATUS_NAMES.get(self.status, str(self.status))


class FemEngine:
    """Pattern, operator, hierarchy and PCG for one mesh / DOF layout.

    bs = 3 (elasticity) or 1 (conduction).  ``ke`` holds unit-modulus element
    matrices: one shared (1, nd, nd) or one per element (n_e, nd, nd).
    """

    def __init__(self, mesh: GridMesh, bs: int, ke: np.ndarray, dirichlet_mask: np.ndarray,
                 mixed: bool = False, multigrid: bool = True, mg_levels: int = 16,
                 mg_coarse_max: int = 200, device=None, matrix_free: bool = True,
                 amg: bool = True):
        self.lib = N.load()
        self.device = device or default_device()
        self.mesh = mesh
        self.bs = bs
        self.nloc = mesh.t.shape[0]
        self.n_dof = bs * mesh.nnodes
        self.mixed = bool(mixed)
        ke = np.ascontiguousarray(ke, dtype=np.float64)
        if ke.ndim == 2:
            ke = ke[None]
        self._t = np.ascontiguousarray(mesh.t, dtype=np.int32)
        self._ke = ke
        self._mask = np.ascontiguousarray(dirichlet_mask, dtype=np.uint8)
        # meshes without a logical grid (read from files) get a
        # smoothed-aggregation hierarchy built on the GPU (amg) or block Jacobi
        use_amg = bool(multigrid and amg and not getattr(mesh, "has_grid", True))
        multigrid = multigrid and getattr(mesh, "has_grid", True)
        if multigrid:
            self._ijk = np.ascontiguousarray(mesh.node_ijk, dtype=np.int32)
            self._cell = np.ascontiguousarray(mesh.cell_of_elem, dtype=np.int32)
        d = N.FemDesc()
        d.bs = bs
        d.nloc = self.nloc
        d.n_nodes = mesh.nnodes
        d.n_elem = mesh.nelements
        d.t = self._t.ctypes.data_as(C.POINTER(C.c_int32))
        d.ke = ke.ctypes.data_as(C.POINTER(C.c_double))
        d.n_ke = ke.shape[0]
        d.dirichlet = self._mask.ctypes.data_as(C.POINTER(C.c_uint8))
        if multigrid:
            d.grid[:] = list(mesh.shape)
            d.node_ijk = self._ijk.ctypes.data_as(C.POINTER(C.c_int32))
            d.cell_of_elem = (self._cell.ctypes.data_as(C.POINTER(C.c_int32))
                              if mesh.kind != "hex" else None)
        d.mixed = 1 if mixed else 0
        d.mg_levels = mg_levels if (multigrid or use_amg) else 1
        d.amg = 1 if use_amg else 0
        self.amg = use_amg
        d.mg_coarse_max = mg_coarse_max
        d.mf_level0 = 1 if matrix_free else 0
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            N.check(self.lib.topt_fem_create(C.byref(d), C.byref(h)))
        self.h = h
        nd, nnzb, nlev = C.c_int64(), C.c_int64(), C.c_int32()
        N.check(self.lib.topt_fem_sizes(self.h, C.byref(nd), C.byref(nnzb), C.byref(nlev)))
        self.nnzb = nnzb.value
        self.n_levels = nlev.value
        self.multigrid = self.n_levels > 1

    def close(self):
        if getattr(self, "h", None):
            self.lib.topt_fem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _bind(self):
        N.check(self.lib.topt_fem_set_stream(self.h, C.c_void_p(stream_handle())))

    def set_interpolation(self, kind: int):
        """0 SIMP, 1 RAMP, 2 RAMP with the SIMP-form sensitivity, for the
        later update / energy calls."""
        N.check(self.lib.topt_fem_set_interpolation(self.h, int(kind)))

    def set_mf_kernel(self, kind: int):
        """Kernel of the matrix-free FP32 level-0 operator: 0 FP32 FMA tiles
        (default), 1 tensor cores."""
        N.check(self.lib.topt_fem_set_mf_kernel(self.h, int(kind)))

    def set_vcycle_graphs(self, on: bool):
        """Replay the multigrid V-cycle as a CUDA graph (default on) or
        launch its kernels one by one."""
        N.check(self.lib.topt_fem_set_vcycle_graphs(self.h, 1 if on else 0))

    def mf_error(self) -> int:
        out = C.c_int32(0)
        N.check(self.lib.topt_fem_mf_error(self.h, C.byref(out)))
        return out.value

    def set_energy_precision(self, fp32: bool):
        """Element energies / sensitivities in FP32 arithmetic (opt-in) or
        FP64 (the default)."""
        N.check(self.lib.topt_fem_set_energy_precision(self.h, 1 if fp32 else 0))

    # ------------------------------------------------------------ launch shapes
    def set_mf_tile(self, ty: int):
        """Node rows per tile of the FP32-FMA fine-level operator (16, 27,
        32; 0 = the rule)."""
        N.check(self.lib.topt_fem_set_mf_tile(self.h, int(ty)))

    def set_row_mapping(self, level: int, mapping: int):
        """Threads per block row of a level's SELL products (1 warp, 2 three
        threads, 3 one thread; 0 = the rule by level size)."""
        N.check(self.lib.topt_fem_set_row_mapping(self.h, int(level), int(mapping)))

    def tuning(self) -> dict:
        """The launch shapes in use: fine-level tile and per-level mapping."""
        ty = C.c_int32(0)
        maps = np.zeros(self.n_levels, np.int32)
        N.check(self.lib.topt_fem_get_tuning(self.h, C.byref(ty), maps.ctypes.data,
                                             self.n_levels))
        return {"mf_tile": ty.value, "row_mapping": maps.tolist()}

    def spmv_level(self, level: int, x: torch.Tensor, y: torch.Tensor):
        """y = A_level x (one column) in the hierarchy's precision (FP32 for
        mixed engines, FP64 otherwise)."""
        self._bind()
        dt = N.TOPT_F32 if self.mixed else N.TOPT_F64
        N.check(self.lib.topt_fem_spmv_level(self.h, int(level), dt, C.c_void_p(x.data_ptr()),
                                             C.c_void_p(y.data_ptr())))

    def time_spmv_level(self, level: int, x: torch.Tensor, y: torch.Tensor,
                        reps: int = 20) -> float:
        """Device time in microseconds of one ``spmv_level`` product, from
        ``reps`` products replayed as a CUDA graph (no host launch overhead)."""
        self._bind()
        dt = N.TOPT_F32 if self.mixed else N.TOPT_F64
        us = C.c_double(0.0)
        N.check(self.lib.topt_fem_time_spmv_level(self.h, int(level), dt,
                                                  C.c_void_p(x.data_ptr()),
                                                  C.c_void_p(y.data_ptr()), int(reps),
                                                  C.byref(us)))
        return us.value

    def level_sizes(self) -> list:
        """Block rows (nodes) of every level of the hierarchy, and whether the
        level is the dense coarsest one (as (nodes, dense) pairs)."""
        nodes = np.zeros(self.n_levels, np.int64)
        dense = np.zeros(self.n_levels, np.int32)
        N.check(self.lib.topt_fem_level_sizes(self.h, nodes.ctypes.data, dense.ctypes.data,
                                              self.n_levels))
        return [(int(a), bool(b)) for a, b in zip(nodes, dense)]

    def amg_export(self, level: int = 0, dtype: int = 1) -> dict:
        """Host copy of the smoothed-aggregation transfer from `level` to
        level + 1 after an update: aggregates, lambda_max(Dinv A), P (CSR
        blocks) and the coarse operator (dense); dtype 1 FP64, 0 FP32."""
        nf, nc, npb = C.c_int64(), C.c_int64(), C.c_int64()
        N.check(self.lib.topt_fem_amg_sizes(self.h, int(level), C.byref(nf), C.byref(nc),
                                            C.byref(npb)))
        bs = self.bs
        agg = np.zeros(nf.value, np.int32)
        lmax = np.zeros(1)
        p_ptr = np.zeros(nf.value + 1, np.int64)
        p_col = np.zeros(npb.value, np.int32)
        p_vals = np.zeros((npb.value, bs, bs))
        coarse = np.zeros((nc.value * bs, nc.value * bs))
        N.check(self.lib.topt_fem_amg_export(
            self.h, int(dtype), int(level), agg.ctypes.data, lmax.ctypes.data,
            p_ptr.ctypes.data, p_col.ctypes.data, p_vals.ctypes.data, coarse.ctypes.data))
        return {"agg": agg, "lmax": float(lmax[0]), "p_ptr": p_ptr, "p_col": p_col,
                "p_vals": p_vals, "coarse": coarse, "n_coarse": nc.value}

    def set_extra(self, extra: torch.Tensor | None):
        """Per-element matrices (n_e, nd, nd) added to the level-0 operator
        from the next update on; the tensor must stay alive (None removes)."""
        if extra is not None:
            assert extra.is_cuda and extra.dtype == torch.float64 and extra.is_contiguous()
        self._extra = extra
        N.check(self.lib.topt_fem_set_element_extra(
            self.h, C.c_void_p(extra.data_ptr()) if extra is not None else None))

    def update(self, rho: torch.Tensor, E0: float, Emin: float, p: float):
        """coef = SIMP(rho); K = sum coef Ke; enforce; refresh the preconditioner."""
        self._bind()
        rho = as_device(rho, device=self.device)
        N.check(self.lib.topt_fem_update(self.h, C.c_void_p(rho.data_ptr()), float(E0),
                                         float(Emin), float(p)))

    def solve(self, F: torch.Tensor, U: torch.Tensor, method: int, precond: int, rtol: float,
              maxiter: int, inner_rtol: float = 1e-4, max_outer: int = 20,
              cheb_degree: int = 2, check_every: int = 1, raise_on_maxiter=False,
              cheb_ratio: float = 30.0, x0: bool = False):
        """Solve K_e U = F_e for every column; returns (compliance, SolveStats).
        With x0 the solve starts from the U passed in (fixed DOFs zeroed)."""
        self._bind()
        L = F.shape[1] if F.dim() == 2 else 1
        o = N.SolveOpts(method=method, precond=precond, rtol=rtol, maxiter=maxiter,
                        inner_rtol=inner_rtol, max_outer=max_outer,
                        cheb_degree=cheb_degree, check_every=check_every,
                        cheb_ratio=cheb_ratio, x0=1 if x0 else 0)
        info = N.SolveInfo()
        comp = np.zeros(L)
        N.check(self.lib.topt_fem_solve(self.h, C.c_void_p(F.data_ptr()),
                                        C.c_void_p(U.data_ptr()), L, C.byref(o),
                                        C.byref(info), comp.ctypes.data_as(C.c_void_p)))
        st = SolveStats(info.status, info.iters, info.outer, info.relres)
        if info.status == N.TOPT_NONFINITE or (raise_on_maxiter and info.status != N.TOPT_OK):
            raise N.ToptError(info.status, f"linear solve failed: {st}")
        return comp, st

    def spmv(self, x: torch.Tensor, dtype=torch.float64, full: bool = False) -> torch.Tensor:
        """y = K x with the enforced operator, or (full) the FP64 operator
        before Dirichlet enforcement."""
        self._bind()
        L = x.shape[1] if x.dim() == 2 else 1
        y = torch.empty_like(x)
        code = N.TOPT_F64_FULL if full else \
            (N.TOPT_F64 if dtype == torch.float64 else N.TOPT_F32)
        N.check(self.lib.topt_fem_spmv(self.h, code, C.c_void_p(x.data_ptr()),
                                       C.c_void_p(y.data_ptr()), L))
        return y

    def export_values(self) -> torch.Tensor:
        self._bind()
        v = torch.empty(self.nnzb * self.bs * self.bs, dtype=torch.float64, device=self.device)
        N.check(self.lib.topt_fem_export_values(self.h, C.c_void_p(v.data_ptr())))
        return v

    def energy(self, U: torch.Tensor, rho: torch.Tensor, E0, Emin, p, dh=None,
               want_energy=True, want_dc=False):
        """Element energies (n_e, L) and dC_drho_simp * dh (n_e, L)."""
        self._bind()
        L = U.shape[1] if U.dim() == 2 else 1
        ne = self.mesh.nelements
        en = torch.empty((ne, L), dtype=torch.float64, device=self.device) if want_energy else None
        dc = torch.empty((ne, L), dtype=torch.float64, device=self.device) if want_dc else None
        N.check(self.lib.topt_fem_energy(
            self.h, C.c_void_p(U.data_ptr()), L, C.c_void_p(rho.data_ptr()), float(E0),
            float(Emin), float(p), C.c_void_p(dh.data_ptr()) if dh is not None else None,
            C.c_void_p(en.data_ptr()) if en is not None else None,
            C.c_void_p(dc.data_ptr()) if dc is not None else None))
        return en, dc


def pattern(mesh: GridMesh):
    """Host pattern (rowptr, colind, cptr, contrib) of a mesh, via the native builder."""
    lib = N.load()
    t = np.ascontiguousarray(mesh.t, dtype=np.int32)
    h = C.c_void_p()
    N.check(lib.topt_pattern_build(mesh.nnodes, mesh.nelements, t.shape[0],
                                   t.ctypes.data_as(C.c_void_p), C.byref(h)))
    try:
        nnzb, nc = C.c_int64(), C.c_int64()
        N.check(lib.topt_pattern_sizes(h, C.byref(nnzb), C.byref(nc)))
        rowptr = np.empty(mesh.nnodes + 1, np.int32)
        colind = np.empty(nnzb.value, np.int32)
        cptr = np.empty(nnzb.value + 1, np.int64)
        contrib = np.empty(nc.value, np.int32)
        N.check(lib.topt_pattern_export(h, rowptr.ctypes.data_as(C.c_void_p),
                                        colind.ctypes.data_as(C.c_void_p),
                                        cptr.ctypes.data_as(C.c_void_p),
                                        contrib.ctypes.data_as(C.c_void_p)))
    finally:
        lib.topt_pattern_free(h)
    return rowptr, colind, cptr, contrib


def block_to_scalar_csr(rowptr, colind, vals, bs):
    """Scalar CSR (indptr, indices, data) with interleaved DOFs bs*node + comp
    from a node pattern and its (nnzb, bs, bs) block values."""
    rowptr = np.asarray(rowptr, np.int64)
    colind = np.asarray(colind, np.int64)
    nnzb = colind.size
    n = rowptr.size - 1
    brow = np.repeat(np.arange(n), np.diff(rowptr))
    k, c, d = np.meshgrid(np.arange(nnzb), np.arange(bs), np.arange(bs), indexing="ij")
    k, c, d = k.ravel(), c.ravel(), d.ravel()
    order = np.lexsort((d, k, brow[k] * bs + c))
    k, c, d = k[order], c[order], d[order]
    indices = bs * colind[k] + d
    data = np.asarray(vals).reshape(nnzb, bs, bs)[k, c, d]
    counts = np.repeat(np.diff(rowptr) * bs, bs)
    indptr = np.zeros(n * bs + 1, np.int64)
    indptr[1:] = np.cumsum(counts)
    return indptr, indices, data
