"""GPU FEM plugin for SIMP steady heat conduction.

Drop-in for ``FEM_SimpLinearHeatConduction`` (sktopt/fea/solver_heat.py:
628-980):

* conductivity k(rho) = kmin + (k0 - kmin) rho^p assembled into the fixed
  scalar pattern (``assemble_conduction_matrix`` composer.py:104-145), plus
  the Robin terms of ``solve_multi_load`` (solver_heat.py:198-253): the
  surface terms h u v on the task's Robin facets (task_heat.py:60-139) and,
  when the task has a Robin coefficient, the density-dependent "virtual"
  terms h rho^p (1 - rho)^q |grad rho| u v on the nodal-average density
  (get_robin_virtual solver_heat.py:552-572), all as per-element matrices
  added to the level-0 operator and its Galerkin coarse levels;
* Dirichlet values: every value is one load case with T = value on the
  Dirichlet nodes (``skfem.enforce`` with x = value).  The solve runs on
  T - value (zero on the Dirichlet nodes), its right-hand side lifted by the
  operator before enforcement applied to the constant field: conduction
  annihilates constants, so the unknown is the small deviation from the
  prescribed temperature and the relative residual bounds its error, not
  the error of a ~value-sized field;
* objectives (705-895): compliance T^T K T (K with Robin terms, before
  enforcement); heat exchange J_num / J_den with its adjoint; averaged
  temperature sum(T) with its adjoint; the ``avg_temp_weight`` combination.
  The adjoint right-hand sides depend on the density only, so the adjoint
  columns are solved in the same block solve as the temperatures;
* energies (897-926) and the sensitivity of compliance_sensitivity_multi_load
  (928-980): dC_drho_simp of 1/2 k |grad T|^2 (SIMP form whatever the
  interpolation) plus, for the compliance objective with Robin data, the
  explicit Robin term.

The volume integrals of the Robin and heat-exchange forms use the
quadrature of a basis with intorder 2: the 2x2x2 Gauss rule on hexahedra
(boxes or the trilinear map of any hexahedron), the 4-point degree-2 rule on
P1 tetrahedra; hexahedron faces take 2x2 Gauss on their bilinear map.  Robin facets
are rows (element, axis, side) on hexahedra and (element, local face) on
tetrahedra.  The nodal density average follows the reference's pairing of
``t.ravel()`` with ``np.repeat(rho, nloc)`` (node t[a, e] receives
rho[(a n_elem + e) // nloc]); ``nodal_pairing="element"`` gives node t[a, e]
the density of element e.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable

import numpy as np
import torch

from .. import _native as N
from .._device import as_device, default_device, stream_handle, write_back
from ..mesh.grid import HEX_OFFSETS, TET_FACES, hex_face_local_nodes
from . import composer
from .engine import FemEngine, SolveStats
from .solver_elastic import LinearSolverConfig, normalize_linear_solver_config

_OBJECTIVES = ("compliance", "heat_exchange", "averaged_temp")


def _p(t):
    return C.c_void_p(t.data_ptr())


def _tri_area(mesh, e, loc):
    X = mesh.p[:, mesh.t[loc, e]]
    return 0.5 * float(np.linalg.norm(np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0])))


_G2 = 0.5 / np.sqrt(3.0)
_FACE_PTS = [(0.5 - _G2, 0.5 - _G2), (0.5 - _G2, 0.5 + _G2), (0.5 + _G2, 0.5 - _G2),
             (0.5 + _G2, 0.5 + _G2)]


def _hex_face_rule(mesh, faces):
    """2x2 Gauss rule on the bilinear map of every hexahedron face (rows
    (element, axis, side)): the face's 4 local nodes (nf, 4), the shape values
    at the 4 points (nf, 4 points, 4 nodes) and the weights times the area
    element |dX/ds x dX/dt| (nf, 4).  Exact for the mass forms of planar
    parallelogram faces (axis-aligned cells in particular)."""
    faces = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
    nf = faces.shape[0]
    loc = np.zeros((nf, 4), dtype=np.int64)
    Nq = np.zeros((nf, 4, 4))
    wq = np.zeros((nf, 4))
    for k, (e, axis, side) in enumerate(faces):
        ln = hex_face_local_nodes(int(axis), int(side))
        ax = [d for d in range(3) if d != axis]
        uv = HEX_OFFSETS[ln][:, ax]                                  # (4, 2) in {0, 1}
        X = mesh.p[:, mesh.t[ln, e]]                                 # (3, 4)
        loc[k] = ln
        for q, (su, tv) in enumerate(_FACE_PTS):
            fu = np.where(uv[:, 0] == 1, su, 1.0 - su)
            fv = np.where(uv[:, 1] == 1, tv, 1.0 - tv)
            du = np.where(uv[:, 0] == 1, 1.0, -1.0) * fv
            dv = fu * np.where(uv[:, 1] == 1, 1.0, -1.0)
            Nq[k, q] = fu * fv
            wq[k, q] = 0.25 * np.linalg.norm(np.cross(X @ du, X @ dv))
    return loc, Nq, wq


def surface_robin_matrices(mesh, faces, h):
    """Per-face h * int N_a N_b over one element face (task_heat.py:
    106-134), in the owning element's local numbering.  Hexahedron faces
    (rows (element, axis, side)): 2x2 Gauss on the face's bilinear map (any
    hexahedron); tetrahedron faces (rows (element, local face)): A/12 (1 +
    delta_ab).  Returns (n_faces, nloc^2)."""
    if mesh.kind != "hex":
        out = np.zeros((len(faces), 4, 4))
        for k, (e, f) in enumerate(faces):
            loc = TET_FACES[int(f)]
            a = _tri_area(mesh, int(e), loc)
            for i, ni in enumerate(loc):
                for j, nj in enumerate(loc):
                    out[k, ni, nj] = h * a / 12.0 * (2.0 if i == j else 1.0)
        return out.reshape(len(faces), 16)
    loc, Nq, wq = _hex_face_rule(mesh, faces)
    m = h * np.einsum("kq,kqi,kqj->kij", wq, Nq, Nq)                 # (nf, 4, 4)
    out = np.zeros((len(loc), 8, 8))
    for i in range(4):
        for j in range(4):
            out[np.arange(len(loc)), loc[:, i], loc[:, j]] = m[:, i, j]
    return out.reshape(len(loc), 64)


def surface_robin_load(mesh, faces, h, t_env):
    """h T_env int N_a over the faces (task_heat.py:121-135): 2x2 Gauss on
    the bilinear map of a hexahedron face, a third of the area at each node
    of a triangle."""
    f = np.zeros(mesh.nnodes)
    if mesh.kind != "hex":
        for e, fc in faces:
            loc = TET_FACES[int(fc)]
            np.add.at(f, mesh.t[loc, int(e)], h * t_env * _tri_area(mesh, int(e), loc) / 3.0)
        return f
    faces = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
    loc, Nq, wq = _hex_face_rule(mesh, faces)
    fl = h * t_env * np.einsum("kq,kqi->ki", wq, Nq)                  # (nf, 4)
    nodes = mesh.t[loc, faces[:, 0][:, None]]                        # (nf, 4)
    np.add.at(f, nodes.ravel(), fl.ravel())
    return f


class HeatRobinOps:
    """The ``topt_heat`` handle: Robin element matrices and heat objectives."""

    def __init__(self, mesh, pairing: str = "reference", device=None):
        self.lib = N.load()
        self.device = device or default_device()
        self.mesh = mesh
        t = np.ascontiguousarray(mesh.t, dtype=np.int32)
        p = np.ascontiguousarray(mesh.p, dtype=np.float64)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            N.check(self.lib.topt_heat_create_mesh(mesh.nnodes, mesh.nelements, t.shape[0],
                                                   t.ctypes.data_as(C.c_void_p),
                                                   p.ctypes.data_as(C.c_void_p),
                                                   0 if pairing == "reference" else 1,
                                                   C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.topt_heat_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _bind(self):
        N.check(self.lib.topt_heat_set_stream(self.h, C.c_void_p(stream_handle())))

    def set_surface(self, elems: np.ndarray, mats: np.ndarray):
        self._bind()
        e = np.ascontiguousarray(elems, dtype=np.int32)
        m = np.ascontiguousarray(mats, dtype=np.float64)
        N.check(self.lib.topt_heat_set_surface(self.h, e.size, e.ctypes.data_as(C.c_void_p),
                                               m.ctypes.data_as(C.c_void_p)))

    def nodal_average(self, rho, out):
        self._bind()
        N.check(self.lib.topt_heat_nodal_average(self.h, _p(rho), _p(out)))

    def robin(self, rho_n, h, t_env, p, q, virtual, extra, load):
        self._bind()
        N.check(self.lib.topt_heat_robin(self.h, _p(rho_n) if rho_n is not None else None,
                                         float(h), float(t_env), float(p), float(q),
                                         1 if virtual else 0, _p(extra),
                                         _p(load) if load is not None else None))

    def exchange(self, rho_n, T, h, t_env):
        """(den, num list) of the heat-exchange objective; T None: den only."""
        self._bind()
        L = 0 if T is None else (T.shape[1] if T.dim() == 2 else 1)
        den = C.c_double()
        num = np.zeros(4)
        N.check(self.lib.topt_heat_exchange(self.h, _p(rho_n),
                                            _p(T) if T is not None else None, L, float(h),
                                            float(t_env), C.byref(den),
                                            num.ctypes.data_as(C.c_void_p)))
        return den.value, num[:L]

    def exchange_adjoint(self, rho_n, h, t_env, p, q, den, out):
        self._bind()
        N.check(self.lib.topt_heat_exchange_adjoint(self.h, _p(rho_n), float(h), float(t_env),
                                                    float(p), float(q), float(den), _p(out)))

    def robin_grad(self, rho_n, T, h, t_env, p, q, grad):
        self._bind()
        N.check(self.lib.topt_heat_robin_grad(self.h, _p(rho_n), _p(T), T.shape[1], float(h),
                                              float(t_env), float(p), float(q), _p(grad)))

    def grad_dot(self, X, Y):
        self._bind()
        L = X.shape[1]
        out = torch.empty((self.mesh.nelements, L), dtype=torch.float64, device=self.device)
        N.check(self.lib.topt_heat_grad_dot(self.h, _p(X), _p(Y), L, _p(out)))
        return out


class FEM_SimpLinearHeatConduction:
    def __init__(self, task, E_min_coeff: float,
                 density_interpolation: Callable = composer.simp_interpolation,
                 solver_config: LinearSolverConfig | None = None,
                 solver_option: str = "spsolve", q: int = 4, device=None,
                 nodal_pairing: str = "reference"):
        kind = composer.interpolation_kind(density_interpolation)
        # the heat sensitivity is dC_drho_simp whatever the interpolation
        # (solver_heat.py:940-946): RAMP operator with the SIMP-form derivative
        self.interp_kind = 2 if kind == 1 else 0
        self.objective = getattr(task, "objective", "compliance")
        if self.objective not in _OBJECTIVES:
            raise ValueError(f"Unknown objective: {self.objective}")
        if nodal_pairing not in ("reference", "element"):
            raise ValueError("nodal_pairing must be 'reference' or 'element'")
        self.task = task
        self.k_max = task.k * 1.0
        self.k_min = task.k * E_min_coeff
        self.E_max, self.E_min = self.k_max, self.k_min
        self.density_interpolation = density_interpolation
        self.solver_config = solver_config if solver_config is not None else \
            normalize_linear_solver_config(solver_option)
        self.solver_option = self.solver_config.solver
        self.q = q
        self.nodal_pairing = nodal_pairing
        v = getattr(task, "dirichlet_values", 0.0)
        self.values = [float(x) for x in v] if isinstance(v, (list, tuple)) else [float(v)]
        self.h = getattr(task, "robin_coefficient", None)
        self.t_env = getattr(task, "robin_bc_value", None)
        self.groups = list(getattr(task, "robin_groups", []))
        self.virtual = self.h is not None
        if self.virtual and (isinstance(self.h, (list, tuple)) or
                             isinstance(self.t_env, (list, tuple))):
            raise ValueError("the density-dependent Robin terms take one scalar "
                             "robin_coefficient and robin_bc_value (get_robin_virtual)")
        if self.groups and not self.virtual:
            raise ValueError("Robin facets need robin_coefficient and robin_bc_value")
        self.has_robin = self.virtual
        self.device = device or default_device()
        self._engine = None
        self._ops = None
        self._F = None
        self._X = []
        self.lam = None
        self.λ_all = None
        self.last_stats: SolveStats | None = None
        self.solve_history: list[SolveStats] = []

    # ------------------------------------------------------------ set-up
    @property
    def engine(self) -> FemEngine:
        if self._engine is None:
            self._setup()
        return self._engine

    def _setup(self):
        cfg = self.solver_config
        tsk = self.task
        mesh = tsk.mesh
        dev = self.device
        _, Kh, _ = composer.element_matrices(mesh, 0.3)
        self._engine = FemEngine(mesh, 1, Kh, tsk.dirichlet_mask,
                                 mixed=(cfg.precision == "mixed"),
                                 multigrid=(cfg.resolved_precond() == "mg"),
                                 mg_levels=cfg.mg_levels, mg_coarse_max=cfg.mg_coarse_max,
                                 device=dev)
        self._engine.set_interpolation(self.interp_kind)
        emit = getattr(tsk, "emit", None)
        F = np.zeros(mesh.nnodes) if emit is None else np.array(emit, dtype=np.float64)
        n = mesh.nnodes
        if self.has_robin:
            self._ops = HeatRobinOps(mesh, self.nodal_pairing, device=dev)
            hs = self.h if isinstance(self.h, (list, tuple)) else [self.h] * len(self.groups)
            ts = self.t_env if isinstance(self.t_env, (list, tuple)) else \
                [self.t_env] * len(self.groups)
            elems, mats = [], []
            for faces, h, te in zip(self.groups, hs, ts):
                if len(faces) == 0:
                    continue
                elems.append(faces[:, 0])
                mats.append(surface_robin_matrices(mesh, faces, float(h)))
                F += surface_robin_load(mesh, faces, float(h), float(te))
            if elems:
                self._ops.set_surface(np.concatenate(elems), np.concatenate(mats))
            self._extra = torch.empty(mesh.nelements * 64, dtype=torch.float64, device=dev)
            self._vload = torch.zeros(n, dtype=torch.float64, device=dev)
            self._rho_n = torch.empty(n, dtype=torch.float64, device=dev)
        self._F = torch.from_numpy(F).to(dev)
        self._ones = torch.ones(n, dtype=torch.float64, device=dev)

    # ------------------------------------------------------------ build / solve
    def build(self, rho: torch.Tensor, p: float):
        eng = self.engine
        if self.has_robin:
            self._ops.nodal_average(rho, self._rho_n)
            self._ops.robin(self._rho_n, self.h, self.t_env, p, self.q, True, self._extra,
                            self._vload)
            eng.set_extra(self._extra.view(-1, 8, 8))
        eng.update(rho, self.k_max, self.k_min, p)
        self._p = float(p)

    def _rhs_base(self):
        return self._F + self._vload if self.virtual else self._F

    def _solve_cols(self, cols, values):
        """Solve K_e X = cols with X = value on the Dirichlet nodes, column
        by column value; blocks of up to 4 columns; returns (n, k)."""
        cfg = self.solver_config
        eng = self.engine
        n = eng.n_dof
        lift = any(v != 0.0 for v in values)
        if lift:
            w = eng.spmv(self._ones.view(-1, 1).contiguous(), full=True).view(-1)
        out = torch.empty((n, len(cols)), dtype=torch.float64, device=self.device)
        method = 0 if cfg.precision != "mixed" else \
            {"fcg": 3, "replace": 4, "reliable": 1, "restart": 2}[cfg.refine]
        for c0 in range(0, len(cols), 4):
            idx = list(range(c0, min(c0 + 4, len(cols))))
            Fb = torch.stack([cols[i] - values[i] * w if (lift and values[i] != 0.0)
                              else cols[i] for i in idx], dim=1).contiguous()
            k = c0 // 4
            if len(self._X) <= k or self._X[k].shape != Fb.shape:
                if len(self._X) <= k:
                    self._X.append(torch.zeros_like(Fb))
                else:
                    self._X[k] = torch.zeros_like(Fb)
            X = self._X[k]
            _, st = eng.solve(Fb, X, method, 1 if eng.multigrid else 0, cfg.resolved_rtol(),
                              cfg.resolved_maxiter(n, eng.multigrid), cfg.inner_rtol, cfg.max_outer,
                              cfg.cheb_degree, cfg.check_every, cheb_ratio=cfg.cheb_ratio,
                              x0=cfg.warm_start)
            self.last_stats = st
            self.solve_history.append(st)
            for j, i in enumerate(idx):
                out[:, i] = X[:, j]
                if values[i] != 0.0:
                    out[:, i] += values[i]
        return out

    def _dot(self, x, y) -> float:
        out = C.c_double()
        N.check(N.load().topt_reduce_dot(x.numel(), _p(x), _p(y), C.byref(out),
                                         C.c_void_p(stream_handle())))
        return out.value

    def solve_built(self, U: torch.Tensor, force_scale: float = 1.0) -> np.ndarray:
        """Solve for every Dirichlet value (and the adjoint columns of the
        heat-exchange / averaged-temperature objectives); write the
        temperatures into U (n_nodes, n_loads) and return the objectives."""
        L = len(self.values)
        obj = self.objective
        b = self._rhs_base()
        cols = [b] * L
        vals = list(self.values)
        den = None
        n_adj = 0
        if obj == "heat_exchange":
            if not self.virtual:
                raise RuntimeError("heat_exchange objective requires Robin boundary data.")
            den, _ = self._ops.exchange(self._rho_n, None, self.h, self.t_env)
            if den > 1e-16:
                r = torch.empty_like(b)
                self._ops.exchange_adjoint(self._rho_n, self.h, self.t_env, self._p, self.q,
                                           den, r)
                cols += [r] * L
                vals += list(self.values)
                n_adj = L
                if self.task.avg_temp_weight != 0.0:
                    cols += [self._ones] * L
                    vals += list(self.values)
        elif obj == "averaged_temp":
            cols += [self._ones] * L
            vals += list(self.values)
            n_adj = L
        X = self._solve_cols(cols, vals)
        U.view(-1, L).copy_(X[:, :L])
        T = X[:, :L].contiguous()
        if obj == "compliance":
            full = self.has_robin or any(v != 0.0 for v in self.values)
            J = np.zeros(L)
            for i in range(L):
                t = T[:, i:i + 1].contiguous()
                kt = self.engine.spmv(t, full=full)
                J[i] = self._dot(t.view(-1), kt.view(-1))
            self.lam = None        # -2 T (solver_heat.py:789), formed on demand
        elif obj == "averaged_temp":
            J = np.array([self._dot(T[:, i].contiguous(), self._ones) for i in range(L)])
            self.lam = X[:, L:2 * L].contiguous()
        else:
            if den is None or den <= 1e-16:
                self.lam = torch.zeros_like(T)
                J = np.zeros(L)
            else:
                num = np.concatenate([
                    self._ops.exchange(self._rho_n, T[:, c:c + 4].contiguous(), self.h,
                                       self.t_env)[1] for c in range(0, L, 4)])
                J = num / den
                lam = X[:, L:2 * L].clone()
                w = self.task.avg_temp_weight
                if w != 0.0:
                    avg = np.array([self._dot(T[:, i].contiguous(), self._ones)
                                    for i in range(L)])
                    lam_avg = X[:, 2 * L:3 * L]
                    if L > 1:
                        hs = max(float(np.mean(np.abs(J))), 1e-12)
                        as_ = max(float(np.mean(np.abs(avg))), 1e-12)
                        J = J / hs + w * (avg / as_)
                        lam = lam / hs + (w / as_) * lam_avg
                    else:
                        J = J + w * avg
                        lam = lam + w * lam_avg
                self.lam = lam.contiguous()
        self.λ_all = self.lam
        return J

    def solve_device(self, rho, p, U, force_scale=1.0):
        self.build(rho, p)
        return self.solve_built(U, force_scale)

    # ------------------------------------------------------------ reference API
    def objectives_multi_load(self, rho, p: float, u_dofs, timer=None,
                              force_scale: float = 1.0) -> np.ndarray:
        """solver_heat.py:705-895: solve, write u_dofs, return the objectives."""
        rho_d = as_device(rho, device=self.device)
        L = len(self.values)
        if isinstance(u_dofs, torch.Tensor) and u_dofs.is_cuda and u_dofs.is_contiguous() \
                and u_dofs.dtype == torch.float64:
            U = u_dofs.view(-1, L)
        else:
            U = as_device(u_dofs, device=self.device).reshape(self.engine.n_dof, L).clone()
        J = self.solve_device(rho_d, p, U)
        write_back(u_dofs, U)
        return J

    def _U(self, u_dofs):
        U = as_device(u_dofs, device=self.device)
        if U.dim() == 1:
            U = U[:, None]
        return U.contiguous()

    def energy_multi_load(self, rho, p: float, u_dofs):
        """solver_heat.py:897-926: 1/2 k |grad T|^2 per element (compliance), or
        grad T . grad lam (heat exchange, averaged temperature)."""
        rho_d = as_device(rho, device=self.device)
        U = self._U(u_dofs)
        if self.objective == "compliance":
            en, _ = self.engine.energy(U, rho_d, self.k_max, self.k_min, p)
        else:
            if self.lam is None:
                raise RuntimeError("adjoint field λ_all is not computed.")
            en = self._ops.grad_dot(U, self.lam) if self._ops is not None else \
                self._grad_dot_plain(U, self.lam)
        return en if isinstance(rho, torch.Tensor) else en.cpu().numpy()

    def _grad_dot_plain(self, X, Y):
        if self._ops is None:
            self._ops = HeatRobinOps(self.task.mesh, self.nodal_pairing, device=self.device)
        return self._ops.grad_dot(X, Y)

    def _sensitivity(self, rho_d, p, U, dh, want_energy):
        explicit = self.objective == "compliance" and self.virtual
        en, dc = self.engine.energy(U, rho_d, self.k_max, self.k_min, p,
                                    dh=None if explicit else dh,
                                    want_energy=want_energy and self.objective == "compliance",
                                    want_dc=True)
        if explicit:
            self._ops.nodal_average(rho_d, self._rho_n)
            self._ops.robin_grad(self._rho_n, U, self.h, self.t_env, p, self.q, dc)
            if dh is not None:
                dc.mul_(dh.view(-1, 1))
        if want_energy and self.objective != "compliance":
            if self.lam is None:
                raise RuntimeError("adjoint field λ_all is not computed.")
            en = self._ops.grad_dot(U, self.lam) if self._ops is not None else \
                self._grad_dot_plain(U, self.lam)
        return en, dc

    def compliance_sensitivity_multi_load(self, rho, p: float, u_dofs):
        """solver_heat.py:928-980."""
        rho_d = as_device(rho, device=self.device)
        _, dc = self._sensitivity(rho_d, p, self._U(u_dofs), None, False)
        return dc if isinstance(rho, torch.Tensor) else dc.cpu().numpy()

    def sensitivity_multi_load(self, rho, p, U, dh=None, want_energy=True):
        """(energy, compliance_sensitivity_multi_load * dh) on the device."""
        return self._sensitivity(rho, p, U if U.dim() == 2 else U[:, None], dh, want_energy)
