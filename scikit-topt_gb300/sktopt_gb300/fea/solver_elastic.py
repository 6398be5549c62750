"""GPU FEM plugin for SIMP linear elasticity.

Drop-in for ``FEM_SimpLinearElasticity`` (sktopt/fea/solver_elastic.py:540-676)
with the same constructor and ``objectives_multi_load`` /
``energy_multi_load`` methods.  ``LinearSolverConfig`` keeps the reference
fields (solver_elastic.py:34-40) and adds the GPU choices:

* ``precision``: "fp64" (plain FP64 PCG) or "mixed" (FP32 operator, FP32
  multigrid and FP32 inner work; FP64 residual, solution update and dots).
  ``refine`` picks the refinement scheme: "replace" (default) is a flexible
  CG preconditioned by one FP32 V-cycle, with FP32 recurrences and operator
  and the solution accumulated in FP64; the FP64 residual Fe - K U replaces
  the recursive one whenever that has dropped by ``inner_rtol`` and before
  convergence is declared.  "fcg" is an FP64 flexible CG (FP64 operator in
  every iteration) around the same V-cycle; "reliable" runs the CG
  recurrences in FP32
  and replaces the FP32 residual by the FP64 one whenever it has dropped by
  ``inner_rtol``; "restart" restarts an FP32 PCG to ``inner_rtol`` for every
  FP64 refinement step.
* ``warm_start``: each solve starts from the ``U`` it is given (the previous
  solution in the optimisation loop) instead of zero; convergence is still
  ``||Fe - K U|| <= rtol ||Fe||``, so the accepted solutions meet the
  reference's tolerance (the reference's SciPy CG starts from zero).
* ``precond``: "mg" (multigrid V-cycle on the logical grid) or "jacobi"
  (3x3 block Jacobi; what the reference's ``cg_jacobi`` uses as scalar Jacobi).

Solver names map onto the GPU PCG: "cg_jacobi" -> block Jacobi; "cg_pyamg",
"petsc" and "auto" -> multigrid; "spsolve" / "petsc_spdirect" (direct in the
reference) -> multigrid PCG driven to ``direct_rtol`` (1e-12 by default).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Literal

import numpy as np
import torch

from .. import _native as N
from .._device import as_device, default_device, write_back
from . import composer
from .engine import FemEngine, SolveStats

SolverSelector = Literal["auto", "cg_jacobi", "spsolve", "cg_pyamg", "petsc",
                         "petsc_spdirect"]


@dataclass(frozen=True)
class LinearSolverConfig:
    solver: SolverSelector = "spsolve"
    rtol: float = 1e-8
    maxiter: int | None = None
    petsc_options: object | None = None
    allow_fallback_to_spsolve: bool = False
    precision: Literal["fp64", "mixed"] = "fp64"
    precond: Literal["mg", "jacobi", "auto"] = "auto"
    refine: Literal["fcg", "replace", "reliable", "restart"] = "replace"
    inner_rtol: float = 1e-1
    max_outer: int = 30
    cheb_degree: int = 2
    cheb_ratio: float = 30.0       # smoother interval [lambda_max / ratio, lambda_max]
    # start each solve from the U passed in (the previous design's solution in
    # the optimisation loop) instead of 0; the stopping rule is unchanged
    warm_start: bool = True
    check_every: int = 1
    direct_rtol: float = 1e-12
    mg_levels: int = 16
    mg_coarse_max: int = 200
    # launch shapes (fine-level tile, SELL row mappings) timed on the device
    # once per problem shape by core.autotune; False keeps the size rules
    autotune: bool = False

    def resolved_precond(self) -> str:
        if self.precond != "auto":
            return self.precond
        return "jacobi" if self.solver == "cg_jacobi" else "mg"

    def resolved_rtol(self) -> float:
        if self.solver in ("spsolve", "petsc_spdirect"):
            return min(self.rtol, self.direct_rtol)
        return self.rtol

    def resolved_maxiter(self, n_dof: int, multigrid: bool = True) -> int:
        """``multigrid`` False: the engine runs block Jacobi (a mesh without
        a logical grid) whatever the configured preconditioner."""
        if self.maxiter is not None:
            return int(self.maxiter)
        if self.resolved_precond() == "jacobi" or not multigrid:
            # solver_elastic.py:201-204 rule, kept for the Jacobi-preconditioned path
            return min(1000, max(300, n_dof // 5)) if self.solver == "cg_jacobi" else 20000
        return 2000


def normalize_linear_solver_config(solver="spsolve", rtol=1e-8, maxiter=None,
                                   petsc_options=None, allow_fallback_to_spsolve=False,
                                   **gpu):
    """solver_elastic.py:43-58."""
    if isinstance(solver, LinearSolverConfig):
        return solver
    return LinearSolverConfig(solver=solver, rtol=rtol, maxiter=maxiter,
                              petsc_options=petsc_options,
                              allow_fallback_to_spsolve=allow_fallback_to_spsolve, **gpu)


class FEM_SimpLinearElasticity:
    """GPU state solve, compliance, energies and sensitivities (SIMP or RAMP)."""

    def __init__(self, task, E_min_coeff: float,
                 density_interpolation: Callable = composer.simp_interpolation,
                 solver_config: LinearSolverConfig | None = None,
                 solver_option: SolverSelector = "spsolve", petsc_options=None,
                 device=None):
        self.interp_kind = composer.interpolation_kind(density_interpolation)
        self.task = task
        self.E_max = task.E * 1.0
        self.E_min = task.E * E_min_coeff
        self.density_interpolation = density_interpolation
        self.solver_config = solver_config if solver_config is not None else \
            normalize_linear_solver_config(solver_option, petsc_options=petsc_options)
        self.solver_option = self.solver_config.solver
        self.device = device or default_device()
        self._engine: FemEngine | None = None
        self._F = None
        self._U = None
        self._rho_built = None
        self._p_built = None
        self.last_stats: SolveStats | None = None
        self.solve_history: list[SolveStats] = []

    # ------------------------------------------------------------------ set-up
    @property
    def engine(self) -> FemEngine:
        if self._engine is None:
            cfg = self.solver_config
            Ke, _, _ = composer.element_matrices(self.task.mesh, self.task.nu)
            self._engine = FemEngine(
                self.task.mesh, 3, Ke, self.task.dirichlet_mask,
                mixed=(cfg.precision == "mixed"),
                multigrid=(cfg.resolved_precond() == "mg"),
                mg_levels=cfg.mg_levels, mg_coarse_max=cfg.mg_coarse_max,
                device=self.device)
            self._engine.set_interpolation(self.interp_kind)
            F = np.column_stack(self.task.neumann_linear)
            self._F = torch.from_numpy(np.ascontiguousarray(F)).to(self.device)
        return self._engine

    def forces(self, force_scale: float = 1.0) -> torch.Tensor:
        self.engine
        return self._F if force_scale == 1.0 else self._F * force_scale

    def build(self, rho: torch.Tensor, p: float):
        """Assemble K(rho) and refresh the preconditioner."""
        self.engine.update(rho, self.E_max, self.E_min, p)
        if self.solver_config.autotune and not getattr(self, "_tuned", False):
            from ..core import autotune
            self.tuning = autotune.tune(self.engine)
            self._tuned = True
        self._rho_built = rho
        self._p_built = p

    # ------------------------------------------------------------------ plugin API
    def solve_device(self, rho: torch.Tensor, p: float, U: torch.Tensor,
                     force_scale: float = 1.0) -> np.ndarray:
        """Device-resident state solve; U (n_dof, L) is overwritten."""
        self.build(rho, p)
        return self.solve_built(U, force_scale)

    def solve_built(self, U: torch.Tensor, force_scale: float = 1.0) -> np.ndarray:
        """Solve with the operator of the last ``build``."""
        cfg = self.solver_config
        eng = self.engine
        F = self.forces(force_scale)
        method = 0 if cfg.precision != "mixed" else \
            {"fcg": 3, "replace": 4, "reliable": 1, "restart": 2}[cfg.refine]
        precond = 1 if eng.multigrid else 0
        comp, st = eng.solve(F, U, method, precond, cfg.resolved_rtol(),
                             cfg.resolved_maxiter(eng.n_dof, eng.multigrid), cfg.inner_rtol,
                             cfg.max_outer,
                             cfg.cheb_degree, cfg.check_every,
                             cheb_ratio=cfg.cheb_ratio, x0=cfg.warm_start)
        self.last_stats = st
        self.solve_history.append(st)
        return comp

    def objectives_multi_load(self, rho, p: float, u_dofs, timer=None,
                              force_scale: float = 1.0) -> np.ndarray:
        """solver_elastic.py:643-666: solve every load case, write u_dofs in place,
        return the compliance F_e . u of each load."""
        rho_d = as_device(rho, device=self.device)
        L = len(self.task.neumann_linear)
        if isinstance(u_dofs, torch.Tensor) and u_dofs.is_cuda and u_dofs.is_contiguous() \
                and u_dofs.dtype == torch.float64:
            U = u_dofs.view(-1, L)
        else:
            U = as_device(u_dofs, device=self.device).reshape(self.engine.n_dof, L).clone()
        comp = self.solve_device(rho_d, p, U, force_scale)
        write_back(u_dofs, U)
        return comp

    def energy_multi_load(self, rho, p: float, u_dofs) -> np.ndarray | torch.Tensor:
        """solver_elastic.py:668-676: element strain energy 1/2 u_e^T K_e(rho) u_e."""
        rho_d = as_device(rho, device=self.device)
        U = as_device(u_dofs, device=self.device)
        if U.dim() == 1:
            U = U[:, None]
        en, _ = self.engine.energy(U, rho_d, self.E_max, self.E_min, p)
        return en if isinstance(rho, torch.Tensor) else en.cpu().numpy()

    def sensitivity_multi_load(self, rho: torch.Tensor, p: float, U: torch.Tensor,
                               dh: torch.Tensor | None = None, want_energy=True):
        """Fused energy + dC_drho_simp(rho, energy) * dh (derivatives.py:42-52)."""
        return self.engine.energy(U, rho, self.E_max, self.E_min, p, dh=dh,
                                  want_energy=want_energy, want_dc=True)
