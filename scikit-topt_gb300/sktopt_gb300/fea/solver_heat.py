"""GPU FEM plugin for SIMP steady heat conduction.

Drop-in for ``FEM_SimpLinearHeatConduction`` (sktopt/fea/solver_heat.py:
628-980) for the thermal-compliance objective:

* conductivity k(rho) = kmin + (k0 - kmin) rho^p assembled into the fixed
  scalar pattern (``assemble_conduction_matrix`` composer.py:104-145);
* T = 0 on the Dirichlet nodes (``skfem.enforce``) and the task's volumetric
  load ``emit`` as right-hand side;
* objective J = T^T K T with the operator before enforcement
  (solver_heat.py:785-789; with T = 0 on the fixed nodes it equals
  T^T K_e T);
* element energies 1/2 k |grad T|^2 (solver_heat.py:256-303) and the
  sensitivity dC_drho_simp of them (solver_heat.py:928-950).

The virtual Robin terms and the heat-exchange / averaged-temperature
objectives are not implemented on the GPU.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable

import numpy as np
import torch

from .. import _native as N
from .._device import as_device, default_device, stream_handle, write_back
from . import composer
from .engine import FemEngine, SolveStats
from .solver_elastic import LinearSolverConfig, normalize_linear_solver_config


class FEM_SimpLinearHeatConduction:
    def __init__(self, task, E_min_coeff: float,
                 density_interpolation: Callable = composer.simp_interpolation,
                 solver_config: LinearSolverConfig | None = None,
                 solver_option: str = "spsolve", q: int = 4, device=None):
        self.interp_kind = composer.interpolation_kind(density_interpolation)
        if getattr(task, "objective", "compliance") != "compliance":
            raise NotImplementedError("the GPU heat path implements the compliance objective")
        if float(getattr(task, "dirichlet_values", 0.0)) != 0.0:
            raise NotImplementedError("the GPU heat path supports T = 0 Dirichlet values")
        self.task = task
        self.k_max = task.k * 1.0
        self.k_min = task.k * E_min_coeff
        self.E_max, self.E_min = self.k_max, self.k_min
        self.density_interpolation = density_interpolation
        self.solver_config = solver_config if solver_config is not None else \
            normalize_linear_solver_config(solver_option)
        self.solver_option = self.solver_config.solver
        self.q = q
        self.device = device or default_device()
        self._engine = None
        self._F = None
        self.last_stats: SolveStats | None = None
        self.solve_history: list[SolveStats] = []

    @property
    def engine(self) -> FemEngine:
        if self._engine is None:
            cfg = self.solver_config
            _, Kh, _ = composer.element_matrices(self.task.mesh, 0.3)
            self._engine = FemEngine(self.task.mesh, 1, Kh, self.task.dirichlet_mask,
                                     mixed=(cfg.precision == "mixed"),
                                     multigrid=(cfg.resolved_precond() == "mg"),
                                     mg_levels=cfg.mg_levels, mg_coarse_max=cfg.mg_coarse_max,
                                     device=self.device)
            self._engine.set_interpolation(self.interp_kind)
            self._F = torch.from_numpy(np.ascontiguousarray(self.task.emit)[:, None]).to(
                self.device)
        return self._engine

    def build(self, rho: torch.Tensor, p: float):
        self.engine.update(rho, self.k_max, self.k_min, p)

    def solve_built(self, U: torch.Tensor, force_scale: float = 1.0) -> np.ndarray:
        """Solve K_e T = emit_e; returns J = T^T K T per load case."""
        cfg = self.solver_config
        eng = self.engine
        method = 0 if cfg.precision != "mixed" else \
            {"fcg": 3, "replace": 4, "reliable": 1, "restart": 2}[cfg.refine]
        _, st = eng.solve(self._F, U, method, 1 if eng.multigrid else 0, cfg.resolved_rtol(),
                          cfg.resolved_maxiter(eng.n_dof), cfg.inner_rtol, cfg.max_outer,
                          cfg.cheb_degree, cfg.check_every,
                          cheb_ratio=cfg.cheb_ratio, x0=cfg.warm_start)
        self.last_stats = st
        self.solve_history.append(st)
        KT = eng.spmv(U)
        out = C.c_double()
        lib = N.load()
        N.check(lib.topt_reduce_dot(U.numel(), C.c_void_p(U.data_ptr()),
                                    C.c_void_p(KT.data_ptr()), C.byref(out),
                                    C.c_void_p(stream_handle())))
        return np.array([out.value])

    def solve_device(self, rho, p, U, force_scale=1.0):
        self.build(rho, p)
        return self.solve_built(U, force_scale)

    def objectives_multi_load(self, rho, p: float, u_dofs, timer=None,
                              force_scale: float = 1.0) -> np.ndarray:
        """solver_heat.py:705-895 (compliance objective): solve, write u_dofs."""
        rho_d = as_device(rho, device=self.device)
        if isinstance(u_dofs, torch.Tensor) and u_dofs.is_cuda and u_dofs.is_contiguous() \
                and u_dofs.dtype == torch.float64:
            U = u_dofs.view(-1, 1)
        else:
            U = as_device(u_dofs, device=self.device).reshape(self.engine.n_dof, 1).clone()
        J = self.solve_device(rho_d, p, U)
        write_back(u_dofs, U)
        return J

    def energy_multi_load(self, rho, p: float, u_dofs):
        """solver_heat.py:897-926: 1/2 k |grad T|^2 per element."""
        rho_d = as_device(rho, device=self.device)
        U = as_device(u_dofs, device=self.device)
        if U.dim() == 1:
            U = U[:, None]
        en, _ = self.engine.energy(U, rho_d, self.k_max, self.k_min, p)
        return en if isinstance(rho, torch.Tensor) else en.cpu().numpy()

    def compliance_sensitivity_multi_load(self, rho, p: float, u_dofs):
        """solver_heat.py:928-950: dC_drho_simp(rho, energy, k0, kmin, p)."""
        rho_d = as_device(rho, device=self.device)
        U = as_device(u_dofs, device=self.device)
        if U.dim() == 1:
            U = U[:, None]
        _, dc = self.engine.energy(U, rho_d, self.k_max, self.k_min, p, want_energy=False,
                                   want_dc=True)
        return dc if isinstance(rho, torch.Tensor) else dc.cpu().numpy()

    def sensitivity_multi_load(self, rho, p, U, dh=None, want_energy=True):
        return self.engine.energy(U, rho, self.k_max, self.k_min, p, dh=dh,
                                  want_energy=want_energy, want_dc=True)
