"""Density-method driver with GPU-resident state.

Drop-in for ``DensityMethod`` (sktopt/core/optimizers/common_density.py:
467-1265): the same config dataclasses, ``parameterize`` / ``optimize`` /
``optimize_steps``, the same per-iteration order (schedules -> filter ->
projection -> state solve -> energies -> sensitivity chain -> filter
transpose -> ``rho_update`` -> masks -> metrics) and the same history series.
Densities, sensitivities and displacements stay in device memory for the
whole run; only scalars (schedules, compliance, bisection results, metrics)
cross to the host each iteration.
"""
from __future__ import annotations

import inspect
import json
import os
from dataclasses import asdict, dataclass, field
from typing import Literal

import numpy as np
import torch

from ... import tools
from ..._device import default_device
from ...fea import composer
from ...fea.solver_elastic import (FEM_SimpLinearElasticity, LinearSolverConfig,
                                   normalize_linear_solver_config)
from ...filters.spacial import SpacialFilter
from ...mesh.task import LinearElasticity, LinearHeatConduction
from ...tools.timer import PhaseTimer
from ..projection import heaviside_projection_device


@dataclass
class DensityState:
    rho: torch.Tensor
    rho_prev: torch.Tensor
    rho_filtered: torch.Tensor
    rho_projected: torch.Tensor
    dH_drho: torch.Tensor
    dC_drho_full: torch.Tensor
    energy_mean: torch.Tensor
    scaling_rate: torch.Tensor
    u_dofs: torch.Tensor
    filter_radius: float
    elements_volume_design: torch.Tensor
    elements_volume_design_sum: float
    iter_begin: int
    iter_end: int
    last_iter: int | None = None
    compliance: float | None = None
    u_max: float | np.ndarray | None = None
    rho_change_max: float | None = None
    kkt_residual: float | None = None
    vol_error: float | None = None


@dataclass
class DensityMethodConfig:
    """Same fields and defaults as common_density.py:62-345, plus GPU options."""
    dst_path: str = "./result/pytests"
    interpolation: Literal["SIMP", "RAMP"] = "SIMP"
    record_times: int = 20
    max_iters: int = 200
    beta_eta: float = 0.50
    eta: float = 0.6
    p: tools.SchedulerConfig = field(default_factory=lambda: tools.SchedulerConfig.step(
        init_value=1.0, target_value=3.0, num_steps=3))
    vol_frac: tools.SchedulerConfig = field(
        default_factory=lambda: tools.SchedulerConfig.constant(target_value=0.8))
    beta: tools.SchedulerConfig = field(
        default_factory=lambda: tools.SchedulerConfig.step_accelerating(
            init_value=1.0, target_value=2.0, num_steps=3, curvature=2.0))
    neumann_scale: tools.SchedulerConfig = field(
        default_factory=lambda: tools.SchedulerConfig.constant_one(name="neumann_scale"))
    filter_type: Literal["spacial", "helmholtz"] = "helmholtz"
    filter_radius: tools.SchedulerConfig = field(
        default_factory=lambda: tools.SchedulerConfig.constant(target_value=0.01))
    E_min_coeff: float = 1e-3
    rho_min: float = 1e-2
    rho_max: float = 1.0
    restart: bool = False
    restart_from: int = -1
    export_img: bool = False
    export_img_opaque: bool = False
    design_dirichlet: bool = False
    sensitivity_filter: bool = False
    solver_option: Literal["spsolve", "cg_pyamg", "cg_jacobi", "petsc",
                           "petsc_spdirect"] = "spsolve"
    petsc_options: object = None
    scaling: bool = False
    check_convergence: bool = False
    tol_rho_change: float = 2e-1
    tol_kkt_residual: float = 5e-3
    # GPU options
    precision: Literal["fp64", "mixed"] = "fp64"
    precond: Literal["mg", "jacobi", "auto"] = "auto"
    solver_rtol: float = 1e-8
    # mixed solves: FP64 residual replacement after the FP32 recursive residual
    # has dropped by this factor.  The loop's solves start from the previous
    # design's solution, where 0.05 saves replacements at no extra iterations
    # (a solve from zero prefers 0.1, the solver's own default)
    inner_rtol: float = 5e-2
    # time the engine's launch shapes once per problem shape (core.autotune)
    autotune: bool = False
    # OC bisection: FP32 evaluation of each step, FP64 only near a decision
    # edge (same result as the all-FP64 bisection); False = FP64 every step
    bisection_fp32_bracket: bool = True
    export: bool = False
    # with export: the VTU of each saved iteration (mesh_rho/info_mesh-*.vtu)
    # and cubic_top.vtu at the end, as the reference writes them
    export_vtu: bool = True

    @classmethod
    def from_defaults(cls, **args):
        keys = inspect.signature(cls).parameters.keys()
        return cls(**{k: v for k, v in args.items() if k in keys})

    def __post_init__(self):
        self.solver_config = normalize_linear_solver_config(
            self.solver_option, rtol=self.solver_rtol, precision=self.precision,
            precond=self.precond, inner_rtol=self.inner_rtol, autotune=self.autotune)

    def vtu_path(self, iter_num: int):
        """common_density.py:338-339."""
        return f"{self.dst_path}/mesh_rho/info_mesh-{iter_num:08d}.vtu"

    def export_cfg(self, path: str):
        d = {k: (asdict(v) if hasattr(v, "__dataclass_fields__") else v)
             for k, v in self.__dict__.items() if k not in ("solver_config", "petsc_options")}
        with open(f"{path}/cfg.json", "w") as f:
            json.dump(d, f, indent=2, default=str)


@dataclass
class DensityMethod_OC_Config(DensityMethodConfig):
    """common_density.py:348-389."""
    lambda_lower: float = 1e-7
    lambda_upper: float = 1e+7
    percentile: tools.SchedulerConfig = field(
        default_factory=lambda: tools.SchedulerConfig.none())
    move_limit: tools.SchedulerConfig = field(
        default_factory=lambda: tools.SchedulerConfig.sawtooth_decay("move_limit", 0.3, 0.1, 3))


class DensityMethod:
    def __init__(self, cfg: DensityMethodConfig, tsk, device=None):
        if cfg.interpolation not in ("SIMP", "RAMP"):
            raise ValueError("Interpolation method must be SIMP or RAMP.")
        if cfg.scaling:
            raise NotImplementedError("length/force scaling is not supported")
        self.cfg = cfg
        self.tsk = tsk
        self.device = device or default_device()
        if cfg.export:
            os.makedirs(cfg.dst_path, exist_ok=True)
            os.makedirs(f"{cfg.dst_path}/data", exist_ok=True)
            os.makedirs(f"{cfg.dst_path}/mesh_rho", exist_ok=True)
            cfg.export_cfg(cfg.dst_path)
        self._snap = None
        if cfg.design_dirichlet is False:
            tsk.exlude_dirichlet_from_design()
        # common_density.py:392-404 (interpolation_funcs)
        interp = composer.ramp_interpolation if cfg.interpolation == "RAMP" else \
            composer.simp_interpolation
        if isinstance(tsk, LinearElasticity):
            self.fem = FEM_SimpLinearElasticity(tsk, cfg.E_min_coeff,
                                                density_interpolation=interp,
                                                solver_config=cfg.solver_config,
                                                device=self.device)
        elif isinstance(tsk, LinearHeatConduction):
            from ...fea.solver_heat import FEM_SimpLinearHeatConduction
            self.fem = FEM_SimpLinearHeatConduction(tsk, cfg.E_min_coeff,
                                                    density_interpolation=interp,
                                                    solver_config=cfg.solver_config,
                                                    device=self.device)
        else:
            raise NotImplementedError("task must be LinearElasticity or LinearHeatConduction")
        self.schedulers = tools.Schedulers(cfg.dst_path)
        self._schedulers_initialized = False
        dev = self.device
        self.design = torch.from_numpy(np.asarray(tsk.design_elements, np.int64)).to(dev)
        vd = np.asarray(tsk.elements_volume, np.float64)[tsk.design_elements]
        self._vol_design = torch.from_numpy(np.ascontiguousarray(vd)).to(dev)
        self._vol_design_sum = float(np.sum(vd))
        self._dV_drho_design = self._vol_design / self._vol_design_sum
        self.kkt_residual = None
        self._state: DensityState | None = None
        self._iter_next = None
        self._completed = False
        self.recorder = self.add_recorder(tsk)
        self.filter = None
        self.timer = PhaseTimer()

    # ------------------------------------------------------------------ set-up
    def add_recorder(self, tsk):
        """common_density.py:591-611; the objective history is named after a
        heat task's objective (_objective_history_name 613-616)."""
        self.objective_name = str(getattr(tsk, "objective", "compliance")) \
            if isinstance(tsk, LinearHeatConduction) else "compliance"
        r = tools.HistoryCollection(self.cfg.dst_path)
        for k in ("rho_projected", "energy", "vol_error", "u_max", self.objective_name,
                  "scaling_rate", "neumann_scale", "rho_change_max", "kkt_residual"):
            r.add(k)
        return r

    def init_schedulers(self, export: bool = False):
        cfg = self.cfg
        S = self.schedulers
        for name in ("p", "vol_frac", "move_limit", "beta", "percentile", "filter_radius"):
            S.add_object_from_config(getattr(cfg, name), name)
        allowed = {"ConstantOne", "StepToOne", "StepAcceleratingToOne", "StepDeceleratingToOne"}
        if cfg.neumann_scale.scheduler_type not in allowed:
            raise ValueError(f"neumann_scale must use one of {allowed}")
        S.add_object_from_config(cfg.neumann_scale, "neumann_scale")
        if isinstance(cfg.eta, tools.SchedulerConfig):
            S.add_object_from_config(cfg.eta, "eta")
        else:
            S.add("eta", cfg.eta, cfg.eta, -1, cfg.max_iters)
        S.set_iters_max(cfg.max_iters)
        self._schedulers_initialized = True

    def parameterize(self):
        """common_density.py:681-703."""
        tsk = self.tsk
        r0 = self.cfg.filter_radius.init_value
        if self.cfg.filter_type == "spacial":
            self.filter = SpacialFilter.from_defaults(tsk.mesh, tsk.elements_volume, r0,
                                                      design_mask=tsk.design_mask,
                                                      device=self.device)
        elif self.cfg.filter_type == "helmholtz":
            from ...filters.helmholtz_filter_nodal import HelmholtzFilterNodal
            self.filter = HelmholtzFilterNodal.from_defaults(tsk.mesh, tsk.elements_volume, r0,
                                                             design_mask=tsk.design_mask,
                                                             device=self.device)
        else:
            raise ValueError("should be spacial or helmholtz")

    def initialize_density(self):
        """common_density.py:711-745 (restart from data/NNNNNN-rho.npz supported)."""
        tsk, cfg = self.tsk, self.cfg
        vi = cfg.vol_frac.init_value if cfg.vol_frac.init_value is not None \
            else cfg.vol_frac.target_value
        rho = np.zeros(tsk.mesh.nelements, dtype=np.float64)
        iter_begin = 1
        if cfg.restart:
            from ..misc import find_latest_iter_file
            if cfg.restart_from > 0:
                path = f"{cfg.dst_path}/data/{cfg.restart_from:06d}-rho.npz"
                iter_begin = cfg.restart_from + 1
            else:
                it, path = find_latest_iter_file(f"{cfg.dst_path}/data")
                iter_begin = it + 1
            rho[tsk.design_elements] = np.load(path)["rho_design_elements"]
            self.recorder.import_histories()
        else:
            rho += vi
            np.clip(rho, cfg.rho_min, cfg.rho_max, out=rho)
        if cfg.design_dirichlet:
            rho[tsk.neumann_elements] = 1.0
        else:
            rho[tsk.dirichlet_neumann_elements] = 1.0
        rho[tsk.fixed_elements] = 1.0
        return rho, iter_begin, cfg.max_iters + 1

    def _ensure_state_initialized(self):
        if self._completed:
            return False
        if not self._schedulers_initialized:
            self.init_schedulers()
        if self.filter is None:
            self.parameterize()
        if self._state is None:
            rho, ib, ie = self.initialize_density()
            dev = self.device
            r = torch.from_numpy(rho).to(dev)
            z = lambda: torch.zeros_like(r)  # noqa: E731
            nd = self.design.numel()
            fr = self.cfg.filter_radius.init_value \
                if isinstance(self.cfg.filter_radius.num_steps, (int, float)) \
                else self.cfg.filter_radius.target_value
            self.filter.update_radius(fr)
            self._state = DensityState(
                rho=r, rho_prev=z(), rho_filtered=z(), rho_projected=z(), dH_drho=z(),
                dC_drho_full=z(), energy_mean=z(),
                scaling_rate=torch.zeros(nd, dtype=torch.float64, device=dev),
                u_dofs=torch.zeros((self.tsk.n_dof, self.tsk.n_tasks), dtype=torch.float64,
                                   device=dev),
                filter_radius=fr, elements_volume_design=self._vol_design,
                elements_volume_design_sum=self._vol_design_sum, iter_begin=ib, iter_end=ie)
            self._iter_next = ib
        return True

    # ------------------------------------------------------------------ loop
    def optimize(self):
        self._optimize_impl()

    def optimize_steps(self, num_steps: int):
        if num_steps <= 0:
            return
        self._optimize_impl(num_steps)

    def _optimize_impl(self, max_steps: int | None = None):
        if not self._ensure_state_initialized():
            return
        st = self._state
        it0 = self._iter_next
        if it0 >= st.iter_end:
            self._finalize()
            return
        it1 = st.iter_end if max_steps is None else min(it0 + max_steps, st.iter_end)
        try:
            self._run_steps(it0, it1)
        finally:
            if self._snap is not None:
                self._snap.flush()
        if self._iter_next >= st.iter_end:
            self._finalize()

    def _run_steps(self, it0, it1):
        for it in range(it0, it1):
            converged = self.step(it)
            self._iter_next = it + 1
            if converged:
                break

    def scheduled_values(self, it):
        return self.schedulers.values_as_list(
            it, ["neumann_scale", "p", "vol_frac", "beta", "move_limit", "eta", "percentile",
                 "filter_radius"])

    def step(self, iter_num: int) -> bool:
        """One iteration of common_density.py:1014-1238."""
        cfg, tsk, st = self.cfg, self.tsk, self._state
        (nscale, p, vol_frac, beta, move_limit, eta, percentile,
         radius) = self.scheduled_values(iter_num)
        st.last_iter = iter_num
        if radius != self.filter.radius:
            self.filter.update_radius(radius)
        T = self.timer
        T.mark("filter_and_project")
        st.rho_prev.copy_(st.rho)
        self.filter.forward_device(st.rho, out=st.rho_filtered)
        heaviside_projection_device(st.rho_filtered, beta, cfg.beta_eta, out=st.rho_projected,
                                    dout=st.dH_drho)
        T.mark("assemble")
        self.fem.build(st.rho_projected, p)
        T.mark("solve")
        comp = self.fem.solve_built(st.u_dofs, force_scale=nscale)
        compliance_avg = float(np.mean(comp))
        T.mark("energy_sensitivity")
        energy, dcp = self.fem.sensitivity_multi_load(st.rho_projected, p, st.u_dofs,
                                                      dh=st.dH_drho)
        T.mark("filter_gradient")
        L = dcp.shape[1]
        if L == 1:
            self.filter_gradient_into(dcp.view(-1), st.dC_drho_full, accumulate=False)
            st.energy_mean.copy_(energy.view(-1))
        else:
            st.dC_drho_full.zero_()
            for i in range(L):
                self.filter_gradient_into(dcp[:, i].contiguous(), st.dC_drho_full,
                                          accumulate=True)
            st.dC_drho_full /= L
            torch.mean(energy, dim=1, out=st.energy_mean)
        if cfg.sensitivity_filter:
            tmp = self.filter.forward_device(st.dC_drho_full)
            st.dC_drho_full.copy_(tmp)
        st.compliance = compliance_avg
        T.mark("rho_update")
        self.rho_update_device(iter_num, st, move_limit, eta, beta, percentile, vol_frac)
        T.mark("metrics")
        rcm = self.filter_design_reduce(1, st.rho, st.rho_prev)
        T.mark("end")
        T.flush()
        st.rho_change_max = rcm
        rec = self.recorder
        rec.feed_data("rho_change_max", rcm)
        rec.feed_data(self.objective_name, compliance_avg)
        rec.feed_data("neumann_scale", nscale)
        converged = False
        if cfg.check_convergence:
            conv_rho = rcm < cfg.tol_rho_change
            kkt = self.kkt_residual
            conv_kkt = (abs(kkt) < cfg.tol_kkt_residual) if np.isfinite(kkt) else True
            converged = conv_rho and conv_kkt
        if cfg.export:
            rec_every = max(cfg.max_iters // cfg.record_times, 1)
            if iter_num % rec_every == 0 or iter_num == 1 or converged or \
                    iter_num == st.iter_end - 1:
                self._export_iteration(iter_num, st)
        return converged

    def _export_iteration(self, iter_num, st):
        """common_density.py:1186-1233: data/NNNNNN-rho.npz and the VTU with
        rho_projected and energy, written off the compute stream."""
        from ..snapshot import SnapshotWriter
        from ..visualization import export_mesh_with_info
        cfg, tsk = self.cfg, self.tsk
        if self._snap is None:
            self._snap = SnapshotWriter(self.device)
        design = np.asarray(tsk.design_elements)

        def write(h):
            np.savez_compressed(f"{cfg.dst_path}/data/{iter_num:06d}-rho.npz",
                                rho_design_elements=h["rho"][design])
            if cfg.export_vtu:
                export_mesh_with_info(tsk.mesh, cell_data_names=["rho_projected", "energy"],
                                      cell_data_values=[h["rho_projected"], h["energy"]],
                                      filepath=cfg.vtu_path(iter_num))
        self._snap.submit({"rho": st.rho, "rho_projected": st.rho_projected,
                           "energy": st.energy_mean}, write)

    def step_host(self, rho_host: torch.Tensor) -> float:
        """One iteration driven from host memory: copy ``rho_host`` (pinned,
        n_elem) to the device, iterate, copy the updated density back and
        return the compliance (the reference's state lives in NumPy arrays)."""
        if not self._ensure_state_initialized():
            return float("nan")
        st = self._state
        st.rho.copy_(rho_host, non_blocking=True)
        it = self._iter_next
        self.step(it)
        self._iter_next = it + 1
        rho_host.copy_(st.rho, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return st.compliance

    def filter_gradient_into(self, v, out, accumulate):
        if not accumulate:
            self.filter.gradient_device(v, out=out)
        else:
            out += self.filter.gradient_device(v)

    def filter_design_reduce(self, op, x, y=None):
        return self.filter.design_reduce(op, x, y)

    def _finalize(self):
        """common_density.py:944-964: histories.npz and the thresholded
        design cubic_top.vtu (elements kept where rho > 0.5)."""
        if self._completed:
            return
        if self.cfg.export:
            self.recorder.export_histories(fname="histories.npz")
            if self.cfg.export_vtu and self._state is not None:
                from ..visualization import export_submesh
                export_submesh(self.tsk, self._state.rho.cpu().numpy(), 0.5,
                               f"{self.cfg.dst_path}/cubic_top.vtu")
        if self._snap is not None:
            self._snap.flush()
        self._completed = True

    def rho_update_device(self, iter_num, st, move_limit, eta, beta, percentile, vol_frac):
        """The update on the device-resident state (the loop's own call):
        reads st.dC_drho_full, st.rho, st.rho_filtered, st.rho_projected and
        updates st.rho and st.scaling_rate in place."""
        raise NotImplementedError("")

    def rho_update(self, iter_num, rho_design_eles, rho_projected, dC_drho_design_eles,
                   u_dofs, strain_energy_mean, scaling_rate, move_limit, eta, beta,
                   rho_clip_lower, rho_clip_upper, percentile, elements_volume_design,
                   elements_volume_design_sum, vol_frac):
        """The reference's update hook with its positional signature, as the
        driver calls it (common_density.py:1112-1129; received at
        oc.py:149-167 and logmoc.py:90-108), for callers that keep their own
        loop.  Arguments are NumPy arrays (or tensors) in the reference's
        layout; they are mutated in place as the reference mutates them:

        * ``rho_design_eles``: the updated design densities;
        * ``scaling_rate``: OC -- the clipped multiplicative factor of the last
          bisection step; log-MOC -- the clipped scaled Lagrangian gradient;
        * ``rho_clip_lower`` / ``rho_clip_upper``: the move-limit bounds (OC:
          in density; log-MOC: in log-density, logmoc.py:47-60);
        * ``dC_drho_design_eles`` (OC only): divided by the running scale.

        As in the reference, the full density (non-design entries) comes from
        this optimizer's state, and ``u_dofs`` / ``strain_energy_mean`` are
        not used.  The filtered density the log-MOC volume chain needs is the
        filter applied to that full density, which is what the driver's state
        holds at this point of the iteration (common_density.py:1043-1045).
        ``elements_volume_design`` must be the task's design-element volumes
        (the only values the reference passes)."""
        if not self._ensure_state_initialized():
            raise RuntimeError("optimization already completed")
        st = self._state
        dev = self.device

        def dev64(x):
            return torch.as_tensor(np.asarray(x) if not isinstance(x, torch.Tensor) else x,
                                   dtype=torch.float64).to(dev)

        def put(dst, src):
            if isinstance(dst, torch.Tensor):
                dst.copy_(src)
            else:
                dst[...] = src.cpu().numpy()

        ev = dev64(elements_volume_design)
        if ev.numel() != self._vol_design.numel() or \
                not torch.equal(ev, self._vol_design):
            raise ValueError("elements_volume_design must be the volumes of the task's "
                             "design elements")
        if not np.isclose(float(elements_volume_design_sum), self._vol_design_sum,
                          rtol=1e-14, atol=0.0):
            raise ValueError("elements_volume_design_sum must be their sum")
        rho_e = dev64(rho_design_eles)
        st.rho[self.design] = rho_e
        st.rho_projected.copy_(dev64(rho_projected))
        self.filter.forward_device(st.rho, out=st.rho_filtered)
        st.dC_drho_full.zero_()
        st.dC_drho_full[self.design] = dev64(dC_drho_design_eles)
        self.rho_update_device(iter_num, st, move_limit, eta, beta, percentile, vol_frac)
        put(rho_design_eles, st.rho[self.design])
        put(scaling_rate, st.scaling_rate)
        lower, upper, dc_scale = self._clip_bounds(rho_e, move_limit)
        put(rho_clip_lower, lower)
        put(rho_clip_upper, upper)
        if dc_scale is not None:
            put(dC_drho_design_eles, st.dC_drho_full[self.design] / dc_scale)

    def _clip_bounds(self, rho_e, move_limit):
        """(lower, upper, dC scale or None) of the method's update."""
        raise NotImplementedError("")
