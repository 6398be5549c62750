"""Oracle OC / LogMOC density loop (TEST INFRASTRUCTURE).

Restates:
* ``bisection_with_physical_volume`` oc.py:16-95 and ``OC_Optimizer.rho_update``
  oc.py:149-250 (max/percentile normalisation with EMA 0.6, bisection with
  max_iter 1000 and tolerance 1e-5, KKT infinity norm).
* ``lagrangian_log_update`` logmoc.py:36-66 and ``LogMOC_Optimizer.rho_update``
  logmoc.py:90-258 (EMA dual, 95th-percentile scale with EMA 0.2).
* ``initialize_density`` common_density.py:711-745 and one iteration of
  ``DensityMethod._optimize_impl`` common_density.py:1014-1157.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import fem
from .filters import heaviside_projection, heaviside_projection_derivative
from . import schedule


def bisection_with_physical_volume(dC, rho_e, rho_full, design, filt, rho_min,
                                   rho_max, move_limit, eta, eps, vol_frac,
                                   beta, beta_eta, vol_d, vol_d_sum,
                                   sr_min=0.7, sr_max=1.3, max_iter=1000,
                                   tolerance=1e-5, vol_tol=1e-4, l1=1e-7,
                                   l2=1e7):
    """oc.py:16-95.  Returns (lmid, vol_error, rho_design, scaling_rate, steps)."""
    it = 0
    lmid = 0.5 * (l1 + l2)
    lower = np.maximum(rho_e - move_limit, rho_min)
    upper = np.minimum(rho_e + move_limit, rho_max)
    while True:
        sr = np.negative(dC) / (lmid + eps)
        sr = np.power(sr, eta)
        sr = np.clip(sr, sr_min, sr_max)
        rd = np.clip(rho_e * sr, lower, upper)
        cand = np.copy(rho_full)
        cand[design] = rd
        proj = heaviside_projection(filt.forward(cand), beta, beta_eta)
        vol_error = np.sum(proj[design] * vol_d) / vol_d_sum - vol_frac
        if abs(vol_error) < vol_tol:
            break
        if it >= max_iter:
            break
        if abs(l2 - l1) <= tolerance:
            break
        if vol_error > 0:
            l1 = lmid
        else:
            l2 = lmid
        it += 1
        lmid = 0.5 * (l1 + l2)
    return lmid, vol_error, rd, sr, it + 1


def lagrangian_log_update(rho, dL, eta, move_limit, rho_min, rho_max, clip):
    """logmoc.py:36-66 (returns new rho, scaling_rate, lower, upper)."""
    sr = np.clip(dL, -clip, clip)
    rho = np.clip(rho, rho_min, rho_max)
    lr = np.log(rho)
    du = np.log(1.0 + move_limit / np.exp(lr))
    lower = lr - du
    upper = lower + 2.0 * du
    x = np.log(rho) - eta * sr
    x = np.clip(x, lower, upper)
    x = np.exp(x)
    return np.clip(x, rho_min, rho_max), sr, lower, upper


@dataclass
class Sched:
    kind: str
    init: float | None = None
    target: float | None = None
    num_steps: int | None = None
    curvature: float | None = None

    def __call__(self, it, iters_max):
        return schedule.value(self.kind, it, iters_max, self.init, self.target,
                              self.num_steps, self.curvature)


@dataclass
class OracleConfig:
    """Defaults of DensityMethodConfig common_density.py:232-300 / OC_Config oc.py:98-108."""
    method: str = "oc"                 # "oc" | "logmoc"
    max_iters: int = 200
    beta_eta: float = 0.5
    p: Sched = field(default_factory=lambda: Sched("Step", 1.0, 3.0, 3))
    vol_frac: Sched = field(default_factory=lambda: Sched("Constant", 0.8, 0.8))
    beta: Sched = field(default_factory=lambda: Sched("StepAccelerating", 1.0, 2.0, 3, 2.0))
    # sawtooth_decay("move_limit", 0.3, 0.1, 3) binds 3 to iters_max, so the
    # cycle count keeps its default of 6 (scheduler.py:659-683)
    move_limit: Sched = field(default_factory=lambda: Sched("SawtoothDecay", 0.3, 0.1, 6))
    # None: OC_Config's constant 0.5 (oc.py:98-108) for "oc", the base
    # DensityMethodConfig's 0.6 (common_density.py:62-345) for "logmoc"
    eta: Sched | None = None
    percentile: Sched = field(default_factory=lambda: Sched("None"))
    filter_radius: Sched = field(default_factory=lambda: Sched("Constant", 0.01, 0.01))
    neumann_scale: Sched = field(default_factory=lambda: Sched("ConstantOne", 1.0, 1.0))
    E_min_coeff: float = 1e-3
    rho_min: float = 1e-2
    rho_max: float = 1.0
    # None: DensityMethod_OC_Config's 1e-7 / 1e7 for "oc", LogMOC_Config's
    # -1e7 / 1e7 for "logmoc" (logmoc.py:13-33)
    lambda_lower: float | None = None
    lambda_upper: float | None = None
    scaling_rate_min: float = 0.7
    scaling_rate_max: float = 1.3
    sensitivity_scale_floor: float = 1e-12
    # LogMOC (logmoc.py:13-33)
    mu_p: float = 5.0
    augmented_lagrangian_mu: float = 0.0
    lambda_v: float = 0.1
    lambda_decay: float = 0.9
    lagrangian_clip: float = 1.0
    lagrangian_percentile: float = 95.0
    lagrangian_scale_floor: float = 1e-8
    dual_update: str = "ema"
    solver: str = "spsolve"
    interpolation: str = "SIMP"        # "SIMP" | "RAMP" (common_density.py:392-404)
    rtol: float = 1e-8
    sensitivity_filter: bool = False   # common_density.py:1102-1106

    def __post_init__(self):
        if self.eta is None:
            v = 0.5 if self.method == "oc" else 0.6
            self.eta = Sched("Constant", v, v)
        if self.lambda_lower is None:
            self.lambda_lower = 1e-7 if self.method == "oc" else -1e7
        if self.lambda_upper is None:
            self.lambda_upper = 1e7


class OracleOptimizer:
    """One-process CPU loop with the reference's state and update order."""

    def __init__(self, cfg: OracleConfig, problem, filt, design_elements,
                 fixed_one_elements, elements_volume):
        self.cfg = cfg
        self.pb = problem
        self.filt = filt
        self.design = np.asarray(design_elements, np.int64)
        self.fixed_one = np.asarray(fixed_one_elements, np.int64)
        self.vol = elements_volume
        self.vol_d = elements_volume[self.design]
        self.vol_d_sum = np.sum(self.vol_d)
        self.dV = self.vol_d / self.vol_d_sum
        ne = elements_volume.size
        vf = cfg.vol_frac.init if cfg.vol_frac.init is not None else cfg.vol_frac.target
        rho = np.zeros(ne) + vf
        rho = np.clip(rho, cfg.rho_min, cfg.rho_max)
        rho[self.fixed_one] = 1.0
        all_el = np.arange(ne)
        rho[np.setdiff1d(all_el, self.design)] = 1.0
        self.rho = rho
        self.iter = 1
        self.running_scale = 0.0
        self.lambda_v = cfg.lambda_v
        self.hist = {k: [] for k in ("compliance", "lmid", "vol_error",
                                     "rho_change_max", "kkt_residual",
                                     "bisection_steps")}
        self.last = {}

    def step(self):
        cfg = self.cfg
        it = self.iter
        T = cfg.max_iters
        p = cfg.p(it, T)
        vf = cfg.vol_frac(it, T)
        beta = cfg.beta(it, T)
        move = cfg.move_limit(it, T)
        eta = cfg.eta(it, T)
        pct = cfg.percentile(it, T)
        radius = cfg.filter_radius(it, T)
        nscale = cfg.neumann_scale(it, T)
        if radius != self.filt.radius:
            self.filt.update_radius(radius)
        rho_prev = self.rho.copy()
        rho_f = self.filt.forward(self.rho)
        rho_p = heaviside_projection(rho_f, beta, cfg.beta_eta)
        Emin = self.pb.E0 * cfg.E_min_coeff
        self.pb.interp = cfg.interpolation
        if isinstance(self.pb, fem.ElasticProblem):
            comp, U = self.pb.objectives(rho_p, p, Emin, cfg.solver, cfg.rtol,
                                         force_scale=nscale)
        else:
            comp, U = self.pb.objectives(rho_p, p, Emin, cfg.solver, cfg.rtol)
        energy = self.pb.energy(rho_p, p, Emin, U)
        dH = heaviside_projection_derivative(rho_f, beta, cfg.beta_eta)
        dC_full = np.zeros_like(self.rho)
        # FEM plugins with compliance_sensitivity_multi_load supply their own
        # sensitivity (common_density.py:1068-1085)
        custom = self.pb.custom_sensitivity(rho_p, p, Emin, U) \
            if hasattr(self.pb, "custom_sensitivity") else None
        for i in range(U.shape[1]):
            if custom is not None:
                dCp = custom[:, i]
            else:
                dCp = fem.sensitivity(cfg.interpolation)(rho_p, energy[:, i], self.pb.E0,
                                                         Emin, p)
            dC_full += self.filt.gradient(dCp * dH)
        dC_full /= U.shape[1]
        if cfg.sensitivity_filter:
            dC_full = self.filt.forward(dC_full)
        dC_d = dC_full[self.design].copy()
        rho_d = self.rho[self.design].copy()
        if cfg.method == "oc":
            rho_d = self._oc_update(it, rho_d, dC_d, move, eta, beta, pct, vf)
        else:
            rho_d = self._logmoc_update(it, rho_d, dC_d, rho_p, rho_f, move,
                                        eta, beta, pct, vf)
        self.rho[self.design] = rho_d
        self.rho[self.fixed_one] = 1.0
        ch = float(np.max(np.abs(self.rho[self.design] - rho_prev[self.design])))
        self.hist["compliance"].append(float(comp.mean()))
        self.hist["rho_change_max"].append(ch)
        self.last = dict(rho_filtered=rho_f, rho_projected=rho_p, U=U,
                         energy=energy, dC_full=dC_full, compliance=comp)
        self.iter += 1
        return float(comp.mean())

    def _oc_update(self, it, rho_d, dC, move, eta, beta, pct, vf):
        cfg = self.cfg
        raw = dC.copy()
        if isinstance(pct, float):
            scale = np.percentile(np.abs(dC), pct)
        else:
            scale = np.max(np.abs(dC))
        scale = max(scale, cfg.sensitivity_scale_floor)
        self.running_scale = 0.6 * self.running_scale + (1 - 0.6) * scale \
            if it > 1 else scale
        dC = dC / self.running_scale
        lmid, verr, rd, sr, steps = bisection_with_physical_volume(
            dC, rho_d, self.rho, self.design, self.filt, cfg.rho_min,
            cfg.rho_max, move, eta, 1e-12, vf, beta, cfg.beta_eta,
            self.vol_d, self.vol_d_sum, cfg.scaling_rate_min,
            cfg.scaling_rate_max, max_iter=1000, tolerance=1e-5,
            l1=cfg.lambda_lower, l2=cfg.lambda_upper)
        m = (rd > cfg.rho_min + 1e-6) & (rd < cfg.rho_max - 1e-6)
        kkt = float(np.linalg.norm(raw[m] + (lmid * self.running_scale) *
                                   self.dV[m], ord=np.inf)) if np.any(m) else 0.0
        self.hist["lmid"].append(lmid)
        self.hist["vol_error"].append(verr)
        self.hist["kkt_residual"].append(kkt)
        self.hist["bisection_steps"].append(steps)
        return rd

    def _logmoc_update(self, it, rho_d, dC, rho_p, rho_f, move, eta, beta,
                       pct, vf):
        cfg = self.cfg
        raw = dC.copy()
        dVp = np.zeros_like(self.rho)
        dVp[self.design] = self.dV
        dVf = heaviside_projection_derivative(rho_f, beta, cfg.beta_eta) * dVp
        back = self.filt.gradient(dVf)
        if np.allclose(back, 0.0) and np.any(dVf > 0.0):
            back = self.filt.forward(dVf)
        chain = back[self.design]
        volume = np.sum(rho_p[self.design] * self.vol_d) / self.vol_d_sum
        verr = volume - vf
        penalty = cfg.mu_p * verr
        if cfg.dual_update == "augmented":
            self.lambda_v = self.lambda_v + penalty if it > 1 else penalty
        else:
            self.lambda_v = (cfg.lambda_decay * self.lambda_v +
                             (1 - cfg.lambda_decay) * penalty) if it > 1 else penalty
        self.lambda_v = float(np.clip(self.lambda_v, cfg.lambda_lower,
                                      cfg.lambda_upper))
        coeff = self.lambda_v + cfg.augmented_lagrangian_mu * verr
        dL = raw + coeff * chain
        sp_ = cfg.lagrangian_percentile
        if isinstance(pct, float):
            sp_ = pct
        scale = max(np.percentile(np.abs(dL), sp_), cfg.lagrangian_scale_floor)
        self.running_scale = 0.2 * self.running_scale + (1 - 0.2) * scale \
            if it > 1 else scale
        dL = dL / self.running_scale
        m = (rho_d > cfg.rho_min + 1e-6) & (rho_d < cfg.rho_max - 1e-6)
        kkt = float(np.linalg.norm(dL[m], ord=np.inf)) if np.any(m) else 0.0
        rd, sr, lo, up = lagrangian_log_update(rho_d, dL, eta, move,
                                               cfg.rho_min, cfg.rho_max,
                                               cfg.lagrangian_clip)
        self.hist["vol_error"].append(verr)
        self.hist["kkt_residual"].append(kkt)
        self.hist["lmid"].append(self.lambda_v)
        return rd
