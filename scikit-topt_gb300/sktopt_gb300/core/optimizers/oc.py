"""OC optimizer with the GPU bisection.

Drop-in for ``OC_Optimizer`` / ``OC_Config`` (sktopt/core/optimizers/oc.py:
98-250): sensitivity normalisation by max |dC| (or a percentile) with the 0.6
EMA from iteration 2 on, the bisection on the volume multiplier in
[lambda_lower, lambda_upper] with every candidate filtered and projected
(``bisection_with_physical_volume`` oc.py:16-95, max_iter 1000, tolerance
1e-5, vol_tol 1e-4), and the KKT infinity norm over interior elements.
The whole bisection runs on the device (``topt_oc_bisect``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Literal

import numpy as np
import torch

from ... import _native as N
from ... import tools
from .common_density import DensityMethod, DensityMethod_OC_Config


@dataclass
class OC_Config(DensityMethod_OC_Config):
    interpolation: Literal["SIMP"] = "SIMP"
    eta: tools.SchedulerConfig = field(
        default_factory=lambda: tools.SchedulerConfig.constant(target_value=0.5))
    scaling_rate_min: float = 0.7
    scaling_rate_max: float = 1.3
    sensitivity_scale_floor: float = 1e-12


class OC_Optimizer(DensityMethod):
    def __init__(self, cfg: OC_Config, tsk, device=None):
        assert cfg.lambda_lower < cfg.lambda_upper
        super().__init__(cfg, tsk, device)
        self.recorder.add("-dC")
        self.recorder.add("lmid")
        self.running_scale = 0.0
        self.last_bisection_steps = 0

    def rho_update_device(self, iter_num, st, move_limit, eta, beta, percentile, vol_frac):
        cfg = self.cfg
        flt = self.filter
        if isinstance(percentile, float):
            scale = flt.design_percentile_abs(st.dC_drho_full, percentile)
        else:
            scale = flt.design_reduce(0, st.dC_drho_full)
        scale = max(scale, cfg.sensitivity_scale_floor)
        self.running_scale = 0.6 * self.running_scale + (1 - 0.6) * scale \
            if iter_num > 1 else scale
        prm = N.OcParams(rho_min=cfg.rho_min, rho_max=cfg.rho_max, move_limit=move_limit,
                         eta=eta, eps=1e-12, vol_frac=vol_frac, beta=beta,
                         beta_eta=cfg.beta_eta, scaling_min=cfg.scaling_rate_min,
                         scaling_max=cfg.scaling_rate_max, vol_tol=1e-4,
                         l1=cfg.lambda_lower, l2=cfg.lambda_upper, tolerance=1e-5,
                         max_iter=1000,
                         flags=0 if cfg.bisection_fp32_bracket else N.TOPT_OC_EXACT)
        lmid, verr, steps = flt.oc_bisect(st.dC_drho_full, self.running_scale, st.rho,
                                          self._vol_design, self._vol_design_sum, prm,
                                          st.scaling_rate)
        # KKT over interior design elements: |dC_raw + lmid * scale * dV| (oc.py:230-240)
        self.kkt_residual = flt.design_reduce(2, st.dC_drho_full, st.rho,
                                              w=self._dV_drho_design,
                                              c=lmid * self.running_scale,
                                              rho_min=cfg.rho_min, rho_max=cfg.rho_max)
        st.vol_error = verr
        st.kkt_residual = self.kkt_residual
        self.last_bisection_steps = steps
        self.recorder.feed_data("lmid", lmid)
        self.recorder.feed_data("vol_error", verr)
        self.recorder.feed_data("kkt_residual", self.kkt_residual)

    def _clip_bounds(self, rho_e, move_limit):
        """oc.py:59-60 (bounds around the densities before the update) and the
        normalisation dC /= running_scale of oc.py:193."""
        cfg = self.cfg
        lower = torch.clamp(rho_e - move_limit, min=cfg.rho_min)
        upper = torch.clamp(rho_e + move_limit, max=cfg.rho_max)
        return lower, upper, self.running_scale
