"""Log-space modified OC with the GPU kernels.

Drop-in for ``LogMOC_Optimizer`` / ``LogMOC_Config``
(sktopt/core/optimizers/logmoc.py:13-258): the volume-constraint chain
dV -> H'(rho_filtered) -> filter transpose (with the forward fallback when
the transpose vanishes, logmoc.py:133-158), the volume error, the EMA or
augmented dual update of the multiplier, dL = dC + c dV_chain, the 95th
percentile scaling with EMA 0.2, the KKT norm and the log-space update with
move-limit bounds.  Percentiles, reductions and the update are native
kernels; the multiplier and the running scale are host scalars.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Literal

import numpy as np
import torch

import ctypes as C

from ... import _native as N
from ..._device import stream_handle
from .common_density import DensityMethod, DensityMethod_OC_Config
from ..projection import heaviside_projection_device


def _max_abs(x: torch.Tensor) -> float:
    out = C.c_double()
    N.check(N.load().topt_reduce_max_abs(x.numel(), C.c_void_p(x.data_ptr()), C.byref(out),
                                         C.c_void_p(stream_handle())))
    return out.value


@dataclass
class LogMOC_Config(DensityMethod_OC_Config):
    interpolation: Literal["SIMP"] = "SIMP"
    mu_p: float = 5.0
    augmented_lagrangian_mu: float = 0.0
    lambda_v: float = 0.1
    lambda_decay: float = 0.90
    lambda_lower: float = -1e+7
    lambda_upper: float = 1e+7
    lagrangian_clip: float = 1.0
    lagrangian_percentile: float = 95.0
    lagrangian_scale_floor: float = 1e-8
    normalize_volume_chain: bool = False
    volume_chain_percentile: float = 95.0
    volume_chain_scale_floor: float = 1e-8
    volume_chain_gain: float = 1.0
    volume_chain_gain_under: float | None = None
    dual_update: Literal["ema", "augmented"] = "ema"
    filter_lagrangian: bool = False
    center_lagrangian: bool = False
    center_objective: bool = False


class LogMOC_Optimizer(DensityMethod):
    def __init__(self, cfg: LogMOC_Config, tsk, device=None):
        super().__init__(cfg, tsk, device)
        for k in ("dL", "-dC", "lambda_v", "constraint_coeff", "dV_chain",
                  "volume_chain_scale", "lmid"):
            self.recorder.add(k)
        self.lambda_v = cfg.lambda_v
        self.running_scale = 0.0
        self._buf = None

    def _buffers(self):
        if self._buf is None:
            st, dev = self._state, self.device
            nd = self.design.numel()
            self._buf = dict(
                dVp=torch.zeros_like(st.rho), dVf=torch.empty_like(st.rho),
                dVb=torch.empty_like(st.rho), dL=torch.empty(nd, dtype=torch.float64, device=dev),
                dC=torch.empty(nd, dtype=torch.float64, device=dev),
                chain=torch.empty(nd, dtype=torch.float64, device=dev))
            self._buf["dVp"][self.design] = self._dV_drho_design
        return self._buf

    def rho_update_device(self, iter_num, st, move_limit, eta, beta, percentile, vol_frac):
        """logmoc.py:90-258."""
        cfg, flt = self.cfg, self.filter
        B = self._buffers()
        # raw objective sensitivity (design order), optionally centred
        flt.gather_axpy(st.dC_drho_full, None, 0.0, B["dC"])
        if cfg.center_objective:
            mean = flt.design_wsum(st.dC_drho_full, self._vol_design) / self._vol_design_sum
            B["dC"] -= mean
        # volume chain: filter^T (H'(rho_filtered) * dV)
        heaviside_projection_device(st.rho_filtered, beta, cfg.beta_eta, dout=B["dVf"])
        B["dVf"] *= B["dVp"]
        flt.gradient_device(B["dVf"], out=B["dVb"])
        if _max_abs(B["dVb"]) <= 1e-8 and _max_abs(B["dVf"]) > 0.0:
            # np.allclose(back, 0) with positive inputs: the clamped Helmholtz
            # transpose; the filter is self-adjoint there (logmoc.py:145-153)
            flt.forward_device(B["dVf"], out=B["dVb"])
        flt.gather_axpy(B["dVb"], None, 0.0, B["chain"])
        volume = flt.design_wsum(st.rho_projected, self._vol_design) / self._vol_design_sum
        vol_error = volume - vol_frac
        chain_scale = 1.0
        if cfg.normalize_volume_chain:
            obj = max(flt.percentile_abs(B["dC"], cfg.lagrangian_percentile),
                      cfg.lagrangian_scale_floor)
            vs = max(flt.percentile_abs(B["chain"], cfg.volume_chain_percentile),
                     cfg.volume_chain_scale_floor)
            gain = cfg.volume_chain_gain
            if cfg.volume_chain_gain_under is not None and vol_error < 0.0:
                gain = cfg.volume_chain_gain_under
            chain_scale = gain * (obj / vs)
            B["chain"] *= chain_scale
        penalty = cfg.mu_p * vol_error
        if cfg.dual_update == "augmented":
            self.lambda_v = self.lambda_v + penalty if iter_num > 1 else penalty
        else:
            self.lambda_v = (cfg.lambda_decay * self.lambda_v +
                             (1.0 - cfg.lambda_decay) * penalty) if iter_num > 1 else penalty
        self.lambda_v = float(np.clip(self.lambda_v, cfg.lambda_lower, cfg.lambda_upper))
        coeff = self.lambda_v + cfg.augmented_lagrangian_mu * vol_error
        # dL = dC + coeff * chain (design order)
        if cfg.center_objective:
            torch.add(B["dC"], B["chain"], alpha=coeff, out=B["dL"])
        else:
            flt.gather_axpy(st.dC_drho_full, B["dVb"], coeff * chain_scale, B["dL"])
        if cfg.filter_lagrangian:
            full = torch.zeros_like(st.rho)
            full[self.design] = B["dL"]
            flt.gather_axpy(flt.forward_device(full), None, 0.0, B["dL"])
        if cfg.center_lagrangian:
            tmp = torch.zeros_like(st.rho)
            tmp[self.design] = B["dL"]
            B["dL"] -= flt.design_wsum(tmp, self._vol_design) / self._vol_design_sum
        q = percentile if isinstance(percentile, float) else cfg.lagrangian_percentile
        scale = max(flt.percentile_abs(B["dL"], q), cfg.lagrangian_scale_floor)
        self.running_scale = 0.2 * self.running_scale + (1.0 - 0.2) * scale \
            if iter_num > 1 else scale
        inv = 1.0 / self.running_scale
        self.kkt_residual = flt.design_kkt(st.rho, B["dL"], inv, cfg.rho_min, cfg.rho_max)
        st.kkt_residual = self.kkt_residual
        st.vol_error = vol_error
        flt.logmoc_update(B["dL"], inv, st.rho, eta, move_limit, cfg.rho_min, cfg.rho_max,
                          cfg.lagrangian_clip, st.scaling_rate)
        rec = self.recorder
        rec.feed_data("lambda_v", self.lambda_v)
        rec.feed_data("lmid", self.lambda_v)
        rec.feed_data("constraint_coeff", coeff)
        rec.feed_data("vol_error", vol_error)
        rec.feed_data("volume_chain_scale", chain_scale)
        rec.feed_data("kkt_residual", self.kkt_residual)

    def _clip_bounds(self, rho_e, move_limit):
        """The log-space bounds of lagrangian_log_update (logmoc.py:47-60):
        with r = clip(rho, rho_min, rho_max) and d = log(1 + move / r),
        lower = log r - d and upper = lower + 2 d."""
        cfg = self.cfg
        lr = torch.log(torch.clamp(rho_e, cfg.rho_min, cfg.rho_max))
        d = torch.log(move_limit / torch.exp(lr) + 1.0)
        lower = lr - d
        return lower, lower + 2.0 * d, None
