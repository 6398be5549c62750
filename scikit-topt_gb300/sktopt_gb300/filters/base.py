"""Filter interface (sktopt/filters/base.py:9-37) and the design-set
operations every GPU filter provides to the optimizers."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .. import _native as N
from .._device import stream_handle


class BaseFilter:
    def __init__(self, mesh, elements_volume, radius, design_mask=None):
        self.mesh = mesh
        self.elements_volume = np.asarray(elements_volume, dtype=np.float64)
        self.radius = radius
        self.design_mask = None if design_mask is None else np.asarray(design_mask, bool)

    def update_radius(self, radius, **args):
        raise NotImplementedError("")

    @classmethod
    def from_defaults(cls, mesh, elements_volume, radius=0.3, design_mask=None):
        raise NotImplementedError("")

    def forward(self, rho_element):
        raise NotImplementedError("")

    def gradient(self, v):
        raise NotImplementedError("")


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class DesignOps:
    """Reductions and updates over the design elements, on the native
    design-set handle ``self.h`` (the Gaussian matrix handle, or the identity
    handle for filters whose forward is a PDE solve).  ``fused_bisection`` is
    True when the handle's matrix is the filter itself, so the whole OC
    bisection can run inside one native call."""

    fused_bisection = False

    def _bind(self):
        N.check(self.lib.topt_filter_set_stream(self.h, C.c_void_p(stream_handle())))

    def design_reduce(self, op, x, y=None, w=None, c=0.0, rho_min=0.0, rho_max=1.0) -> float:
        """op 0: max |x[d]|; op 1: max |x[d]-y[d]|; op 2: KKT max |x[d] + c w| (oc.py)."""
        self._bind()
        out = C.c_double()
        N.check(self.lib.topt_design_reduce(self.h, int(op), _p(x), _p(y), _p(w), float(c),
                                            float(rho_min), float(rho_max), C.byref(out)))
        return out.value

    def design_wsum(self, x, w) -> float:
        self._bind()
        out = C.c_double()
        N.check(self.lib.topt_design_wsum(self.h, _p(x), _p(w), C.byref(out)))
        return out.value

    def design_kkt(self, rho, w, c, rho_min, rho_max) -> float:
        self._bind()
        out = C.c_double()
        N.check(self.lib.topt_design_kkt(self.h, _p(rho), _p(w), float(c), float(rho_min),
                                         float(rho_max), C.byref(out)))
        return out.value

    def gather_axpy(self, x, y, c, out):
        self._bind()
        N.check(self.lib.topt_design_gather_axpy(self.h, _p(x), _p(y), float(c), _p(out)))
        return out

    def design_percentile_abs(self, x_full, q) -> float:
        """numpy.percentile(|x[design]|, q)."""
        self._bind()
        out = C.c_double()
        N.check(self.lib.topt_percentile_abs(self.n_design, _p(self._design_idx), _p(x_full),
                                             float(q), C.byref(out),
                                             C.c_void_p(stream_handle())))
        return out.value

    def percentile_abs(self, x, q) -> float:
        """numpy.percentile(|x|, q) of a design-order vector."""
        out = C.c_double()
        N.check(self.lib.topt_percentile_abs(x.numel(), None, _p(x), float(q), C.byref(out),
                                             C.c_void_p(stream_handle())))
        return out.value

    def logmoc_update(self, dl, inv_scale, rho, eta, move, rho_min, rho_max, clip, scaling):
        self._bind()
        N.check(self.lib.topt_logmoc_update(self.h, _p(dl), float(inv_scale), _p(rho),
                                            float(eta), float(move), float(rho_min),
                                            float(rho_max), float(clip), _p(scaling)))

    def oc_bisect(self, dc, dc_scale, rho, vol, vol_sum, prm, scaling):
        """Bisection of oc.py:16-95; returns (lmid, vol_error, steps)."""
        self._bind()
        lmid, verr, steps = C.c_double(), C.c_double(), C.c_int32()
        if self.fused_bisection:
            N.check(self.lib.topt_oc_bisect(self.h, _p(dc), float(dc_scale), _p(rho), _p(vol),
                                            float(vol_sum), C.byref(prm), _p(scaling),
                                            C.byref(lmid), C.byref(verr), C.byref(steps)))
            return lmid.value, verr.value, steps.value
        import torch
        cand = rho.clone()
        filt = torch.empty_like(rho)
        done = C.c_int32(0)
        N.check(self.lib.topt_oc_begin(self.h, _p(rho), C.byref(prm)))
        w, max_steps = prm.l2 - prm.l1, 1
        while w > prm.tolerance and max_steps < 4096:
            w *= 0.5
            max_steps += 1
        max_steps = min(max_steps + 1, prm.max_iter + 1)
        for _ in range(max_steps):
            N.check(self.lib.topt_oc_candidate(self.h, _p(dc), float(dc_scale), C.byref(prm),
                                               _p(cand), _p(scaling)))
            self.forward_device(cand, out=filt)
            self._bind()
            N.check(self.lib.topt_oc_volume(self.h, _p(filt), _p(vol), float(vol_sum),
                                            C.byref(prm), C.byref(done), C.byref(lmid),
                                            C.byref(verr), C.byref(steps)))
            if done.value:
                break
        if not done.value:
            raise N.ToptError(N.TOPT_MAXITER, "OC bisection did not terminate")
        N.check(self.lib.topt_oc_finish(self.h, _p(rho)))
        return lmid.value, verr.value, steps.value
