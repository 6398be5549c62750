"""GPU Gaussian density filter.

Drop-in for ``SpacialFilter`` (sktopt/filters/spacial.py:106-166): the same
``from_defaults(mesh, elements_volume, radius, design_mask)``,
``update_radius``, ``forward`` and ``gradient``.  The row-normalised Gaussian
matrix W (sigma = r/3, support r; spacial.py:37-103) is built once per radius
by the native library and applied on the GPU; the reference rebuilds it on
every ``forward`` call.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .. import _native as N
from .._device import as_device, default_device
from ..mesh.grid import element_centers
from .base import BaseFilter, DesignOps


class SpacialFilter(DesignOps, BaseFilter):
    fused_bisection = True

    def __init__(self, mesh, elements_volume, radius, design_mask=None, device=None):
        BaseFilter.__init__(self, mesh, elements_volume, radius, design_mask)
        self.lib = N.load()
        self.device = device or default_device()
        self.element_centers = np.ascontiguousarray(element_centers(mesh))
        n = mesh.nelements
        self._mask = np.ones(n, np.uint8) if design_mask is None else \
            np.ascontiguousarray(design_mask, dtype=np.uint8)
        self._design_idx = torch.from_numpy(
            np.nonzero(self._mask)[0].astype(np.int32)).to(self.device)
        self.h = None
        self._build(radius)

    @classmethod
    def from_defaults(cls, mesh, elements_volume, radius=0.3, design_mask=None, device=None):
        return cls(mesh, elements_volume, radius, design_mask, device)

    def _build(self, radius):
        self.close()
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            N.check(self.lib.topt_filter_gauss_create(
                self.mesh.nelements, self.element_centers.ctypes.data_as(C.c_void_p),
                self._mask.ctypes.data_as(C.c_void_p), float(radius), C.byref(h)))
        self.h = h
        self.radius = radius
        # structured hex grid: the FP32 bisection steps may use W as a stencil
        m = self.mesh
        if getattr(m, "kind", None) == "hex" and getattr(m, "has_grid", False):
            N.check(self.lib.topt_filter_set_grid(self.h, *[int(v) for v in m.shape]))
        nd, nnz = C.c_int64(), C.c_int64()
        N.check(self.lib.topt_filter_sizes(self.h, C.byref(nd), C.byref(nnz)))
        self.n_design, self.nnz = nd.value, nnz.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.topt_filter_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stencil_size(self) -> int:
        """Offsets of the stencil form of W (0: the FP32 steps use the CSR)."""
        n = C.c_int32()
        N.check(self.lib.topt_filter_stencil_size(self.h, C.byref(n)))
        return n.value

    def update_radius(self, radius, **_):
        if radius != self.radius:
            self._build(radius)

    def forward_device(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        self._bind()
        y = torch.empty_like(x) if out is None else out
        N.check(self.lib.topt_filter_forward(self.h, C.c_void_p(x.data_ptr()),
                                             C.c_void_p(y.data_ptr())))
        return y

    def gradient_device(self, v: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        self._bind()
        y = torch.empty_like(v) if out is None else out
        N.check(self.lib.topt_filter_gradient(self.h, C.c_void_p(v.data_ptr()),
                                              C.c_void_p(y.data_ptr())))
        return y

    def forward(self, rho_element):
        """spacial.py:135-157: y[design] = W rho[design], passthrough elsewhere."""
        x = as_device(rho_element, device=self.device)
        y = self.forward_device(x)
        return y if isinstance(rho_element, torch.Tensor) else y.cpu().numpy()

    def gradient(self, v):
        """spacial.py:159-166: y[design] = W^T v[design], zero elsewhere."""
        x = as_device(v, device=self.device)
        y = self.gradient_device(x)
        return y if isinstance(v, torch.Tensor) else y.cpu().numpy()

    def export_matrix(self):
        """W as (indptr, indices, data) over design-element positions."""
        rp = np.empty(self.n_design + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        va = np.empty(self.nnz, np.float64)
        N.check(self.lib.topt_filter_export(self.h, rp.ctypes.data_as(C.c_void_p),
                                            ci.ctypes.data_as(C.c_void_p),
                                            va.ctypes.data_as(C.c_void_p)))
        return rp, ci, va
