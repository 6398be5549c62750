"""GPU Helmholtz (PDE) density filter on nodes.

Drop-in for ``HelmholtzFilterNodal`` (sktopt/filters/helmholtz_filter_nodal.py:
160-233):

* forward: volume-weighted element -> node average (non-design elements count
  as 1), solve (M + r^2 K) rho_n = M rho_avg with the nodes of non-design
  elements held at 1 (condensation, helmholtz_filter_nodal.py:146-152), node
  -> element mean;
* gradient: the same average with non-design elements counting as 0, a pure
  Neumann solve, node -> element mean and the reference's clamp to <= 0
  (helmholtz_filter_nodal.py:200-233).  Like the reference, ``gradient`` is
  not the exact transpose of ``forward``;
* vjp: the exact transpose of forward's linear part (the derivative of the
  filtered density with respect to the design densities), for gradients
  that must pass a finite-difference check: v -> node sums v_e / nloc ->
  solve with the non-design nodes held at 0 -> M -> element e gets
  vol_e sum over its nodes n of (M z)_n / wsum_n, wsum_n the volume of the
  elements around n (zero on non-design elements).

The nodal systems are solved on the GPU by multigrid-preconditioned CG to a
relative residual of 1e-12 (the reference uses a direct solver).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .. import _native as N
from .._device import as_device, default_device, stream_handle
from ..fea import composer
from ..fea.engine import FemEngine
from .base import BaseFilter, DesignOps


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class HelmholtzFilterNodal(DesignOps, BaseFilter):
    fused_bisection = False

    def __init__(self, mesh, elements_volume, radius, design_mask=None, device=None,
                 rtol=1e-12):
        BaseFilter.__init__(self, mesh, elements_volume, radius, design_mask)
        self.lib = N.load()
        self.device = dev = device or default_device()
        self.rtol = rtol
        ne, nn = mesh.nelements, mesh.nnodes
        dmask = np.ones(ne, bool) if design_mask is None else np.asarray(design_mask, bool)
        self._mask = dmask.astype(np.uint8)
        self._design_idx = torch.from_numpy(np.nonzero(dmask)[0].astype(np.int32)).to(dev)
        h = C.c_void_p()
        with torch.cuda.device(dev):
            N.check(self.lib.topt_filter_identity_create(
                ne, self._mask.ctypes.data_as(C.c_void_p), C.byref(h)))
        self.h = h
        self.n_design = int(dmask.sum())
        # node -> element incidence (elements ascending) for the averaging
        t = np.asarray(mesh.t, np.int64)
        nodes = t.T.ravel()
        elems = np.repeat(np.arange(ne), t.shape[0])
        order = np.argsort(nodes, kind="stable")
        ptr = np.zeros(nn + 1, np.int64)
        np.add.at(ptr, nodes + 1, 1)
        self._nptr = torch.from_numpy(np.cumsum(ptr).astype(np.int32)).to(dev)
        self._nel = torch.from_numpy(elems[order].astype(np.int32)).to(dev)
        self._t = torch.from_numpy(np.ascontiguousarray(t, dtype=np.int32)).to(dev)
        self._vol = torch.from_numpy(np.ascontiguousarray(self.elements_volume)).to(dev)
        self._dflag = torch.from_numpy(self._mask).to(dev)
        fixed_nodes = np.unique(t[:, ~dmask].ravel())
        self._fixed_mask = np.zeros(nn, np.uint8)
        self._fixed_mask[fixed_nodes] = 1
        self._x0 = torch.from_numpy(self._fixed_mask.astype(np.float64)[:, None]).to(dev)
        # for the exact transpose: elements per node / nloc, the volume of the
        # elements around each node, and vol_e * nloc on design elements
        cnt = np.zeros(nn)
        wsum = np.zeros(nn)
        np.add.at(cnt, t.ravel(), 1.0)
        np.add.at(wsum, t.ravel(), np.repeat(self.elements_volume[None, :], t.shape[0],
                                             axis=0).ravel())
        self._cnt_nloc = torch.from_numpy((cnt / t.shape[0])[:, None]).to(dev)
        self._inv_wsum = torch.from_numpy(
            np.where(wsum > 0, 1.0 / np.where(wsum > 0, wsum, 1.0), 0.0)[:, None]).to(dev)
        self._vol_nloc_design = torch.from_numpy(
            np.where(dmask, self.elements_volume * t.shape[0], 0.0)).to(dev)
        self._ones_e = torch.ones(ne, dtype=torch.float64, device=dev)
        self._all_design = torch.ones(ne, dtype=torch.uint8, device=dev)
        _, self._Kh, self._M = composer.element_matrices(mesh, 0.3)
        self._eng = None
        self.radius = None
        self.update_radius(radius)

    @classmethod
    def from_defaults(cls, mesh, elements_volume, radius=0.3, design_mask=None, device=None):
        return cls(mesh, elements_volume, radius, design_mask, device)

    def update_radius(self, radius, **_):
        if radius == self.radius:
            return
        self.radius = radius
        mesh, dev = self.mesh, self.device
        nn = mesh.nnodes
        zeros = np.zeros(nn, np.uint8)
        A = self._M + (radius ** 2) * self._Kh
        ones = torch.ones(mesh.nelements, dtype=torch.float64, device=dev)
        self._eng_M = FemEngine(mesh, 1, self._M, zeros, multigrid=False, device=dev)
        self._eng_free = FemEngine(mesh, 1, A, zeros, multigrid=True, device=dev)
        self._eng_fixed = FemEngine(mesh, 1, A, self._fixed_mask, multigrid=True, device=dev) \
            if self._fixed_mask.any() else None
        for e in (self._eng_M, self._eng_free, self._eng_fixed):
            if e is not None:
                e.update(ones, 1.0, 0.0, 1.0)

    def _solve(self, eng, F):
        U = torch.empty_like(F)
        _, st = eng.solve(F, U, 0, 1 if eng.multigrid else 0, self.rtol, 5000)
        if st.status != 0:
            raise N.ToptError(st.status, f"Helmholtz solve failed: {st}")
        return U

    def _e2n(self, x, fixed):
        out = torch.empty((self.mesh.nnodes, 1), dtype=torch.float64, device=self.device)
        N.check(self.lib.topt_elem_to_node(self.mesh.nnodes, _p(self._nptr), _p(self._nel),
                                           _p(self._vol), _p(x), _p(self._dflag), float(fixed),
                                           _p(out), C.c_void_p(stream_handle())))
        return out

    def _n2e(self, xn, clamp, out):
        N.check(self.lib.topt_node_to_elem(self.mesh.nelements, self._t.shape[0], _p(self._t),
                                           _p(xn), int(clamp), _p(out),
                                           C.c_void_p(stream_handle())))
        return out

    def forward_device(self, x, out=None):
        """helmholtz_filter_nodal.py:180-198."""
        out = torch.empty_like(x) if out is None else out
        b = self._eng_M.spmv(self._e2n(x.contiguous(), 1.0))
        if self._eng_fixed is not None:
            rhs = b - self._eng_free.spmv(self._x0)
            xn = self._solve(self._eng_fixed, rhs) + self._x0
        else:
            xn = self._solve(self._eng_free, b)
        return self._n2e(xn, False, out)

    def gradient_device(self, v, out=None):
        """helmholtz_filter_nodal.py:200-233 (clamped, not the exact transpose)."""
        out = torch.empty_like(v) if out is None else out
        b = self._eng_M.spmv(self._e2n(v.contiguous(), 0.0))
        return self._n2e(self._solve(self._eng_free, b), True, out)

    def vjp_device(self, v, out=None):
        """Exact transpose of forward_device's linear part, applied to v."""
        out = torch.empty_like(v) if out is None else out
        # w_n = sum over the elements e around n of v_e / nloc: the unweighted
        # average over all of them, times their count / nloc
        wn = torch.empty((self.mesh.nnodes, 1), dtype=torch.float64, device=self.device)
        N.check(self.lib.topt_elem_to_node(self.mesh.nnodes, _p(self._nptr), _p(self._nel),
                                           _p(self._ones_e), _p(v.contiguous()),
                                           _p(self._all_design), 0.0, _p(wn),
                                           C.c_void_p(stream_handle())))
        wn *= self._cnt_nloc
        z = self._solve(self._eng_fixed if self._eng_fixed is not None else self._eng_free, wn)
        u = self._eng_M.spmv(z)
        u *= self._inv_wsum
        self._n2e(u, False, out)
        out *= self._vol_nloc_design
        return out

    def forward(self, rho_element):
        x = as_device(rho_element, device=self.device)
        y = self.forward_device(x)
        return y if isinstance(rho_element, torch.Tensor) else y.cpu().numpy()

    def gradient(self, v):
        x = as_device(v, device=self.device)
        y = self.gradient_device(x)
        return y if isinstance(v, torch.Tensor) else y.cpu().numpy()

    def close(self):
        if getattr(self, "h", None):
            self.lib.topt_filter_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
