"""Smooth Heaviside projection on the GPU (sktopt/core/projection.py:27-118)."""
from __future__ import annotations

import ctypes as C

import torch

from .. import _native as N
from .._device import as_device, stream_handle


def heaviside_projection_device(x: torch.Tensor, beta: float, eta: float = 0.5,
                                out: torch.Tensor | None = None,
                                dout: torch.Tensor | None = None):
    """out = H(x), dout = H'(x); either may be None (not computed)."""
    N.check(N.load().topt_projection(
        x.numel(), C.c_void_p(x.data_ptr()), float(beta), float(eta),
        C.c_void_p(out.data_ptr()) if out is not None else None,
        C.c_void_p(dout.data_ptr()) if dout is not None else None,
        C.c_void_p(stream_handle())))
    return out, dout


def heaviside_projection_inplace(rho, beta, eta=0.5, out=None):
    """projection.py:27-77."""
    x = as_device(rho)
    y = torch.empty_like(x)
    heaviside_projection_device(x, beta, eta, out=y)
    if out is not None:
        if isinstance(out, torch.Tensor):
            out.copy_(y)
        else:
            out[...] = y.cpu().numpy()
        return out
    return y if isinstance(rho, torch.Tensor) else y.cpu().numpy()


def heaviside_projection_derivative_inplace(rho, beta, eta=0.5, out=None):
    """projection.py:80-118."""
    x = as_device(rho)
    y = torch.empty_like(x)
    heaviside_projection_device(x, beta, eta, dout=y)
    if out is not None:
        if isinstance(out, torch.Tensor):
            out.copy_(y)
        else:
            out[...] = y.cpu().numpy()
        return out
    return y if isinstance(rho, torch.Tensor) else y.cpu().numpy()
