"""Device-memory plumbing (torch owns the allocations; kernels are ours)."""
from __future__ import annotations

import numpy as np
import torch


def default_device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("sktopt_gb300 needs a CUDA device (GB300); none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def as_device(x, dtype=torch.float64, device=None) -> torch.Tensor:
    """Contiguous device tensor view/copy of a numpy array or tensor."""
    device = device or default_device()
    if isinstance(x, torch.Tensor):
        if x.device == device and x.dtype == dtype and x.is_contiguous():
            return x
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x)).to(device=device, dtype=dtype)


def write_back(dst, src: torch.Tensor):
    """Copy a device result into ``dst`` (numpy array or tensor) in place."""
    if isinstance(dst, torch.Tensor):
        if dst.data_ptr() != src.data_ptr():
            dst.copy_(src.reshape(dst.shape))
    else:
        dst[...] = src.reshape(dst.shape).cpu().numpy()


def stream_handle() -> int:
    return torch.cuda.current_stream().cuda_stream
