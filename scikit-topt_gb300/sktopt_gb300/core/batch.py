"""Many independent designs on one GPU.

The batched-designs configuration (256 cantilevers of uneven sizes, each its
own OC loop) has no coupling between designs.  ``BatchedDesigns`` gives every
design a complete optimizer -- its own FEM handle, filter handle and state --
bound to its own CUDA stream, and steps the designs from a pool of host
threads.  The library calls release the GIL and every host synchronisation
of a design waits on that design's stream only, so the small, latency-bound
kernels of different designs overlap on the device instead of running one
design after another.  A design's work is ordered on its stream and every
kernel is deterministic, so each design's trajectory is bit-identical to
running it alone.

The fine-level FP32 operator keeps its unit element matrix in the device's
constant bank, shared by all handles: the designs of one batch must use
elements of the same shape (the unit hexahedra of the cantilevers do).
"""
from __future__ import annotations

import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from .._device import default_device


class BatchedDesigns:
    """Step a list of optimizers concurrently.

    ``makers`` holds one zero-argument callable per design that builds its
    optimizer (not yet parameterized); each is called on the main thread
    under the design's stream, so every tensor of the design is allocated on
    that stream.
    """

    def __init__(self, makers, n_workers: int = 8, device=None):
        self.device = device or default_device()
        self.n_workers = max(1, int(n_workers))
        self.streams = []
        self.opts = []
        for make in makers:
            s = torch.cuda.Stream(device=self.device)
            with torch.cuda.stream(s):
                opt = make()
                opt.parameterize()
                opt.fem.engine   # build the FEM handle here, on the design's stream
            self.streams.append(s)
            self.opts.append(opt)
        self._check_shared_element_matrix()
        self._errors: list[BaseException] = []
        self._lock = threading.Lock()

    def _check_shared_element_matrix(self):
        ref = None
        for opt in self.opts:
            ke = opt.fem.engine._ke
            if not opt.fem.engine.mixed:
                continue   # the FP64 operator keeps no constant-bank copy
            if ref is None:
                ref = ke
            elif ke.shape != ref.shape or not np.array_equal(ke, ref):
                raise ValueError("batched designs must share one element matrix "
                                 "(the operator's constant bank is process-wide)")

    def _run(self, i: int, steps: int):
        try:
            with torch.cuda.stream(self.streams[i]):
                self.opts[i].optimize_steps(steps)
            self.streams[i].synchronize()
        except BaseException as e:   # surfaced by step()
            with self._lock:
                self._errors.append(e)

    def step(self, steps: int = 1):
        """Advance every design by ``steps`` OC iterations."""
        with ThreadPoolExecutor(max_workers=self.n_workers) as ex:
            list(ex.map(lambda i: self._run(i, steps), range(len(self.opts))))
        if self._errors:
            raise self._errors[0]

    def __len__(self):
        return len(self.opts)
