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

Every handle carries its own element matrices (the fine-level FP32
operator takes its unit matrix as a kernel argument), so the designs of one
batch may differ in element shape and material.

The designs launch their V-cycles kernel by kernel: with 16 host threads
stepping 256 designs the device is already kept busy by the other streams,
and replaying the V-cycle as a CUDA graph (re-recorded after every operator
update) measured slower, 352 against 403 design iterations per second
(pass ``vcycle_graphs=True`` to use it anyway).
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

    def __init__(self, makers, n_workers: int = 8, device=None, vcycle_graphs: bool = False):
        self.device = device or default_device()
        self.n_workers = max(1, int(n_workers))
        self.streams = []
        self.opts = []
        for make in makers:
            s = torch.cuda.Stream(device=self.device)
            with torch.cuda.stream(s):
                opt = make()
                opt.parameterize()
                # build the FEM handle here, on the design's stream
                opt.fem.engine.set_vcycle_graphs(vcycle_graphs)
            self.streams.append(s)
            self.opts.append(opt)
        self._errors: list[BaseException] = []
        self._lock = threading.Lock()

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


def partition_designs(costs, world_size: int) -> list:
    """Split designs over ``world_size`` ranks, balancing the summed cost
    (e.g. element or nonzero counts): largest first onto the least loaded
    rank, ties to the lower rank; each rank's list in ascending design order.
    Deterministic, so every rank computes the same partition without a
    collective."""
    costs = np.asarray(costs, dtype=np.float64)
    load = np.zeros(world_size)
    parts = [[] for _ in range(world_size)]
    for i in np.argsort(-costs, kind="stable"):
        r = int(np.argmin(load))
        parts[r].append(int(i))
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def gather_design_results(local: dict, group=None) -> dict | None:
    """The one collective of a sharded batch: every rank's {design index:
    result} is gathered on the group's rank 0 (None elsewhere); a single
    process returns its own results.  ``group`` may be any process group:
    the destination is the global rank of its first member."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return dict(local)
    world = dist.get_world_size(group)
    dst = 0 if group is None else dist.get_global_rank(group, 0)
    out = [None] * world if dist.get_rank(group) == 0 else None
    dist.gather_object(local, out, dst=dst, group=group)
    if out is None:
        return None
    merged = {}
    for part in out:
        merged.update(part)
    return merged


def run_sharded(makers, costs, steps: int, rank: int = 0, world_size: int = 1,
                n_workers: int = 8, device=None, result=None):
    """Run this rank's share of a batch of designs (``partition_designs``)
    for ``steps`` OC iterations and gather the per-design results on rank 0.
    ``result(opt)`` extracts what is gathered (default: the objective
    history)."""
    mine = partition_designs(costs, world_size)[rank]
    local = {}
    if mine:
        batch = BatchedDesigns([makers[i] for i in mine], n_workers=n_workers, device=device)
        batch.step(steps)
        for i, opt in zip(mine, batch.opts):
            local[i] = result(opt) if result else \
                list(opt.recorder.histories[getattr(opt, "objective_name", "compliance")])
    return gather_design_results(local)
