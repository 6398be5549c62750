"""Device -> host snapshots off the compute stream.

The export of an iteration (the ``data/NNNNNN-rho.npz`` checkpoint and the
VTU of common_density.py:1186-1233) needs device state on the host.  Reading
it with a blocking copy stalls the loop; here the compute stream only
records a device-to-device copy into a snapshot slot (a few microseconds),
a side stream copies the slot to pinned host memory, and a writer thread
waits for that copy and writes the files.  Two slots are kept: a slot is
reused only after the files of its previous snapshot are written.
"""
from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

import torch


class SnapshotWriter:
    def __init__(self, device, n_slots: int = 2):
        self.device = device
        self.stream = torch.cuda.Stream(device=device)
        self.pool = ThreadPoolExecutor(max_workers=1)
        self.slots = [None] * n_slots      # (device copies, pinned copies)
        self.pending = [None] * n_slots    # future of the slot's last write
        self.next = 0
        self.errors = []

    def _slot(self, k, tensors: dict):
        cur = self.slots[k]
        if cur is None or any(cur[0][n].shape != t.shape for n, t in tensors.items()):
            dev = {n: torch.empty_like(t) for n, t in tensors.items()}
            host = {n: torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                    for n, t in tensors.items()}
            self.slots[k] = (dev, host)
        return self.slots[k]

    def submit(self, tensors: dict, write_fn):
        """Snapshot ``tensors`` (name -> device tensor) as of the current
        stream position and call ``write_fn(host arrays)`` on the writer
        thread once they are on the host."""
        k = self.next
        self.next = (k + 1) % len(self.slots)
        if self.pending[k] is not None:
            self.pending[k].result()
        dev, host = self._slot(k, tensors)
        compute = torch.cuda.current_stream(self.device)
        for n, t in tensors.items():
            dev[n].copy_(t)
        ready = torch.cuda.Event()
        ready.record(compute)
        self.stream.wait_event(ready)
        with torch.cuda.stream(self.stream):
            for n in tensors:
                host[n].copy_(dev[n], non_blocking=True)
            done = torch.cuda.Event()
            done.record(self.stream)

        def job():
            done.synchronize()
            write_fn({n: host[n].numpy() for n in tensors})
        self.pending[k] = self.pool.submit(job)

    def flush(self):
        """Wait for every submitted snapshot to be written (re-raises)."""
        for k, f in enumerate(self.pending):
            if f is not None:
                f.result()
                self.pending[k] = None

    def close(self):
        self.flush()
        self.pool.shutdown(wait=True)
