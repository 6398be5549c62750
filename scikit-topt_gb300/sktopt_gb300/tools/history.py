"""Per-iteration history with the reference's series names and npz layout.

Mirrors ``HistoryCollection`` (sktopt/tools/history.py:278-713): series are
fed once per iteration; ``export_histories`` writes ``histories.npz`` with one
array per series (plots are not produced).
"""
from __future__ import annotations

import os

import numpy as np


class HistoryCollection:
    def __init__(self, dst_path: str = "."):
        self.dst_path = dst_path
        self.histories: dict[str, list] = {}

    def add(self, name: str, **_):
        self.histories.setdefault(name, [])

    def feed_data(self, name: str, data):
        if hasattr(data, "detach"):
            data = data.detach().cpu().numpy()
        self.histories.setdefault(name, []).append(
            np.asarray(data).copy() if np.ndim(data) else float(data))

    def latest(self, name: str):
        h = self.histories.get(name)
        return h[-1] if h else None

    def as_object(self):
        class _O:
            pass
        o = _O()
        for k, v in self.histories.items():
            setattr(o, k, v)
        return o

    def export_histories(self, fname: str = "histories.npz"):
        os.makedirs(self.dst_path, exist_ok=True)
        out = {}
        for k, v in self.histories.items():
            try:
                out[k] = np.asarray(v, dtype=float)
            except (ValueError, TypeError):
                out[k] = np.asarray([np.asarray(x, dtype=float).mean() for x in v])
        np.savez(os.path.join(self.dst_path, fname), **out)

    def import_histories(self, fname: str = "histories.npz"):
        path = os.path.join(self.dst_path, fname)
        if os.path.exists(path):
            data = np.load(path)
            for k in data.files:
                self.histories[k] = list(data[k])
