"""CUDA-event section timer (replaces the wall-clock ``SectionTimer`` of
sktopt/tools/timer.py:21-633; same section names as the reference loop)."""
from __future__ import annotations

from collections import defaultdict

import torch


class PhaseTimer:
    def __init__(self):
        self.enabled = False
        self._marks: list[tuple[str, torch.cuda.Event]] = []
        self.totals: dict[str, float] = defaultdict(float)
        self.counts: dict[str, int] = defaultdict(int)

    def mark(self, name: str):
        """Start phase `name` (ends the previous one)."""
        if not self.enabled:
            return
        e = torch.cuda.Event(enable_timing=True)
        e.record(torch.cuda.current_stream())
        self._marks.append((name, e))

    def flush(self):
        """Close the current iteration and accumulate phase times (ms)."""
        if not self.enabled or len(self._marks) < 2:
            self._marks.clear()
            return
        self._marks[-1][1].synchronize()
        for (name, e0), (_, e1) in zip(self._marks[:-1], self._marks[1:]):
            self.totals[name] += e0.elapsed_time(e1)
            self.counts[name] += 1
        self._marks.clear()

    def report(self) -> dict[str, float]:
        return {k: self.totals[k] / max(self.counts[k], 1) for k in self.totals}
