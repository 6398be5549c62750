"""Launch-shape autotuner of the FEM engine.

Two launch shapes of the engine are free: the node rows per tile of the
FP32-FMA fine-level operator (16, 27 or 32) and the threads per block row of
each level's SELL products (a warp, three threads, or one thread).  The
engine's rules pick them from the grid's y extent and the level size; this
tuner times every candidate on the device (``FemEngine.time_spmv_level``:
back-to-back products replayed as a CUDA graph, so host launch overhead --
larger than the kernel on the small levels -- does not decide) and keeps the
fastest when it beats the rule's choice by more than `margin`, once per
problem shape.  The choices are cached process-wide, so
every design of a batch with the same shape, and a solo run of that shape,
use the same launch shapes and compute the same bits.

No reference counterpart: the reference multiplies with SciPy.
"""
from __future__ import annotations

import threading

import torch

_CACHE: dict = {}
_LOCK = threading.Lock()        # guards _CACHE and _SHAPE_LOCKS
_SHAPE_LOCKS: dict = {}         # one per problem shape: shapes tune concurrently


def _key(engine) -> tuple:
    mesh = engine.mesh
    shape = tuple(mesh.shape) if getattr(mesh, "has_grid", False) else \
        (mesh.kind, mesh.nnodes, mesh.nelements)
    return (engine.bs, bool(engine.mixed), shape, engine.n_levels)


def _time_us(engine, li, x, y, reps: int) -> float:
    # the better of two graph replays
    return min(engine.time_spmv_level(li, x, y, reps) for _ in range(2))


def _measure(engine, margin: float, reps: int) -> dict:
    dt = torch.float32 if engine.mixed else torch.float64
    rule = engine.tuning()
    sizes = engine.level_sizes()
    rec = {"mf_tile": rule["mf_tile"], "row_mapping": list(rule["row_mapping"]),
           "rule": rule, "times_us": {}}
    for li, (nodes, dense) in enumerate(sizes):
        if dense:
            continue
        n = nodes * engine.bs
        g = torch.Generator(device=engine.device).manual_seed(li)
        x = torch.rand(n, dtype=dt, device=engine.device, generator=g)
        y = torch.empty_like(x)
        run = lambda: _time_us(engine, li, x, y, reps)  # noqa: E731
        if li == 0 and rule["mf_tile"]:
            times = {}
            for ty in (16, 27, 32):
                engine.set_mf_tile(ty)
                times[ty] = run()
            best = min(times, key=times.get)
            pick = best if times[best] < (1.0 - margin) * times[rule["mf_tile"]] \
                else rule["mf_tile"]
            engine.set_mf_tile(pick)
            rec["mf_tile"] = pick
            rec["times_us"]["mf_tile"] = {str(k): round(v, 2) for k, v in times.items()}
            continue
        cands = (1, 2, 3) if engine.bs == 3 else (1, 3)
        times = {}
        for m in cands:
            engine.set_row_mapping(li, m)
            times[m] = run()
        best = min(times, key=times.get)
        auto = rule["row_mapping"][li]
        pick = best if times[best] < (1.0 - margin) * times[auto] else auto
        engine.set_row_mapping(li, pick)
        rec["row_mapping"][li] = pick
        rec["times_us"][f"level{li}"] = {str(k): round(v, 2) for k, v in times.items()}
    return rec


def _apply(engine, rec: dict):
    if rec["mf_tile"]:
        engine.set_mf_tile(rec["mf_tile"])
    for li, m in enumerate(rec["row_mapping"]):
        if m:
            engine.set_row_mapping(li, m)


def tune(engine, margin: float = 0.03, reps: int = 20) -> dict:
    """Set the engine's launch shapes: measured once per problem shape (the
    engine must hold an operator, i.e. after an update), then reused from
    the process-wide cache.  Returns the record (choices, the rule's
    choices, candidate times in microseconds)."""
    key = _key(engine)
    with _LOCK:
        rec = _CACHE.get(key)
        shape_lock = None if rec is not None else _SHAPE_LOCKS.setdefault(key, threading.Lock())
    if rec is None:
        # designs of other shapes (other host threads of a batch) tune
        # meanwhile; a second design of this shape waits for the first
        with shape_lock:
            with _LOCK:
                rec = _CACHE.get(key)
            if rec is None:
                rec = _measure(engine, margin, reps)
                with _LOCK:
                    _CACHE[key] = rec
    _apply(engine, rec)
    return rec


def cache() -> dict:
    """The choices made so far, by problem shape."""
    with _LOCK:
        return {str(k): {"mf_tile": v["mf_tile"], "row_mapping": v["row_mapping"]}
                for k, v in _CACHE.items()}


def clear():
    with _LOCK:
        _CACHE.clear()
        _SHAPE_LOCKS.clear()
