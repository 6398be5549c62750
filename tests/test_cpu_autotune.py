"""Host logic of the launch-shape autotuner: designs of different shapes
(host threads of a batch) measure concurrently, designs of one shape measure
once and share the record, and a candidate replaces the size rule's choice
only when it is faster by more than the margin.  The device measurement is
replaced by stand-ins, so no device is needed."""
import threading
import time
from types import SimpleNamespace

from sktopt_gb300.core import autotune


class _Mesh(SimpleNamespace):
    has_grid = True


def _engine(shape):
    applied = []
    eng = SimpleNamespace(bs=3, mixed=True, n_levels=3, mesh=_Mesh(shape=shape),
                          set_mf_tile=lambda ty: applied.append(("ty", ty)),
                          set_row_mapping=lambda li, m: applied.append((li, m)))
    eng.applied = applied
    return eng


def _run_threads(engines, monkeypatch, hold=0.3):
    calls = []
    lock = threading.Lock()

    def fake_measure(engine, margin, reps):
        with lock:
            calls.append(tuple(engine.mesh.shape))
        time.sleep(hold)
        return {"mf_tile": 27, "row_mapping": [0, 3, 1], "rule": {}, "times_us": {}}

    monkeypatch.setattr(autotune, "_measure", fake_measure)
    autotune.clear()
    out = [None] * len(engines)

    def work(i):
        out[i] = autotune.tune(engines[i])

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(engines))]
    t0 = time.perf_counter()
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    return calls, out, time.perf_counter() - t0


def test_different_shapes_tune_concurrently(monkeypatch):
    engines = [_engine((8 + i, 8, 8)) for i in range(6)]
    calls, out, dt = _run_threads(engines, monkeypatch)
    assert sorted(calls) == sorted(tuple(e.mesh.shape) for e in engines)
    assert dt < 3 * 0.3, dt            # six 0.3 s measurements overlapped, not serialised
    for e in engines:
        assert ("ty", 27) in e.applied and (1, 3) in e.applied and (2, 1) in e.applied
    autotune.clear()


def test_one_shape_measures_once(monkeypatch):
    engines = [_engine((16, 8, 8)) for _ in range(5)]
    calls, out, _ = _run_threads(engines, monkeypatch)
    assert calls == [(16, 8, 8)]
    assert all(r is out[0] for r in out)
    assert all(("ty", 27) in e.applied for e in engines)
    assert list(autotune.cache().values()) == [{"mf_tile": 27, "row_mapping": [0, 3, 1]}]
    autotune.clear()


class _TimedEngine:
    """Stand-in engine whose level products take the tabulated device times
    of the launch shape in use."""

    def __init__(self, tile_times, map_times, rule_tile=27, rule_maps=(0, 3, 2, 1, 0)):
        import torch
        self.bs, self.mixed, self.device = 3, True, torch.device("cpu")
        self.n_levels = len(rule_maps)
        self.mesh = _Mesh(shape=(11, 7, 5))
        self._rule = {"mf_tile": rule_tile, "row_mapping": list(rule_maps)}
        self.tile, self.maps = rule_tile, list(rule_maps)
        self.tile_times, self.map_times = tile_times, map_times

    def tuning(self):
        return {"mf_tile": self.tile, "row_mapping": list(self.maps)}

    def level_sizes(self):
        return [(40, False)] * (self.n_levels - 1) + [(4, True)]

    def set_mf_tile(self, ty):
        self.tile = ty

    def set_row_mapping(self, li, m):
        self.maps[li] = m

    def time_spmv_level(self, li, x, y, reps):
        return self.tile_times[self.tile] if li == 0 else self.map_times[li][self.maps[li]]


def test_tuner_keeps_the_rule_unless_beaten_by_the_margin():
    # level 0: 16-row tiles 2.7 % faster than the rule's 27 (inside the 3 %
    # margin: keep 27); level 1: a warp 10 % faster than the rule's one
    # thread (take it); level 2: the rule is fastest; level 3: three threads
    # exactly 3 % faster (not more than the margin: keep the warp)
    eng = _TimedEngine({16: 72.0, 27: 74.0, 32: 90.0},
                       {1: {1: 40.5, 2: 47.0, 3: 45.0},
                        2: {1: 9.0, 2: 7.5, 3: 8.0},
                        3: {1: 6.0, 2: 5.82, 3: 9.0}})
    autotune.clear()
    rec = autotune.tune(eng, margin=0.03, reps=5)
    assert rec["mf_tile"] == 27 and eng.tile == 27
    assert rec["row_mapping"] == [0, 1, 2, 1, 0]
    assert eng.maps == [0, 1, 2, 1, 0]
    assert rec["times_us"]["level1"] == {"1": 40.5, "2": 47.0, "3": 45.0}
    eng2 = _TimedEngine({16: 60.0, 27: 74.0, 32: 90.0},
                        {1: {1: 50.0, 2: 47.0, 3: 45.0}, 2: {1: 9.0, 2: 7.5, 3: 8.0},
                         3: {1: 6.0, 2: 7.0, 3: 9.0}})
    eng2.mesh = _Mesh(shape=(12, 7, 5))
    rec2 = autotune.tune(eng2, margin=0.03, reps=5)
    assert rec2["mf_tile"] == 16 and eng2.tile == 16
    assert rec2["row_mapping"] == [0, 3, 2, 1, 0]
    autotune.clear()
