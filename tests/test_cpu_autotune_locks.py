"""Host logic of the launch-shape autotuner's cache: designs of different
shapes (host threads of a batch) measure concurrently, designs of one shape
measure once and share the record.  The measurement itself is replaced by a
timed stand-in, so no device is needed."""
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
