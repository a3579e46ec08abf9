"""The autotuner's JSON cache and selection, on the host: keys name the
workload's shape and precision, entries survive a round trip through the
file (written atomically), and the fastest candidate is the one kept."""
import json
import os

from tbsla_gb300 import autotune as A


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "sub" / "tune.json")
    k1 = A.key("batch_cg", "DIA", 17120768, 64, 884736, 1, "precond1")
    k2 = A.key("pagerank_batched", "CSR", 4194304, 67108864, 4096, 2, "nvec32")
    assert k1 == "batch_cg|DIA|17120768|64|884736|f32|precond1"
    assert A.lookup(k1, path) is None  # no file yet
    A.store(k1, {"settings": {"rows_per_thread": 4, "ctas_per_sm": 2}, "iterations": 30}, path)
    A.store(k2, {"settings": {"gather": 16}}, path)
    assert A.lookup(k1, path)["settings"] == {"rows_per_thread": 4, "ctas_per_sm": 2}
    assert A.lookup(k2, path)["settings"] == {"gather": 16}
    with open(path) as f:
        on_disk = json.load(f)
    assert set(on_disk) == {k1, k2}
    assert not [p for p in os.listdir(os.path.dirname(path)) if p.startswith(".tune.")]  # no temporaries left
    # an unreadable file reads as an empty cache
    with open(path, "w") as f:
        f.write("{not json")
    assert A.load(path) == {}


def test_cache_path_from_environment(tmp_path, monkeypatch):
    monkeypatch.setenv(A.CACHE_ENV, str(tmp_path / "t.json"))
    assert A.cache_path() == str(tmp_path / "t.json")
    assert A.cache_path("/explicit.json") == "/explicit.json"


def test_pick_keeps_the_fastest():
    times = {8: 3.0, 16: 2.0, 4: 2.5}
    best, trials = A.pick([{"gather": g} for g in (8, 16, 4)], lambda c: times[c["gather"]])
    assert best == {"gather": 16}
    assert [t for _, t in trials] == [3.0, 2.0, 2.5]


class _FakeBatch:
    """Stands in for tbsla_gb300.Batch on the host: records the settings it
    is given and the solves it is asked for; a solve 'takes' a time set by
    the current settings."""

    def __init__(self, cost):
        self.offsets = [0, 1000, 3000]
        self.rows, self.ctas = 4, 0
        self.cost = cost
        self.calls = []

    def tuning(self):
        return {"rows_per_thread": self.rows, "ctas_per_sm": self.ctas}

    def set_rows_per_thread(self, r):
        self.rows = r

    def set_ctas_per_sm(self, c):
        self.ctas = c

    def cg(self, rhs, max_iterations, rel_tol, precond, refresh):
        import time
        self.calls.append((self.rows, self.ctas, rel_tol, precond, refresh))
        time.sleep(self.cost[(self.rows, self.ctas)])


def test_tune_batch_cg_times_whole_solves_and_caches(tmp_path):
    """Every (rows per thread, CTAs per SM) candidate is timed on whole
    solves to the requested tolerance; the fastest is applied and cached, and
    a second call applies the cached choice without solving."""
    import numpy as np

    path = str(tmp_path / "t.json")
    cost = {(4, 0): 0.02, (4, 2): 0.005, (1, 0): 0.03, (1, 2): 0.04}
    b = _FakeBatch(cost)
    r = A.tune_batch_cg(b, np.zeros(3000), 1, precond=1, rel_tol=1e-8, reps=1, path=path)
    assert r["settings"] == {"rows_per_thread": 4, "ctas_per_sm": 2} and not r["cached"]
    assert b.tuning() == r["settings"]
    assert {(c[0], c[1]) for c in b.calls} == set(cost)
    assert all(c[2] == 1e-8 and c[3] == 1 and c[4] == 50 for c in b.calls)
    b2 = _FakeBatch(cost)
    b2.rows, b2.ctas = 1, 0
    r2 = A.tune_batch_cg(b2, np.zeros(3000), 1, precond=1, path=path)
    assert r2["cached"] and b2.tuning() == r["settings"] and not b2.calls
