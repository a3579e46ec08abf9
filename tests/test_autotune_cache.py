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
