"""CPU tests of the autotuner's search and cache logic (adeco_gb300/tune.py),
with fake timings in place of GPU runs."""
import json

from adeco_gb300 import tune


def test_search_finds_the_minimum_of_a_separable_cost():
    space = {"zoom_tile": [32, 48, 64, 96, 128], "share_chunk": [256, 512, 1024, 2048], "clip_batch": [64, 96, 128]}
    best_vals = {"zoom_tile": 96, "share_chunk": 256, "clip_batch": 96}

    def cost(p):
        return sum(abs(space[k].index(p[k]) - space[k].index(best_vals[k])) for k in space) + 1.0

    best, t, trials = tune.search(space, cost)
    assert best == best_vals
    assert t == 1.0
    # coordinate descent measures far fewer settings than the full grid (60)
    assert len(trials) < 5 * 4 * 3


def test_search_measures_each_setting_once_and_keeps_defaults_when_best():
    space = tune.SPACES["leaf"]
    calls = []

    def cost(p):
        calls.append(tuple(sorted(p.items())))
        return 1.0 if p == {"clip_batch": 128, "ctas_per_sm": 2} else 2.0

    best, t, trials = tune.search(space, cost)
    assert best == {"clip_batch": 128, "ctas_per_sm": 2}
    assert len(calls) == len(set(calls)) == len(trials)


def test_search_with_an_interacting_cost_needs_a_second_pass():
    space = {"a": [0, 1, 2], "b": [0, 1, 2]}

    def cost(p):  # the best b depends on a: the first pass stops at (1, 1)
        return (p["a"] - 2) ** 2 + 0.5 * (p["b"] - p["a"]) ** 2

    best, t, _ = tune.search(space, cost, start={"a": 0, "b": 0})
    assert best == {"a": 2, "b": 2} and t == 0


def test_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "sub" / "tuning.json"
    monkeypatch.setenv("ADECO_TUNE_CACHE", str(path))
    c = tune.TuneCache()
    key = tune.TuneCache.key("GB300/152sm", "zoom", "512 requests")
    assert c.get(key) is None
    c.put(key, {"zoom_tile": 48, "share_chunk": 1024, "clip_batch": 96}, 0.5, 11)
    c2 = tune.TuneCache()
    assert c2.get(key) == {"zoom_tile": 48, "share_chunk": 1024, "clip_batch": 96}
    assert c2.get(tune.TuneCache.key("GB300/152sm", "leaf", "512 requests")) is None
    data = json.loads(path.read_text())
    assert data[key]["trials"] == 11


def test_cache_ignores_a_damaged_file(tmp_path):
    p = tmp_path / "tuning.json"
    p.write_text("{not json")
    c = tune.TuneCache(str(p))
    assert c.get("x") is None
    c.put("x", {"clip_batch": 64}, 1.0, 1)
    assert tune.TuneCache(str(p)).get("x") == {"clip_batch": 64}


class FakeSession:
    """Stands in for deposit.Session: timings from the parameters."""

    def __init__(self):
        self.t = dict(tune.DEFAULTS)
        self.applied = []

    def set_tuning(self, **kw):
        self.t.update(kw)
        self.applied.append(dict(kw))

    def replay_leaves(self, reps):
        ms = 100.0 - (10.0 if self.t["clip_batch"] == 96 else 0.0) - (5.0 if self.t["ctas_per_sm"] == 2 else 0.0)
        return {"kernel_ms": ms}


def test_tune_leaves_searches_then_uses_the_cache(tmp_path):
    cache = tune.TuneCache(str(tmp_path / "t.json"))
    s = FakeSession()
    best, info = tune.tune_leaves(s, "c2", cache=cache)
    assert best == {"clip_batch": 96, "ctas_per_sm": 2} and info["source"] == "search"
    s2 = FakeSession()
    best2, info2 = tune.tune_leaves(s2, "c2", cache=cache)
    assert best2 == best and info2["source"] == "cache"
    assert s2.applied == [best]
