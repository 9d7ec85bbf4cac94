"""The schedule autotuner's search and cache (no GPU: the timing functions
are synthetic)."""
import json

from pot_gb300 import tune


def test_key_buckets_by_workload_class():
    k1 = tune.schedule_key("f32", [1000] * 64, [900] * 64)
    k2 = tune.schedule_key("f32", [1100] * 70, [1000] * 70)
    k3 = tune.schedule_key("f32", [100] * 64, [900] * 64)
    k4 = tune.schedule_key("f64", [1000] * 64, [900] * 64)
    assert k1 == k2 and k1 != k3 and k1 != k4
    # a batch with one problem 16x the mean work is another class
    assert tune.schedule_key("f32", [1000] * 63 + [16000], [900] * 64) != k1


def test_search_finds_the_fastest_and_caches(tmp_path):
    path = str(tmp_path / "sched.json")
    t = tune.Tuner(path)
    calls = []

    def fill(s):
        calls.append(s)
        return abs(s.ctas_per_sm - 3) + 0.1 * abs(s.units_per_warp - 16) + 0.01 * abs(s.cap_fill - 8)

    def tail(s):
        return abs(s.cap_tail - 32)

    best = t.search("k", "f32", fill, tail, reps=1)
    assert best == tune.Schedule(3, 16, 8, 32)
    assert all(s.cap_tail == tune.DEFAULT.cap_tail for s in calls)  # fill timings keep the tail cap
    assert json.load(open(path))["k"] == [3, 16, 8, 32]
    assert tune.Tuner(path).get("k") == best
    assert len(t.trials["k"]) == 1 + 2 + 2 + 2 + 1 + 2


def test_search_without_tail_timing_keeps_the_default_tail(tmp_path):
    t = tune.Tuner(str(tmp_path / "s.json"))
    best = t.search("k", "f64", lambda s: s.ctas_per_sm, None, reps=1)
    assert best.ctas_per_sm == 1 and best.cap_tail == tune.DEFAULT.cap_tail


def test_unwritable_or_corrupt_cache_is_not_an_error(tmp_path):
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    t = tune.Tuner(str(bad))
    assert t.get("k") is None
    t2 = tune.Tuner(str(tmp_path / "dir_is_a_file"))
    (tmp_path / "dir_is_a_file").mkdir()
    t2.put("k", tune.DEFAULT)  # writing fails quietly; the schedule stays in memory
    assert t2.get("k") == tune.DEFAULT
