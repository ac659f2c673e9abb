"""The launch-shape autotuner's host logic (168861_gb300/autotune.py) with a fake timer:
candidate sets, the choice, the sample, and the per-device cache."""
import importlib
import json

import pytest

at = importlib.import_module("168861_gb300.autotune")
lib = importlib.import_module("168861_gb300._lib")


class Tree:
    def __init__(self, n):
        self.num_elem = n


def test_candidates():
    mixed = at.candidates(lib.NRT_EXPLICIT, "mixed")
    assert {c["tile_ctas_per_sm"] for c in mixed if c["tiled"]} == {1, 2, 3, 4}
    assert {c["step_threads"] for c in mixed if not c["tiled"]} == {64, 128, 256}
    assert [c["step_threads"] for c in at.candidates(lib.NRT_EXPLICIT, "fp64")] == [32, 64, 128, 256]
    assert at.candidates(lib.NRT_IMPLICIT_BE, "mixed") == [{"tile_ctas_per_sm": c} for c in (2, 3, 4)]
    both = at.candidates(lib.NRT_IMPLICIT_BE, "mixed", [16, 20])
    assert both == [{"restart": r, "tile_ctas_per_sm": c} for r in (16, 20) for c in (2, 3, 4)]


def test_choose():
    assert at.choose([3.0, 1.0, 2.0]) == 1
    assert at.choose([2.0, 1.0, 1.0]) == 1  # first of a tie
    assert at.choose([None, float("inf"), float("nan"), 5.0]) == 3
    with pytest.raises(ValueError):
        at.choose([None, float("inf")])


def test_sample():
    """A stride through the trees (the size mix kept), about sample_elements compartments,
    at least min_trees trees."""
    trees = [Tree(n) for n in (1000, 3000, 5000, 100)]
    assert [t.num_elem for t in at.sample(trees, 4600)] == [1000, 5000]  # every 2nd
    assert [t.num_elem for t in at.sample(trees, 10)] == [1000]  # at least one tree
    assert len(at.sample(trees, 1e9)) == 4
    assert len(at.sample(trees, 10, min_trees=2)) == 2
    many = [Tree(n) for n in range(1000, 5096)]  # 4096 trees of rising size
    part = at.sample(many, 4e6 / 22)
    sizes = [t.num_elem for t in part]
    assert sizes[0] == 1000 and sizes[-1] > 5000 and len(part) < 100  # small to large
    assert len(at.sample(many, 4e6 / 22, min_trees=1024)) >= 1024


def test_key_separates_devices_modes_and_sizes():
    a = [Tree(1000)] * 64
    k = at.workload_key("GB300", lib.NRT_EXPLICIT, "mixed", a)
    assert k != at.workload_key("B200", lib.NRT_EXPLICIT, "mixed", a)
    assert k != at.workload_key("GB300", lib.NRT_EXPLICIT, "fp64", a)
    assert k != at.workload_key("GB300", lib.NRT_IMPLICIT_BE, "mixed", a)
    assert k != at.workload_key("GB300", lib.NRT_EXPLICIT, "mixed", [Tree(1000)] * 4096)
    assert k == at.workload_key("GB300", lib.NRT_EXPLICIT, "mixed", [Tree(1100)] * 64)


def test_tune_picks_the_fastest_and_caches(tmp_path):
    cache = str(tmp_path / "tune.json")
    trees = [Tree(20000)] * 300
    seen = []

    def timer(ps, mode, prec, ov):
        seen.append(dict(ov))
        assert sum(p.num_elem for p in ps) <= 4e6  # a sample, not the whole workload
        if ov.get("tile_ctas_per_sm") == 3:
            raise lib.NeuriteError(1, "nrt_batch_create")  # skipped, not fatal
        return {1: 5.0, 2: 2.0, 4: 3.0}.get(ov.get("tile_ctas_per_sm"), 4.0)

    r = at.tune(trees, lib.NRT_EXPLICIT, "mixed", cache=cache, timer=timer, device_key="dev")
    assert r["options"] == {"tiled": True, "tile_ctas_per_sm": 2}
    assert r["times"][2] is None and len(seen) == 7
    stored = json.load(open(cache))
    assert stored[r["key"]]["options"] == r["options"]
    # served from the cache: no timing
    r2 = at.tune(trees, lib.NRT_EXPLICIT, "mixed", cache=cache, timer=timer, device_key="dev")
    assert r2["options"] == r["options"] and r2["times"] is None and len(seen) == 7
    # another device is tuned on its own
    at.tune(trees, lib.NRT_EXPLICIT, "mixed", cache=cache, timer=timer, device_key="other")
    assert len(seen) == 14


def test_tune_ignores_a_stale_cache_entry(tmp_path):
    cache = tmp_path / "tune.json"
    trees = [Tree(5000)] * 8
    key = at.workload_key("dev", lib.NRT_EXPLICIT, "fp64", trees)
    cache.write_text(json.dumps({key: {"options": {"step_threads": 96}}}))  # not a candidate
    r = at.tune(trees, lib.NRT_EXPLICIT, "fp64", cache=str(cache), device_key="dev",
                timer=lambda ps, m, p, ov: 1.0 / ov["step_threads"])
    assert r["options"] == {"step_threads": 256} and r["times"] is not None


def test_implicit_tunes_its_cta_count(tmp_path):
    """The implicit batch kernel's shape: CTAs per SM, the fastest by the timer; the restart
    length joins the search only when asked for."""
    r = at.tune([Tree(1000)] * 4, lib.NRT_IMPLICIT_BE, "mixed", cache=str(tmp_path / "c.json"),
                timer=lambda ps, m, p, ov: abs(ov["tile_ctas_per_sm"] - 3) + 1.0,
                device_key="dev")
    assert r["options"] == {"tile_ctas_per_sm": 3} and len(r["times"]) == 3
    r = at.tune([Tree(1000)] * 4, lib.NRT_IMPLICIT_BE, "mixed", cache=str(tmp_path / "d.json"),
                timer=lambda ps, m, p, ov: ov["restart"] + ov["tile_ctas_per_sm"] / 10,
                device_key="dev", restarts=[16, 20])
    assert r["options"] == {"restart": 16, "tile_ctas_per_sm": 2}


def test_timer_gets_the_sampled_trees_runs(tmp_path):
    """With runs, each sampled tree is timed with its own loop range and stimulus window."""
    trees = [Tree(1000 + i) for i in range(40)]
    runs = [(1, 100 + i, 0.0, 1e-3 * i) for i in range(40)]
    got = []

    def fake_time(ps, m, prec, ov, steps, warmup, runs=None, **opts):
        got.append(([p.num_elem for p in ps], runs))
        return 1.0

    orig = at.time_candidate
    at.time_candidate = fake_time
    try:
        at.tune(trees, lib.NRT_EXPLICIT, "fp64", cache="", sample_elements=10000, runs=runs,
                device_key="dev")
    finally:
        at.time_candidate = orig
    sizes, rs = got[0]
    assert len(sizes) < 40 and rs == [runs[s - 1000] for s in sizes]
