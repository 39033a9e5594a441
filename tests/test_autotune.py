"""Autotuner host logic (no GPU): shape buckets, the JSON cache, and the
choice of the fastest candidate."""
import json

import pytest

from slothdb_gb300 import autotune


def test_bucket_and_shape_key():
    assert autotune.bucket(0) == 0
    assert autotune.bucket(1) == 1
    assert autotune.bucket(3) == 1
    assert autotune.bucket(4) == 2
    assert autotune.bucket(1_000_000) == autotune.bucket(1_048_575)
    k1 = autotune.shape_key("groupby", 100_000_000, 8_000_000, [3], [("count_star", -1), ("sum", 1)])
    k2 = autotune.shape_key("groupby", 99_000_000, 8_100_000, [3], [("count_star", -1), ("sum", 1)])
    assert k1 == k2
    assert k1 != autotune.shape_key("groupby", 100_000_000, 8_000_000, [2], [("count_star", -1), ("sum", 1)])


def test_cache_roundtrip_and_corrupt_file(tmp_path):
    p = tmp_path / "sub" / "tune.json"
    c = autotune.TuneCache(str(p))
    assert c.get("x") is None
    c.put("x", {"mode": 1, "tile_rows": 8192}, 1.5)
    c.save()
    c2 = autotune.TuneCache(str(p))
    assert c2.get("x") == {"mode": 1, "tile_rows": 8192}
    assert json.loads(p.read_text())["x"]["ms"] == 1.5
    p.write_text("{not json")
    assert autotune.TuneCache(str(p)).get("x") is None


def test_pick_best_skips_failing_candidates():
    times = {1: 5.0, 2: 3.0, 3: 4.0}

    def run(c):
        if c == 4:
            raise RuntimeError("rejected")
        return times[c]

    best, ms, table = autotune.pick_best([1, 2, 3, 4], run, reps=3)
    assert best == 2 and ms == 3.0
    assert [t[2] for t in table if t[0] == 4] == ["rejected"]
    with pytest.raises(RuntimeError):
        autotune.pick_best([4], run)


def test_candidate_sets_are_valid_option_names():
    names = {"mode", "smem_slots", "tile_rows", "ctas_per_sm", "radix_bits", "radix_precombine"}
    for c in autotune.groupby_candidates(1 << 20):
        assert set(c) <= names
    assert any(c.get("mode") == 2 for c in autotune.groupby_candidates(1 << 20))
    assert not any(c.get("mode") == 2 for c in autotune.groupby_candidates(1000))
    for c in autotune.batch_candidates():
        assert set(c) <= {"tile_rows", "smem_slots", "order", "ctas_per_sm"}
