"""bench.py's reference arm on the host cores (no GPU): every workload prints
one JSON line with the contract's keys, `impl: reference`, a cpu_baseline
describing the run and an e2e equal to its own value with no copies."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = {
    "plain1m": [],
    "zipf100m": ["--rows", "200000", "--cpu-sample", "200000"],
    "distinct100m": ["--rows", "200000", "--cpu-sample", "100000"],
    "parquet200m": ["--pq-rows", "300000", "--cpu-sample", "100000"],
    "parquet200m_snappy": ["--pq-rows", "300000", "--cpu-sample", "100000"],
    "parquet200m_zstd": ["--pq-rows", "300000", "--cpu-sample", "100000"],
    "dictsum200m": ["--pq-rows", "300000", "--cpu-sample", "100000"],
    "batch256": ["--tables", "1"],
    "serve": ["--duration", "0.05", "--scale", "0.001"],
}

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"}


@pytest.mark.parametrize("workload", sorted(CASES))
def test_reference_arm_json_line(workload):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", workload, "--steps", "1",
                          "--warmup", "1"] + CASES[workload], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 1
    assert d["higher_is_better"] is True and d["vs_baseline"] is None
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["kind"] == "port" and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def _as_gpu(orc):
    """An oracle result in the operator's result shape: [(values, valid)]."""
    cols = [(k, ~np.asarray(n, bool)) for k, n in zip(orc["keys"], orc["key_null"])]
    return cols + [(v, ~np.asarray(n, bool)) for v, n, _ in orc["aggs"]]


def test_oracle_mismatch_helper():
    """bench.oracle_mismatch: equal results (any row order) pass; a changed
    key, count, DOUBLE sum beyond 1e-12 or NULL flag is reported."""
    sys.path.insert(0, ROOT)
    import bench
    import oracle
    rng = np.random.default_rng(3)
    n = 5000
    a = rng.integers(0, 50, n).astype(np.int32)
    b = rng.integers(0, 4, n).astype(np.int16)
    x = rng.normal(5, 1, n)
    v = rng.integers(0, 100, n).astype(np.int64)
    vn = rng.random(n) < 0.3
    vn[a == 3] = True
    aggs = [("count_star", -1), ("sum", 2), ("max", 3)]
    orc = oracle.run_query([2, 1, 4, 3], [0, 1], aggs, [a, b, x, v], nulls=[None, None, None, vn])
    gpu = _as_gpu(orc)
    perm = rng.permutation(orc["n_groups"])
    shuffled = [(c[perm], m[perm]) for c, m in gpu]
    assert bench.oracle_mismatch(shuffled, orc, 2) is None
    bad = [(c.copy(), m.copy()) for c, m in shuffled]
    bad[2][0][0] += 1
    assert "aggregate 0" in bench.oracle_mismatch(bad, orc, 2)
    bad = [(c.copy(), m.copy()) for c, m in shuffled]
    bad[3][0][0] *= 1 + 1e-9
    assert "rel err" in bench.oracle_mismatch(bad, orc, 2)
    bad = [(c.copy(), m.copy()) for c, m in shuffled]
    bad[4][1][:] = True
    assert "NULLs" in bench.oracle_mismatch(bad, orc, 2)
    bad = [(c.copy(), m.copy()) for c, m in shuffled]
    bad[1][0][0] = 99
    assert "key column 1" in bench.oracle_mismatch(bad, orc, 2)
    assert "groups" in bench.oracle_mismatch([(c[1:], m[1:]) for c, m in shuffled], orc, 2)
    # VARCHAR keys (object arrays of bytes) in both results
    strs = np.array([b"s%d" % i for i in range(40)], dtype=object)
    pick = rng.integers(0, 40, n)
    offs = np.zeros(n + 1, np.int64)
    np.cumsum([len(strs[i]) for i in pick], out=offs[1:])
    data = np.frombuffer(b"".join(strs[pick]), np.uint8)
    orc = oracle.run_query([5, 3], [0], [("count_star", -1), ("sum", 1)], [(offs, data), v])
    gpu = _as_gpu(orc)
    perm = rng.permutation(orc["n_groups"])
    assert bench.oracle_mismatch([(c[perm], m[perm]) for c, m in gpu], orc, 1) is None
