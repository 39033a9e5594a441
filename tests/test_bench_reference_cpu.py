"""bench.py's reference arm on the host cores (no GPU): every workload prints
one JSON line with the contract's keys, `impl: reference`, a cpu_baseline
describing the run and an e2e equal to its own value with no copies."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = {
    "zipf100m": ["--rows", "200000", "--cpu-sample", "200000"],
    "distinct100m": ["--rows", "200000", "--cpu-sample", "100000"],
    "parquet200m": ["--pq-rows", "300000", "--cpu-sample", "100000"],
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
