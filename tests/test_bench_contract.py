"""The benchmark's reference arm (the FP64 CPU oracle on the host cores) prints one JSON line with
every key of the benchmark contract; under a multi-rank launch only rank 0 prints."""
import json
import os
import subprocess
import sys

from conftest import ROOT

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"}


def run_bench(tmp_path, **env):
    e = dict(os.environ, SPOCK_BENCH_DIR=str(tmp_path), **env)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, env=e, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [l for l in r.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_line(tmp_path):
    lines = run_bench(tmp_path)
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert KEYS <= set(out), KEYS - set(out)
    assert out["impl"] == "reference" and out["unit"] == "solves/s" and out["higher_is_better"] is True
    assert (out["steps"], out["warmup"], out["n_gpus"]) == (1, 0, 1)
    assert out["value"] > 0 and out["ms_per_step"] > 0
    cb = out["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == out["value"] and cb["sample"]
    assert out["e2e"] == {"value": out["value"], "unit": "solves/s", "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}
    assert "workload" in out["config"]


def test_reference_arm_other_ranks_silent(tmp_path):
    assert run_bench(tmp_path, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1") == []
