"""bench.py's reference arm on the CPU: one JSON line with the keys the
result contract names (impl, metric, value, unit, the step counts, a
cpu_baseline describing the run and an e2e with no host copies), printed by
rank 0 alone; other ranks exit 0 without work."""
import json
import os
import subprocess
import sys

from conftest import ROOT

ARGS = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "laplacian256",
        "--steps", "1", "--warmup", "3"]


def run(env_extra):
    env = dict(os.environ, **env_extra)
    p = subprocess.run(ARGS, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return [json.loads(line) for line in p.stdout.splitlines() if line.startswith("{")]


def test_reference_arm_line():
    lines = run({"RANK": "0", "WORLD_SIZE": "1", "OMP_NUM_THREADS": "2"})
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference"
    assert d["unit"] == "GFLOPS" and d["value"] > 0 and d["higher_is_better"] is True
    assert (d["steps"], d["warmup"], d["n_gpus"]) == (1, 3, 1)
    assert d["config"]["products"] == 1_629_192
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "GFLOPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_without_work():
    assert run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []
