"""bench.py's reference arm on the CPU: one JSON line with the contract's
keys, the oracle timed on a bounded sample (a small lattice here), and the
reference fields (impl, cpu_baseline, e2e without transfers)."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_line():
    env = dict(os.environ, PF_REF_BUDGET_S="2")
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1",
                          "--nx", "32", "--ny", "16", "--nz", "16", "--platelets", "1", "--fibrin", "100"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=300, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "MLUPS" and d["higher_is_better"]
    assert "workload" in d["config"] and d["config"]["timed_steps"] >= 1
    # the same config keys as the GPU arm's line
    for k in ("lattice", "nodes", "elements", "fibrin_nodes", "receptors", "parallelism", "l2", "precision"):
        assert k in d["config"], k
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "stencil-local" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
