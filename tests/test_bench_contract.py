"""bench.py's reference arm, run on CPU: `--impl reference` times the
reference's own PARENT.x where it was built on this machine (oracle/_ref),
else the oracle port of its algorithm, on a bounded DOF sample and prints one
JSON line with the contract's keys; under a multi-rank launch only rank 0
runs and prints, the other ranks exit 0 without work."""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _run(extra_env: dict, *args: str) -> subprocess.CompletedProcess:
    env = dict(os.environ)
    env.update(extra_env)
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_the_contract_line():
    p = _run({}, "--impl", "reference", "--steps", "2", "--warmup", "1", "--workload", "plain_294dof_20k",
             "--cpu-sample-atoms", "10")
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["config"]["workload"] == "plain_294dof_20k"
    cb = d["cpu_baseline"]
    sys.path.insert(0, str(ROOT))
    import bench
    assert cb["kind"] == ("reference" if bench.reference_exe() is not None else "port")
    assert cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "24 DOFs (10 atoms) x 20000 frames" in cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_without_work():
    p = _run({"RANK": "1", "WORLD_SIZE": "2"}, "--impl", "reference", "--steps", "1", "--warmup", "0",
             "--workload", "plain_294dof_20k", "--cpu-sample-atoms", "10")
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
