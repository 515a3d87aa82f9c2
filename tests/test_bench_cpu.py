"""The reference arm of bench.py (`--impl reference`) on a small lattice: one
JSON line with the benchmark's metric, unit and config, `impl: reference`,
a cpu_baseline describing the run (its value the line's own) and an e2e
block with no host<->device bytes.  The arm times the reference library
built from its sources where it is present (kind "reference"), else the
oracle port (kind "port")."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--L", "6", "--nx",
                        "4", "--steps", "1", "--warmup", "3"], cwd=ROOT, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert "unavailable" not in d
    assert d["unit"] == "evals/s" and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["lattice_L"] == 6 and d["config"]["nx"] == 4
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert set(cb) >= {"value", "unit", "cores", "kind", "sample"}
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
