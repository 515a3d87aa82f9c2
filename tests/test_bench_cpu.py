"""The reference arm of bench.py (`--impl reference`) on a small lattice: one
JSON line with the benchmark's metric, unit and config, `impl: reference`,
a cpu_baseline describing the run (its value the line's own) and an e2e
block with no host<->device bytes.  The arm times the reference library
built from its sources where it is present (kind "reference"), else the
oracle port (kind "port").  Also under the environment torchrun gives its
ranks (OMP_NUM_THREADS=1: the reference library sizes its per-thread scratch
at initialise, so the arm must not run more threads than it sized for) and
as two torchrun ranks on the CPU, of which rank 0 alone prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


ARGS = ["bench.py", "--impl", "reference", "--L", "6", "--nx", "4", "--steps", "1",
        "--warmup", "3"]


def _one_line(r):
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


@pytest.mark.parametrize("omp", [None, "1"])
def test_reference_arm_prints_the_contract_line(omp):
    env = dict(os.environ)
    if omp:
        env["OMP_NUM_THREADS"] = omp
    d = _one_line(subprocess.run([sys.executable] + ARGS, cwd=ROOT, capture_output=True,
                                 text=True, timeout=300, env=env))
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


def test_reference_arm_under_torchrun_two_ranks():
    sk = socket.socket()
    sk.bind(("127.0.0.1", 0))
    port = sk.getsockname()[1]
    sk.close()
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                        str(port)] + ARGS + ["--gpus", "2"], cwd=ROOT, capture_output=True,
                       text=True, timeout=300)
    d = _one_line(r)
    assert d["impl"] == "reference" and d["n_gpus"] == 2
