"""The bench's reference arm on CPU: `bench.py --impl reference` times the FP64
oracle (the reference has no CPU implementation of this path) and prints
one JSON line with the keys of the bench contract; under torch.distributed.run
rank 0 alone runs it and the other ranks exit 0 without output."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BENCH = os.path.join(ROOT, "bench.py")


def _lines(stdout):
    return [json.loads(x) for x in stdout.splitlines() if x.startswith("{")]


def _check_reference_line(d, steps, warmup):
    assert d["impl"] == "reference"
    for key in ("metric", "unit", "config", "dtype", "data"):
        assert d[key], key
    assert d["value"] > 0 and d["higher_is_better"] is True and d["unit"] == "traces/s"
    assert d["steps"] == steps and d["warmup"] == warmup and d["n_gpus"] == 1
    assert d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_line():
    r = subprocess.run([sys.executable, BENCH, "--impl", "reference", "--case", "crust4", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = _lines(r.stdout)
    assert len(rows) == 1
    _check_reference_line(rows[0], 1, 1)


def test_reference_arm_two_ranks_rank0_only():
    pytest.importorskip("torch.distributed")
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", "29519", BENCH, "--gpus", "2", "--impl", "reference",
           "--case", "crust4", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = _lines(r.stdout)
    assert len(rows) == 1
    d = rows[0]
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
