"""Replicas on two ranks (gloo on CPU): the bench's data path has no
collective; ranks run their own seeded models and only the step time is
max-reduced."""
import json
import os
import re
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_two_rank_replicas():
    pytest.importorskip("torch.distributed")
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", "29517", os.path.join(HERE, "dist_child.py")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=240, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = [json.loads(x) for x in re.findall(r"\{[^{}]*\}", r.stdout)]
    assert sorted(x["rank"] for x in rows) == [0, 1]
    assert all(x["ws"] == 2 and x["max"] == 2.0 for x in rows)
    # each rank draws its own models
    assert rows[0]["hs"] != rows[1]["hs"]
