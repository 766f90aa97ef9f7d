"""bench.py's multi-rank logic on CPU: two gloo ranks (127.0.0.1) go through the same
dist_init / barrier / max-over-ranks path the GPU run uses, and the reference arm does its work
on rank 0 only (the other rank returns 0 without work).  No GPU, no oracle run."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

CHILD = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import bench
rank, ws, tdist = bench.dist_init()
bench.barrier(tdist)
t = bench.max_over_ranks(tdist, 10.0 * (rank + 1))
called = []
bench.cpu_baseline = lambda steps=None, budget_s=0: (called.append(1) or (1.0, dict(sample="s", mhex_per_s=1.0, sec_per_iter=1.0)))
class A: steps = 1; warmup = 0; gpus = ws
rc = bench.run_reference(A())
print(json.dumps(dict(rank=rank, ws=ws, max=t, rc=rc, worked=bool(called))))
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_ranks_barrier_max_and_rank0_only_reference():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=240)
        assert p.returncode == 0, e[-2000:]
        outs.append(o)
    import json
    res = {}
    for o in outs:
        lines = [json.loads(line) for line in o.splitlines() if line.startswith('{"rank"')]
        assert len(lines) == 1, o
        res[lines[0]["rank"]] = lines[0]
        if lines[0]["rank"] == 0:
            assert any('"impl": "reference"' in line for line in o.splitlines()), o
        else:
            assert '"impl": "reference"' not in o
    assert res[0]["max"] == res[1]["max"] == 20.0
    assert res[0]["ws"] == res[1]["ws"] == 2
    assert res[0]["worked"] and not res[1]["worked"]
    assert res[0]["rc"] == res[1]["rc"] == 0
