"""The N>1 path of bench.py on CPU: two ranks over gloo (127.0.0.1).  Every
rank solves its own replica, so the only cross-rank steps are the barrier and
the max-reduction of the timing; the reference arm runs on rank 0 alone."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


WORKER = r"""
import os, sys, json
sys.path.insert(0, sys.argv[1])
import bench
ws, rank, local = bench.dist_setup()
assert ws == 2
v = bench.barrier_max(float(rank + 1) * 1.5, ws)
bench.barrier(ws)
# the reference arm: rank 0 alone does the work and prints; rank 1 returns at once
class A: steps = 1; warmup = 0
if rank == 1:
    bench.run_reference(A(), ws, rank)
print(json.dumps({"rank": rank, "max": v}))
import torch.distributed as dist
dist.destroy_process_group()
"""


def test_two_rank_barrier_and_max_over_gloo(tmp_path):
    port = _free_port()
    script = tmp_path / "worker.py"
    script.write_text(WORKER)
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script), ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            out, err = p.communicate(timeout=180)
        except subprocess.TimeoutExpired:
            p.kill()
            pytest.fail("a gloo rank did not finish")
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    assert all(o["max"] == 3.0 for o in outs)
