"""The multi-GPU mode of bench.py is replicas only: every rank erodes its own
neighbourhoods (no data-path collective), the slowest rank's time is taken
with one max-reduction, and only rank 0 reports.  Checked with two gloo
processes on the CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo")
reqs = bench.requests(4, rank)
elapsed = bench.max_over_ranks(1.5 + rank, dist, "cpu")
dist.barrier()
print(json.dumps({{"rank": rank, "elapsed": elapsed, "chunks": [(r["ChunkX"], r["ChunkY"]) for r in reqs]}}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_ranks(code, world=2, extra_env=None):
    port = free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), **(extra_env or {}))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    out = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        out.append(o)
    return out


def test_two_replicas_take_the_slowest_time_and_disjoint_work():
    outs = run_ranks(WORKER.format(root=ROOT))
    res = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert [r["elapsed"] for r in res] == [2.5, 2.5]
    a, b = (set(map(tuple, r["chunks"])) for r in res)
    assert not a & b
    # neighbourhoods (3x3 chunks around each centre) of different requests never overlap
    cells = [(x + dx, y + dy) for r in res for (x, y) in r["chunks"] for dx in (-1, 0, 1) for dy in (-1, 0, 1)]
    assert len(cells) == len(set(cells))


def test_reference_arm_reports_on_rank_zero_only():
    code = f"""
import sys
sys.path.insert(0, {ROOT!r})
import bench
class A: steps, warmup, gpus = 1, 0, 2
if int(__import__("os").environ["RANK"]) != 0:
    bench.run_reference(A())
"""
    outs = run_ranks(code)
    assert outs[1].strip() == ""
