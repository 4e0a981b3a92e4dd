"""The N > 1 path of bench.py is replicas: every rank solves its own propagator, the only
communication is one barrier and a max over the ranks' step times (no data-path collective).
Its host logic runs here on two CPU processes over gloo; the reference arm lets ranks > 0 exit
without work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


WORKER = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
class A: impl = "reference"
rank, world = bench.dist_init(A)
assert world == 2 and dist.get_backend() == "gloo"
bench.barrier(world)
t = bench.max_over_ranks(0.5 + rank, world)
print(json.dumps({{"rank": rank, "max": t}}), flush=True)
dist.destroy_process_group()
"""


def test_max_over_ranks_two_gloo_processes():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
        assert '"max": 1.5' in o


def test_reference_arm_rank1_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="1")
    # world size 1 but rank 1: run_reference returns before any work
    code = ("import sys; sys.path.insert(0, %r); import bench\n"
            "class A: impl='reference'; dims=None; warmup=0; steps=0; gpus=2\n"
            "assert bench.run_reference(A, 1, 2) is None\n") % ROOT
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
