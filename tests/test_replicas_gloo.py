"""The multi-rank host logic of bench.py (replicas: one independent lattice per rank, a
barrier around the timed region, the max of the per-rank times) on two CPU ranks over the
gloo backend; the reference arm prints on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, json
sys.path.insert(0, os.environ["PSC_ROOT"])
import bench
world, rank, local, dist = bench.dist_setup()
assert world == 2 and dist is not None
bench.barrier(dist)
m = bench.max_over_ranks(dist, 10.0 + 5.0 * rank)
assert m == 15.0, m
bench.barrier(dist)
print(json.dumps({"rank": rank, "max": m}), flush=True)
dist.destroy_process_group()
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_gloo_ranks_barrier_and_max():
    pytest.importorskip("torch")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), PSC_ROOT=ROOT, CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
        assert '"max": 15.0' in out
