"""The multi-GPU path of bench.py on the CPU: two ranks over gloo (world size 2).

The path shards as replicas: every rank renders its own block of sample indices of the same
image and the ranks meet only to time the step (a barrier, the maximum of the ranks' device
times, the sum of their samples). This runs that host logic as two processes, checks the
reductions and that the ranks' sample blocks are disjoint, and that the reference arm does its
work on rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import argparse, json, sys
sys.path.insert(0, sys.argv[1])
import bench
world, rank, local = bench.dist_setup()
bench.barrier(world)
out = {
    "world": world, "rank": rank, "local": local,
    "max": bench.allmax(world, 1.5 + rank),
    "sum": bench.allsum(world, 10.0 * (rank + 1)),
    "blocks": [[bench.rank_sample_base(rank, spp, w, k), bench.rank_sample_base(rank, spp, w, k)
                + spp * (w + k + bench.E2E_MAX_STEPS)] for (spp, w, k) in ((64, 3, 5), (32, 3, 1), (1, 10, 100))],
}
if rank == 1:
    # the reference arm: rank 0 alone runs the oracle and prints; the others return at once
    bench.run_reference(argparse.Namespace(gpus=world, steps=1, warmup=0), world, rank)
bench.barrier(world)
print("RESULT " + json.dumps(out), flush=True)
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reduce_and_keep_their_samples_apart():
    pytest.importorskip("torch.distributed")
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    results = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        lines = [l for l in out.splitlines() if l.startswith("RESULT ")]
        assert len(lines) == 1 and not [l for l in out.splitlines() if l.startswith("{")], out
        results.append(json.loads(lines[0][len("RESULT "):]))
    assert [r["rank"] for r in results] == [0, 1]
    for r in results:
        assert r["world"] == 2 and r["max"] == 2.5 and r["sum"] == 30.0
    for case in range(3):
        (a0, a1), (b0, b1) = results[0]["blocks"][case], results[1]["blocks"][case]
        assert a0 == 0 and a1 <= b0 < b1
