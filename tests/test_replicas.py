"""The benchmark's multi-process path on CPU, world size 2 over gloo: the
barrier and the max over ranks, independent seeded replicas per rank, and
the reference arm launched the way the driver launches N > 1 runs
(torch.distributed.run), where rank 0 alone measures and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytest.importorskip("torch")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


RANK_SCRIPT = r"""
import json, sys
sys.path.insert(0, {repo!r})
import bench
import torch.distributed as dist
world, rank, local = bench.dist_setup()
bench.barrier(world)
m = bench.max_over_ranks(world, float(rank + 1))
_, n, d, max_d, seed, x = bench.workload("uniform-100k-6", rank)
print(json.dumps({{"rank": rank, "world": world, "max": m, "n": n, "first": float(x[0, 0])}}))
bench.barrier(world)
dist.destroy_process_group()
"""


def test_barrier_max_and_replicas_two_ranks():
    port = str(free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(repo=REPO)],
                                      env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert [o["rank"] for o in outs] == [0, 1]
    assert all(o["world"] == 2 and o["max"] == 2.0 and o["n"] == 100000 for o in outs)
    assert outs[0]["first"] != outs[1]["first"]  # each rank has its own replica


def test_reference_arm_under_torchrun():
    port = str(free_port())
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", port, os.path.join(REPO, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--workload", "uniform-100k-6", "--cpu-sample", "2000"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout  # rank 0 alone prints
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["value"] > 0
    assert j["cpu_baseline"]["kind"] in ("port", "reference")
    assert j["e2e"]["h2d_bytes_per_step"] == 0 and j["e2e"]["d2h_bytes_per_step"] == 0
