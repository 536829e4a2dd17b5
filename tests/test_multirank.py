"""The multi-process path of bench.py on the CPU: two gloo ranks (one
process per GPU on a GPU node) agree on the max-over-ranks time, pass the
barrier, and align different shards; the reference arm runs on rank 0 only.
No GPU is used: the ranks exchange only host values."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
world, rank, local = bench.dist_env()
dist.init_process_group("gloo", rank=rank, world_size=world)
t = bench.reduce_max(1.5 + rank, world)
bench.barrier(world)
seeds = [None] * world
dist.all_gather_object(seeds, bench.shard_seed(rank))
dist.destroy_process_group()
print(json.dumps({{"rank": rank, "world": world, "local": local, "max": t, "seeds": seeds}}))
"""


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reduce_max_and_barrier():
    pytest.importorskip("torch.distributed")
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        outs.append(__import__("json").loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["world"] == 2 and o["local"] == o["rank"]
        assert o["max"] == 2.5                       # max over ranks, as every rank reports
        assert len(set(o["seeds"])) == 2             # each rank aligns its own shard
        assert o["seeds"] == outs[0]["seeds"]


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "1"], env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""                    # other ranks exit without work
