"""The multi-process path of bench.py, on the CPU with the gloo backend and
two ranks: the max-over-ranks timing every rank agrees on, distinct replica
seeds (replicas: each rank solves its own configuration, no collective in
the data path), and the reference arm that only rank 0 runs."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, sys
sys.path.insert(0, %r)
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
ws, rank, _ = bench.dist_env()
m = bench.max_over_ranks(0.5 + rank, ws, device="cpu")
seeds = [None]*ws
dist.all_gather_object(seeds, bench.replica_seeds(rank))
dist.barrier()
print(json.dumps({"rank": rank, "ws": ws, "max": m, "seeds": seeds}))
dist.destroy_process_group()
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _env(rank, ws, port):
    return dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws),
                RANK=str(rank), LOCAL_RANK=str(rank))


def test_two_gloo_ranks_time_and_seeds():
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", WORKER % ROOT], env=_env(r, 2, port),
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
             for r in range(2)]
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=180)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for o in outs:
        assert o["ws"] == 2
        assert o["max"] == 1.5                       # the slower rank's time, on every rank
        assert o["seeds"][0] != o["seeds"][1]        # independent replicas
        assert tuple(o["seeds"][0]) == (1004, 2400)  # rank 0 keeps the single-GPU inputs


def test_reference_arm_runs_on_rank_zero_only():
    """under torchrun the other ranks of --impl reference exit 0 at once,
    without output and without a process group"""
    env = _env(1, 2, _free_port())
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "3"], env=env,
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
