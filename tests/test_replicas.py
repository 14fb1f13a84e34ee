"""The multi-GPU form of the benchmark is N independent replicas (no data-path
collective): the whole-job time is the slowest rank's and the rays are the
sum over the ranks, and under torchrun only rank 0 runs the CPU reference arm.
Checked here with two gloo ranks on the CPU."""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

_RANK = """
import os, sys
sys.path.insert(0, {root!r})
import torch
import torch.distributed as dist
import bench
rank = int(os.environ["RANK"])
dist.init_process_group("gloo")
# rank r: times (1 + r, 10 - r, 0.5), rays (100 * (r + 1), 7)
out = bench.reduce_replicas((1.0 + rank, 10.0 - rank, 0.5), (100 * (rank + 1), 7), 2, torch.device("cpu"))
dist.barrier()
dist.destroy_process_group()
assert out == (2.0, 10.0, 0.5, 300.0, 14.0), out
print("rank", rank, "ok")
"""


def _spawn(code: str, rank: int, port: int) -> subprocess.Popen:
    env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(port))
    return subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                            text=True)


def test_replica_reduction_max_time_sum_rays():
    pytest.importorskip("torch.distributed")
    port = 29500 + (os.getpid() % 2000)
    code = _RANK.format(root=str(ROOT))
    procs = [_spawn(code, r, port) for r in range(2)]
    outs = [p.communicate(timeout=300) for p in procs]
    for r, (p, (so, se)) in enumerate(zip(procs, outs)):
        assert p.returncode == 0, f"rank {r}: {so[-1000:]} {se[-3000:]}"
        assert f"rank {r} ok" in so


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2"], env=env,
                         capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr[-3000:]
    assert out.stdout.strip() == ""
