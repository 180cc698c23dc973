"""The N > 1 path of bench.py (replicas, no data-path collective), on CPU with
two gloo ranks: the job time is the slowest rank's, every rank sees it, the
throughput counts every replica, and only rank 0 prints."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
rank = int(os.environ["RANK"]); world = int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo")
ms = bench.job_ms([10.0 + rank, 12.0 + rank], world, "cpu")
print(json.dumps({{"rank": rank, "ms": ms, "value": bench.replica_throughput(1000, world, ms)}}))
dist.destroy_process_group()
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _launch(code, world=2, extra=()):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(world), LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", code, *extra], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(o)
    return outs


def test_job_time_is_the_slowest_rank():
    import json
    outs = _launch(CHILD.format(root=ROOT))
    rows = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert [r["ms"] for r in rows] == [12.0, 12.0]          # max of the means 11, 12
    assert all(abs(r["value"] - 2 * 1000 / 0.012) < 1e-6 for r in rows)


def test_reference_arm_prints_on_rank_0_only():
    code = (f"import sys; sys.path.insert(0, {ROOT!r}); import bench; "
            "bench.reference_arm(type('A', (), {'workload': 'graphene_72', 'pixels': 8, "
            "'warmup': 0, 'steps': 1, 'cpu_seconds': 0.2, 'gpus': 2})(), "
            "int(__import__('os').environ['RANK']))")
    outs = _launch(code)
    assert outs[1].strip() == ""
    import json
    line = json.loads(outs[0].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
