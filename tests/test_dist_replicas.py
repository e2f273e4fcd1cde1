"""The multi-process path of bench.py on CPU (gloo, world size 2): the replicas'
barrier, the max-over-ranks reduction of the step time, the whole-job value, and
the reference arm leaving ranks other than 0 without work. Under torchrun on GPUs
the same functions run over NCCL; each rank holds an independent window, and no
collective touches the data path."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import bench
ws, rank, local = bench.dist_setup()
assert ws == 2 and rank == int(os.environ["RANK"])
bench.barrier(ws)
ms = [12.5, 20.0][rank]
m = bench.max_over_ranks(ws, ms)
v = bench.job_value(ws, 4096, 20, m)
rc = bench.run_reference_arm(type("A", (), {{"steps": 1, "warmup": 0}})()) if rank == 1 else 0
print(json.dumps({{"rank": rank, "max": m, "value": v, "ref_rc": rc}}), flush=True)
import torch.distributed as dist
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_agree_on_the_slowest_time():
    pytest.importorskip("torch")
    import json
    port = free_port()
    code = CHILD.format(root=ROOT)
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), G4_BENCH_GLOO="1")
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["max"] == 20.0
        # 2 replicas x 4096 slices x 20 steps in 20 ms
        assert abs(o["value"] - 2 * 4096 * 20 / 0.020) < 1e-6 * o["value"]
        assert o["ref_rc"] == 0
