"""A time window sharded over ranks (genesis-1.3-version4_gb300/sharded.py) on CPU
ranks: gloo, world size 2 and 3, each rank holding its block of one field on the
host with the engine's shift semantics and slippage bookkeeping
(g4gpu_slip_shifts); the blocks exchange their boundary slices through
torch.distributed as the GPU ranks do over NCCL. After a sequence of slippages
(forwards and backwards, several shifts per step, zero-filled and periodic windows)
the ranks' blocks, put together, must equal the slippage of the whole window by the
oracle (Control::applySlippage restated bit-exactly, Control.cpp:158-276).
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# slippage of the steps, in slices (sample = 1): the workload's 2.26 per period, a
# quadrupole step's extra slices, a step without slippage, backwards slippage
SLIPS = [2.2616, 2.2616, 3.0, 0.0, 2.2616, -1.7, -0.4, 1.1]

CHILD = r"""
import os, sys, json
import numpy as np
sys.path.insert(0, {root!r})
sys.path.insert(0, os.path.join({root!r}, "genesis-1.3-version4_gb300"))
import torch.distributed as dist
import sharded
dist.init_process_group("gloo")
rank, size = dist.get_rank(), dist.get_world_size()
ns, ng, periodic = {ns}, {ng}, {periodic}
rng = np.random.default_rng(5)
full = rng.standard_normal((ns, ng * ng)) + 1j * rng.standard_normal((ns, ng * ng))
s0, n = sharded.block(ns, rank, size)
blk = sharded.HostBlock(full[s0:s0 + n], 0, 1.0)
ring = sharded.TorchRing(blk.slice_bytes(), rank, size, periodic, device="cpu")
for slip in {slips!r}:
    sharded.step(blk, 0, slip, ring, 1, stages=0)
w = blk.window()
print(json.dumps({{"rank": rank, "re": w.real.tolist(), "im": w.imag.tolist(), "acc": blk.accuslip}}), flush=True)
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_ranks(size, ns, ng, periodic):
    port = free_port()
    code = CHILD.format(root=ROOT, ns=ns, ng=ng, periodic=periodic, slips=SLIPS)
    procs = []
    for rank in range(size):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(size),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    outs.sort(key=lambda o: o["rank"])
    return outs


@pytest.mark.parametrize("size,periodic", [(2, 0), (2, 1), (3, 0), (3, 1)])
def test_sharded_slippage_matches_whole_window(oracle, size, periodic):
    pytest.importorskip("torch")
    import g4cases as T
    ns, ng = 12, 5
    outs = run_ranks(size, ns, ng, periodic)
    got = np.concatenate([np.array(o["re"]) + 1j * np.array(o["im"]) for o in outs])
    # the whole window through the oracle's slippage (stage 4 only)
    rng = np.random.default_rng(5)
    full = rng.standard_normal((ns, ng * ng)) + 1j * rng.standard_normal((ns, ng * ng))
    lat = np.zeros((len(SLIPS), len(T.LAT_COLS)))
    lat[:, T.C["slip"]] = SLIPS
    lat[:, T.C["dz"]] = 0.015
    part = np.zeros((ns, 4, 6))
    part[..., 0] = 11357.8
    _, f, first, acc = oracle.run_steps(lat, 11357.8, part, np.zeros(ns), 1e-10, 1.0, [1], [1e-4], full[None], [0],
                                        time_run=1, periodic=periodic, stages=4)
    want = f[0][(np.arange(ns) + first[0]) % ns]
    assert np.array_equal(got, want)
    for o in outs:
        assert o["acc"] == acc[0]


def test_block_partition_follows_the_reference():
    """Time::finishInit (GenTime.cpp:74-78): ceil(nslice / size) slices per rank."""
    import sharded
    assert [sharded.block(4096, r, 4) for r in range(4)] == [(0, 1024), (1024, 1024), (2048, 1024), (3072, 1024)]
    assert sharded.block(10, 2, 3) == (8, 4)
    assert sharded.neighbours(0, 3, 1) == (1, 2) and sharded.neighbours(0, 3, -1) == (2, 1)
    assert sharded.sends_and_receives(2, 3, 1, False) == (False, True)
    assert sharded.sends_and_receives(0, 3, 1, False) == (True, False)
    assert sharded.sends_and_receives(0, 3, -1, False) == (False, True)
    assert sharded.sends_and_receives(0, 3, 1, True) == (True, True)
