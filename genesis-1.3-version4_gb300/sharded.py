"""A time window sharded over ranks: one engine handle per rank, each holding a
contiguous block of the window's slices, as the reference runs one MPI rank per
block (Time::finishInit, src/Main/GenTime.cpp:74-77).

The integration step of every slice is local to its rank (a slice's push reads only
its own field slot, that slot's solve only its own beam slice). The one exchange is
the slippage (Control::applySlippage, src/Core/Control.cpp:183-275): per slice shift
every rank sends the slice leaving its block to the next rank and receives the
entering slice from the previous one (the other way round when the slippage runs
backwards); rank 0 (the last rank, backwards) zero-fills unless the window is
periodic, when the ring closes. The engine does its half of every shift
(g4gpu_shift_out / g4gpu_shift_in); a ring object here moves the slice between the
ranks:

  TorchRing  one process per rank, torch.distributed point-to-point transfers (NCCL
             between GPUs, ordered on the handle's stream; gloo with host buffers);
  LocalRing  the ranks' handles driven in lockstep by one process (copies between
             the ranks' device buffers), which reproduces a multi-rank run on one GPU
             without kernels that wait on each other.

block(nslice, rank, size) is the reference's partition of the window.
"""
import ctypes

import numpy as np

STAGE_PUSH, STAGE_FIELD = 1, 2
SLIP_COLUMN = 14  # G4GPU_LAT_SLIP


def block(nslice, rank, size):
    """(first window slice, slices) of rank's block: ns_node = ceil(nslice / size)
    slices per rank, the window rounded up to size * ns_node (GenTime.cpp:74-78)."""
    ns_node = nslice // size + (1 if nslice % size else 0)
    return ns_node * rank, ns_node


def neighbours(rank, size, direction):
    """(rank sent to, rank received from) for a shift in `direction`
    (Control.cpp:188-197)."""
    nxt, prv = (rank + 1) % size, (rank - 1) % size
    return (nxt, prv) if direction > 0 else (prv, nxt)


def sends_and_receives(rank, size, direction, periodic):
    """Whether rank sends its leaving slice and receives its entering one. Without
    the periodic ring the head's leaving slice leaves the window and the tail's
    entering slice is zero (Control.cpp:251-262), so neither is transferred."""
    head = size - 1 if direction > 0 else 0
    tail = 0 if direction > 0 else size - 1
    return periodic or rank != head, periodic or rank != tail


def step(h, istep, slippage, ring, nfield, stages=STAGE_PUSH | STAGE_FIELD):
    """One integration step of a rank's block: the push and field solve on the
    device, then the slippage of every field through `ring`."""
    if stages:
        h.run(istep, 1, stages)
    for k in range(nfield):
        n, d = h.slip_count(k, slippage)
        for _ in range(n):
            ring.shift(h, k, d)


class TorchRing:
    """The slippage transfers of one rank through torch.distributed. Buffers live on
    `device` ("cuda" for NCCL, "cpu" for gloo with host-side blocks)."""

    def __init__(self, slice_bytes, rank, size, periodic, device="cuda", group=None):
        import torch
        self.torch = torch
        self.rank, self.size, self.periodic, self.group = rank, size, bool(periodic), group
        self.device = device
        self.send = torch.empty(slice_bytes, dtype=torch.uint8, device=device)
        self.recv = torch.empty(slice_bytes, dtype=torch.uint8, device=device)

    def shift(self, h, k, direction):
        import torch.distributed as dist
        torch = self.torch
        nxt, prv = neighbours(self.rank, self.size, direction)
        snd, rcv = sends_and_receives(self.rank, self.size, direction, self.periodic)
        if self.size == 1:
            # a single periodic rank receives its own leaving slice
            h.shift_out(k, direction, self.send.data_ptr() if snd else 0)
            h.shift_in(k, self.send.data_ptr() if rcv else 0)
            return
        ctx = None
        if self.device != "cpu" and h.stream() is not None:
            ctx = torch.cuda.stream(torch.cuda.ExternalStream(h.stream()))
            ctx.__enter__()
        try:
            h.shift_out(k, direction, self.send.data_ptr() if snd else 0)
            ops = []
            if snd:
                ops.append(dist.P2POp(dist.isend, self.send, nxt, self.group))
            if rcv:
                ops.append(dist.P2POp(dist.irecv, self.recv, prv, self.group))
            if ops:
                for r in dist.batch_isend_irecv(ops):
                    r.wait()
            h.shift_in(k, self.recv.data_ptr() if rcv else 0)
        finally:
            if ctx is not None:
                ctx.__exit__(None, None, None)


class LocalRing:
    """The ranks' handles of one process, in rank order, stepped in lockstep."""

    def __init__(self, handles, periodic):
        import torch
        self.handles = list(handles)
        self.periodic = bool(periodic)
        nb = self.handles[0].slice_bytes()
        self.bufs = [torch.empty(nb, dtype=torch.uint8, device="cuda") for _ in self.handles]

    def step(self, istep, slippage, nfield, stages=STAGE_PUSH | STAGE_FIELD):
        for h in self.handles:
            if stages:
                h.run(istep, 1, stages)
        size = len(self.handles)
        for k in range(nfield):
            counts = [h.slip_count(k, slippage) for h in self.handles]
            if len(set(counts)) != 1:
                raise RuntimeError("the ranks' accumulated slippage differs")
            n, d = counts[0]
            for _ in range(n):
                for r, h in enumerate(self.handles):
                    snd, _ = sends_and_receives(r, size, d, self.periodic)
                    h.shift_out(k, d, self.bufs[r].data_ptr() if snd else 0)
                for h in self.handles:
                    h.synchronize()
                for r, h in enumerate(self.handles):
                    _, prv = neighbours(r, size, d)
                    _, rcv = sends_and_receives(r, size, d, self.periodic)
                    h.shift_in(k, self.bufs[prv].data_ptr() if rcv else 0)
                for h in self.handles:
                    h.synchronize()


class HostBlock:
    """A rank's block of one field held on the host (numpy), with the engine's shift
    semantics: the exchange logic without a device, for tests of the transfers on
    CPU ranks. Its slippage bookkeeping is the engine's own (g4gpu_slip_shifts)."""

    def __init__(self, field, first, sample, time_run=True):
        self.field = np.array(field, dtype=np.complex128, order="C", copy=True)
        self.first = int(first)
        self.sample = float(sample)
        self.time_run = bool(time_run)
        self.accuslip = 0.0
        self.slot = -1

    def stream(self):
        return None

    def slice_bytes(self):
        return self.field.shape[1] * 16

    def slip_count(self, k, slippage):
        import g4gpu
        if not self.time_run:
            return 0, 1
        n, d, self.accuslip = g4gpu.slip_shifts(self.accuslip, slippage, self.sample)
        return n, d

    def shift_out(self, k, direction, send_ptr):
        ns = self.field.shape[0]
        last = (self.first + ns - 1) % ns
        if direction < 0:
            last = (last + 1) % ns
        if send_ptr:
            ctypes.memmove(send_ptr, self.field[last].ctypes.data, self.slice_bytes())
        self.first = last if direction > 0 else (last + 1) % ns
        self.slot = last

    def shift_in(self, k, recv_ptr):
        if recv_ptr:
            ctypes.memmove(self.field[self.slot].ctypes.data, recv_ptr, self.slice_bytes())
        else:
            self.field[self.slot] = 0
        self.slot = -1

    def window(self):
        """The block's slices in window order."""
        ns = self.field.shape[0]
        return self.field[(np.arange(ns) + self.first) % ns]
