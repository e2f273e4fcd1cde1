#!/usr/bin/env python3
"""Throughput of the GENESIS 1.3 v4 undulator step on GB300, in slice-steps/s.

Workload (one "step" = one integration step of the whole time window): the
time-dependent SASE configuration with 4096 slices at sample = 1, 8192 particles
per slice (33.5 M particles), ngrid = 151 over dgrid = 1e-4 m, planar undulator
aw = 1.7, lambda_u = 15 mm, 4 modules of 110 periods with FODO quadrupoles
(k1 = +-1.5 m^-2, l = 0.08 m) between them, gamma0 = 11357.8, lambda0 = 1e-10 m,
delgam = 2.0, normalised emittance 0.4 um, beta 15 m, a flat-top current of
3000 A with Gaussian edges of rms 0.2 fs, shot noise from seed 7, ADI solver,
slippage with zero-fill. Inputs are synthetic with those shapes (the reference
publishes no dataset). Every array the step touches (1.6 GB of particles, 0.75 /
1.5 GB of field) is larger than the 129 MB L2, so no flush is needed between
steps.

Arms:
  default             the engine through its C ABI: the mixed form (FP32 field,
                      FP64 phase) is the headline `value`; the plain FP64 form is
                      timed beside it, and the mixed form's error against it is
                      reported. `e2e` times a whole track window through the ABI
                      with host buffers: upload of beam and field from pinned
                      memory, K steps each followed by the per-slice power /
                      bunching read-back, download of the final beam and field.
  --impl reference    the CPU implementation of the step on the host cores, all
                      threads: the reference compiled from its own sources where
                      it is built (oracle/_ref), else the C restatement of it
                      (oracle/g4oracle.c), on a bounded sample of the workload.

Under torchrun (N > 1) every rank runs its own window on its GPU (independent
replicas, weak scaling); the slowest rank's time sets the value.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "genesis-1.3-version4_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

import g4cases as T  # noqa: E402  (lattice / profile helpers)

NS, NPART, NGRID, GRIDMAX = 4096, 8192, 151, 1e-4
LAMBDA0, GAMMA0 = 1e-10, 11357.8
EDGE_SIGMA = 0.2e-15 * 299792458.0  # 0.2 fs rms edges
METRIC = "slice-steps/s on 1 GB300: plain FP64 vs mixed/batched/learned at <=1% power error"


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload_inputs(ns=None):
    ns = ns or NS
    cur = flat_top(ns)
    sp = T.slice_params(ns, GAMMA0, 2.0, 0.4e-6, 15.0, currents=cur)
    lat = T.undulator_lattice(1.7, 0.015, 110, 4, LAMBDA0, GAMMA0, quad_k1=1.5, quad_l=0.08)
    return lat, sp, cur


def flat_top(ns):
    """3000 A flat top whose Gaussian edges (rms EDGE_SIGMA) start one sigma from the window ends."""
    s = np.arange(ns) * LAMBDA0
    lo, hi = EDGE_SIGMA, s[-1] - EDGE_SIGMA
    cur = np.full(ns, 3000.0)
    cur[s < lo] = 3000.0 * np.exp(-0.5 * ((s[s < lo] - lo) / EDGE_SIGMA) ** 2)
    cur[s > hi] = 3000.0 * np.exp(-0.5 * ((s[s > hi] - hi) / EDGE_SIGMA) ** 2)
    return cur


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("G4_BENCH_GLOO") is None else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch
        import torch.distributed as dist
        dist.barrier()
        torch.cuda.synchronize()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def alg_bytes_per_slice_step(mixed):
    """Algorithmic bytes of one slice-step (fused step: particles and field read and
    written once): plain 96 npart + 32 ngrid^2; mixed 56 npart + 16 ngrid^2."""
    ncell = NGRID * NGRID
    return (56 * NPART + 16 * ncell) if mixed else (96 * NPART + 32 * ncell)


def kernel_alg_bytes(kernel, mixed, ns=None):
    """Algorithmic bytes of one launch of a kernel class over the whole window:
    what the kernel must read and write at least, per slice:
      push        particles read + written (plain 96 B, mixed 56 B per particle) and
                  the field slice gathered once (16 / 8 B per cell); in the plain form
                  the push also deposits, writing the source once (16 B per cell)
      adi_x       (plain, and mixed for ngrid > 168) field + source read, intermediate
                  written: 3 x 16 / 3 x 8 B per cell
      adi_y       intermediate + source read, field written: same
      field       (fused mixed kernel) field read + written (16 B per cell) and the
                  particle coordinates the deposition needs (x, y, gamma FP32, theta
                  FP64: 20 B per particle)"""
    ns = ns or NS
    ncell = NGRID * NGRID
    if kernel == "push":
        per = (56 * NPART + 8 * ncell) if mixed else (96 * NPART + 32 * ncell)
    elif kernel in ("adi_x", "adi_y"):
        per = (24 if mixed else 48) * ncell
    elif kernel == "field":
        per = 16 * ncell + 20 * NPART
    else:
        return None
    return ns * per


def time_form(g4gpu, torch, precision, beam, cur, lat, steps, warmup, profile=True):
    cfg = g4gpu.Config(nslice=NS, npart=NPART, ngrid=NGRID, gridmax=GRIDMAX, lambda0=LAMBDA0,
                       sample=1.0, gammaref=GAMMA0, precision=precision, time_run=1,
                       device=torch.cuda.current_device())
    h = g4gpu.Handle(cfg)
    h.set_lattice(lat)
    h.load_beam(beam, cur)
    h.load_field(0, np.zeros((NS, NGRID * NGRID), dtype=np.complex128))
    nlat = lat.shape[0]
    for i in range(warmup):
        h.run(i % nlat, 1)
    h.synchronize()
    stream = torch.cuda.ExternalStream(h.stream())
    h.reset_stats()
    h.set_profiling(profile)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        h.run((warmup + i) % nlat, 1)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    stats = h.kernel_stats()
    h.set_profiling(False)
    return h, ms, stats


def e2e_window(g4gpu, torch, precision, beam_pinned, cur, field_pinned, lat, steps, reps):
    """Track windows through the ABI with host buffers: upload, `steps` steps each
    followed by the per-slice diagnostics read-back, download of beam and field."""
    cfg = g4gpu.Config(nslice=NS, npart=NPART, ngrid=NGRID, gridmax=GRIDMAX, lambda0=LAMBDA0,
                       sample=1.0, gammaref=GAMMA0, precision=precision, time_run=1,
                       device=torch.cuda.current_device())
    h = g4gpu.Handle(cfg)
    h.set_lattice(lat)
    out_beam = torch.empty_like(beam_pinned).pin_memory()
    out_field = torch.empty_like(field_pinned).pin_memory()
    cur_np = np.ascontiguousarray(cur)
    times = []
    d2h_diag = 0
    for rep in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h.load_beam_ptr(beam_pinned.data_ptr(), cur_np.ctypes.data)
        h.load_field_ptr(0, field_pinned.data_ptr())
        d2h_diag = 0
        for i in range(steps):
            h.run(i, 1)
            bd, fd = h.diag(1)
            d2h_diag += bd.nbytes + fd.nbytes
        h.get_beam(out_beam.numpy())
        h.get_field(0, out_field.numpy().view(np.complex128).reshape(NS, NGRID * NGRID))
        t1 = time.perf_counter()
        if rep > 0:  # the first window is the warm-up
            times.append(t1 - t0)
    h.close()
    h2d = beam_pinned.numel() * 8 + cur_np.nbytes + field_pinned.numel() * 8
    d2h = d2h_diag + out_beam.numel() * 8 + out_field.numel() * 8
    return min(times), h2d, d2h


def cpu_baseline(nthreads, target_seconds=12.0, prefer_reference=True):
    """Times the CPU step (oracle/_ref when built here, else the oracle port) on a
    bounded sample: full-size slices (8192 particles, ngrid 151) of the workload."""
    import g4oracle
    import build_oracle
    build_oracle.build_oracle()
    ref = g4oracle.reference() if prefer_reference else None
    kind = "reference" if ref is not None else "port"
    lib = ref if ref is not None else g4oracle.oracle()
    threads = 1 if ref is not None else nthreads
    lat, _, _ = workload_inputs()
    import g4gpu
    ns = max(threads, 1)
    cur = flat_top(NS)[NS // 2 - ns // 2:NS // 2 - ns // 2 + ns]
    sp = T.slice_params(ns, GAMMA0, 2.0, 0.4e-6, 15.0, currents=cur)
    beam = g4gpu.host_load_beam(sp, NS // 2 - ns // 2, NPART, 4, 7, 1, LAMBDA0, 1.0)
    fld = np.zeros((1, ns, NGRID * NGRID), dtype=np.complex128)
    # one step first to size the sample
    t0 = time.perf_counter()
    kw = dict(time_run=1)
    if kind == "port":
        kw["nthreads"] = threads
    lib.run_steps(lat[:1], GAMMA0, beam, cur, LAMBDA0, 1.0, [1], [GRIDMAX], fld, [0], **kw)
    dt = time.perf_counter() - t0
    nsteps = int(max(1, min(lat.shape[0], target_seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    lib.run_steps(lat[:nsteps], GAMMA0, beam, cur, LAMBDA0, 1.0, [1], [GRIDMAX], fld, [0], **kw)
    dt = time.perf_counter() - t0
    return {"value": ns * nsteps / dt, "unit": "slice-steps/s", "cores": threads, "kind": kind,
            "sample": f"{ns} slices x {nsteps} steps of the workload (8192 particles, ngrid 151, "
                      f"plain FP64), {threads} host thread(s), {dt:.1f} s"}


def run_reference_arm(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    import g4oracle
    import build_oracle
    build_oracle.build_oracle()
    nthreads = os.cpu_count() or 1
    ref = g4oracle.reference()
    kind = "reference" if ref is not None else "port"
    lib = ref if ref is not None else g4oracle.oracle()
    lat, _, _ = workload_inputs()
    import g4gpu
    ns = nthreads if kind == "port" else 2
    cur = flat_top(NS)[NS // 2 - ns // 2:NS // 2 - ns // 2 + ns]
    sp = T.slice_params(ns, GAMMA0, 2.0, 0.4e-6, 15.0, currents=cur)
    beam = g4gpu.host_load_beam(sp, NS // 2 - ns // 2, NPART, 4, 7, 1, LAMBDA0, 1.0)
    fld = np.zeros((1, ns, NGRID * NGRID), dtype=np.complex128)
    kw = dict(time_run=1)
    if kind == "port":
        kw["nthreads"] = nthreads
    times = []
    state = (beam, fld, [0])
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        p, f, first, _ = lib.run_steps(lat[i % lat.shape[0]:i % lat.shape[0] + 1], GAMMA0, state[0], cur,
                                       LAMBDA0, 1.0, [1], [GRIDMAX], state[1], state[2], **kw)
        dt = time.perf_counter() - t0
        state = (p, f, first)
        if i >= args.warmup:
            times.append(dt)
    tot = sum(times)
    value = ns * args.steps / tot
    line = {"metric": METRIC, "value": value, "unit": "slice-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": "time-dependent SASE, 4096 slices x 8192 particles, ngrid 151, ADI",
                       "sample_per_step": f"{ns} slices x 1 integration step",
                       "cache": "inputs larger than L2"},
            "cpu_baseline": {"value": value, "unit": "slice-steps/s",
                             "cores": nthreads if kind == "port" else 1, "kind": kind,
                             "sample": f"{ns} full-size slices per step, {args.steps} timed steps"},
            "e2e": {"value": value, "unit": "slice-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-steps", type=int, default=None, help="timed steps of the plain form")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--nslice", type=int, default=None,
                    help="slices of the window (default 4096); smaller values are for profiling only")
    ap.add_argument("--forms", default="mixed,plain", help="forms to time: mixed, plain or both")
    args = ap.parse_args()
    global NS
    if args.nslice:
        NS = args.nslice
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)

    ws, rank, local = dist_setup()
    import torch
    torch.cuda.set_device(local)
    import g4gpu
    lat, sp, cur = workload_inputs()
    beam_pinned = torch.empty((NS, NPART, 6), dtype=torch.float64).pin_memory()
    beam = beam_pinned.numpy()
    g4gpu.host_load_beam(sp, 0, NPART, 4, 7, 1, LAMBDA0, 1.0, out=beam)

    peak, peak_kind = measured_peaks()
    sampler = ClockSampler(local)
    barrier(ws)
    sampler.start()
    # headline: mixed form
    hm, ms_m, st_m = time_form(g4gpu, torch, g4gpu.MIXED, beam, cur, lat, args.steps, args.warmup)
    barrier(ws)
    clocks = sampler.stop()
    ms_m = max_over_ranks(ws, ms_m)
    # plain FP64 form, same initial state and steps
    psteps = args.plain_steps if args.plain_steps is not None else args.steps
    do_plain = "plain" in args.forms
    if do_plain:
        hp, ms_p, st_p = time_form(g4gpu, torch, g4gpu.PLAIN, beam, cur, lat, psteps, args.warmup)
        ms_p = max_over_ranks(ws, ms_p)
    # error of the mixed form against the plain one after the same steps
    err = None
    if do_plain and psteps == args.steps:
        bm, fm = hm.diag(1)
        bp, fp = hp.diag(1)
        pw_m, pw_p = fm[0][:, 0], fp[0][:, 0]
        err = {"power_max_rel": float(np.max(np.abs(pw_m - pw_p)) / max(np.max(np.abs(pw_p)), 1e-300)),
               "energy_rel": float(abs(pw_m.sum() / pw_p.sum() - 1)) if pw_p.sum() > 0 else None,
               "bunching_max_rel": float(np.max(np.abs(bm[:, 24] - bp[:, 24])) / np.max(np.abs(bp[:, 24]))),
               "after_steps": args.warmup + args.steps}
    hm.close()
    if do_plain:
        hp.close()

    value = NS * ws / (ms_m / args.steps / 1e3)
    plain_value = NS * ws / (ms_p / psteps / 1e3) if do_plain else None
    launches = sum(v[0] for v in st_m.values())

    def kernel_table(st, mixed):
        # the mixed form's deposition + ADI runs as one fused kernel when the slice
        # fits in shared memory; it is accounted under the adi_x class
        fused = mixed and NGRID <= 168
        tot = max(sum(x[1] for x in st.values()), 1e-12)
        out = {}
        for k, (n, ms) in st.items():
            if n == 0:
                continue
            name = "field" if (fused and k == "adi_x") else k
            avg = ms / n
            ab = kernel_alg_bytes(name, mixed)
            row = {"launches": n, "ms_total": ms, "ms_avg": avg, "share": ms / tot}
            if ab is not None:
                row["alg_bytes"] = ab
                row["achieved_gbs"] = ab / (avg / 1e3) / 1e9
                row["frac_hbm"] = row["achieved_gbs"] / peak
            out[name] = row
        return out

    kernels = kernel_table(st_m, True)
    kernels_plain = kernel_table(st_p, False) if do_plain else None
    dom = max(kernels, key=lambda k: kernels[k]["ms_total"])
    dk = kernels[dom]

    line = {"metric": METRIC, "value": value, "unit": "slice-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_m / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": "time-dependent SASE, 4096 slices x 8192 particles, ngrid 151, "
                                   "ADI, 4x110-period planar undulator with FODO, shot noise seed 7",
                       "form": "mixed (FP32 field/solver/deposition, FP64 phase)",
                       "cache": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{ws}"},
            "forms": {"mixed": {"value": value, "ms_per_step": ms_m / args.steps},
                      "plain_fp64": ({"value": plain_value, "ms_per_step": ms_p / psteps,
                                      "steps": psteps, "kernels": kernels_plain} if do_plain else None)},
            "mixed_error_vs_plain": err,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": dk.get("achieved_gbs"), "peak": peak,
                         "unit": "GB/s", "frac": dk.get("frac_hbm"), "traffic": None,
                         "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                         "alg_bytes_per_launch": dk.get("alg_bytes"), "ms_per_launch": dk["ms_avg"]},
            "kernels": kernels, "gpu_launches": launches, "clocks": clocks}

    if rank == 0 and not args.no_e2e:
        field_pinned = torch.zeros((NS, NGRID * NGRID, 2), dtype=torch.float64).pin_memory()
        t, h2d, d2h = e2e_window(g4gpu, torch, g4gpu.MIXED, beam_pinned, cur, field_pinned, lat,
                                 args.steps, 2)
        line["e2e"] = {"value": NS * args.steps / t, "unit": "slice-steps/s",
                       "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
                       "window": f"upload beam+field, {args.steps} steps with per-step diagnostics read-back, download"}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
