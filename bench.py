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
                      reported. `e2e` times whole runs through the ABI with host
                      buffers, as Gencore::run tracks a beam through the whole
                      lattice: upload of beam and field from pinned memory, every
                      step of the 443-step lattice with its per-slice diagnostics
                      read back, download of the final beam and field.
                      `e2e_short_window` does the same over K steps only.
  --impl reference    the CPU implementation of the step on the host cores, all
                      threads: the reference compiled from its own sources where
                      it is built (oracle/_ref), else the C restatement of it
                      (oracle/g4oracle.c), on a bounded sample of the workload.

Under torchrun (N > 1) every rank runs its own window on its GPU (independent
replicas, weak scaling); the slowest rank's time sets the value. The environment
variable G4_BENCH_GLOO selects the gloo backend for the ranks' barrier and
reduction (CPU tests of the multi-process path); NCCL otherwise.
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
WORKLOAD = ("time-dependent SASE, 4096 slices x 8192 particles, ngrid 151, ADI, 4x110-period planar undulator "
            "with FODO, shot noise seed 7")
# the resonant companion of the workload: the same beam and lattice at the resonant
# wavelength lambda_u (1 + aw^2) / (2 gamma0^2) = 2.262e-10 m (the workload's 1e-10 m is
# off resonance and does not lase); slippage is then one slice per period
LAMBDA_RES = 0.015 * (1 + 1.7 ** 2) / (2 * GAMMA0 ** 2)


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
        if not dist.is_initialized():
            dist.init_process_group("nccl" if os.environ.get("G4_BENCH_GLOO") is None else "gloo")
    return ws, rank, local


def _on_gpu():
    import torch.distributed as dist
    return dist.get_backend() == "nccl"


def barrier(ws):
    if ws > 1:
        import torch
        import torch.distributed as dist
        dist.barrier()
        if _on_gpu():
            torch.cuda.synchronize()


def max_over_ranks(ws, v):
    """The largest of the ranks' values (every rank gets it): the slowest replica's
    time sets the job's."""
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if _on_gpu() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(ws, slices_per_rank, steps, ms_max):
    """Whole-job slice-steps/s: every rank advances its own window of slices_per_rank
    slices by `steps` steps (independent replicas), and the slowest rank's time
    ms_max bounds the job."""
    return slices_per_rank * ws * steps / (ms_max / 1e3)


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per slice of one launch,
# from the ncu --set full capture of a 608-slice window of the same workload
# (profiles/ncu_full_k_push_f_k_field_fused_f_sase608.md); the traffic of these kernels
# grows in proportion to the slices of a launch, so a full launch's is the per-slice
# figure times the slices.
TRAFFIC_PER_SLICE = {"field": 447986.0, "push": 431960.0}
TRAFFIC_SOURCE = "ncu capture of a 608-slice window, scaled to the launch's slices"
# FP64 instructions (DFMA + DMUL + DADD, thread level) per particle of the plain push and
# per cell of each plain ADI sweep, from ncu captures of a 152-slice window
# (profiles/ncu_fp64_k_push_k_adi_plain_sase152.md); nominal GB300 FP64 rate: 1.25 TFLOP/s
# with FMA counted as two operations, i.e. 625 G FP64 instructions/s.
FP64_INSTR = {"push_per_particle": 414.1, "adi_per_cell": 17.9}
FP64_NOMINAL_GINSTR = 625.0


def fp64_peak(g4gpu, device):
    """The device's FP64 instruction rate, measured by the library's FMA-chain kernel
    (g4gpu_measure_fp64_rate), in G instructions/s; the nominal 1.25 TFLOP/s (625 G
    FMA/s) if the measurement fails."""
    import ctypes
    r = ctypes.c_double()
    if g4gpu.load_library().g4gpu_measure_fp64_rate(device, ctypes.byref(r)) == 0 and r.value > 0:
        return r.value / 1e9, "measured: g4gpu_measure_fp64_rate (independent DFMA chains, CUDA events)"
    return FP64_NOMINAL_GINSTR, "nominal 1.25 TFLOP/s (measurement failed)"


def fp64_roofline(kernels_plain, peak_ginstr, peak_source):
    """The plain form is bound by the FP64 rate: FP64 instructions per launch (ncu
    counts per particle / cell times the launch's particles / cells) over the measured
    launch time, against the device's FP64 instruction rate."""
    out = {"bound": "fp64", "peak_ginstr_s": peak_ginstr, "peak_source": peak_source,
           "instr_source": "ncu dfma+dmul+dadd counts of a 152-slice capture"}
    for k, n in (("push", NS * NPART * FP64_INSTR["push_per_particle"]),
                 ("adi_x", NS * NGRID * NGRID * FP64_INSTR["adi_per_cell"]),
                 ("adi_y", NS * NGRID * NGRID * FP64_INSTR["adi_per_cell"])):
        if k in kernels_plain:
            g = n / (kernels_plain[k]["ms_avg"] / 1e3) / 1e9
            out[k] = {"ginstr_s": g, "frac": g / peak_ginstr}
    return out


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
                  FP64: 20 B per particle)
      step        (the whole step of a slice in one kernel) particles read + written
                  (56 B per particle) and the field read + written (16 B per cell): the
                  step's algorithmic bytes"""
    ns = ns or NS
    ncell = NGRID * NGRID
    if kernel == "push":
        per = (56 * NPART + 8 * ncell) if mixed else (96 * NPART + 32 * ncell)
    elif kernel in ("adi_x", "adi_y"):
        per = (24 if mixed else 48) * ncell
    elif kernel == "field":
        per = 16 * ncell + 20 * NPART
    elif kernel == "step":
        per = 56 * NPART + 16 * ncell
    else:
        return None
    return ns * per


def far_field_spectrum(fd):
    """The window's spectrum as the reference's post-processing forms it
    (examples/Example3-TimeDependent/Example3.py:129-136): |FFT over the slices of
    sqrt(I_ff) exp(i phi_ff)|^2, from each slice's far-field intensity and phase
    (a field record [nslice][cols] in window order)."""
    import g4gpu
    i_ff = fd[:, g4gpu.DF_COLS.index("intensity-farfield")]
    phi = fd[:, g4gpu.DF_COLS.index("phase-farfield")]
    return np.abs(np.fft.fftshift(np.fft.fft(np.sqrt(np.maximum(i_ff, 0.0)) * np.exp(1j * phi)))) ** 2


def mixed_error(hm, hp, after_steps):
    """The mixed handle's slice power and bunching against the plain FP64 handle's
    (both at the same step): the largest slice-power difference over the largest
    slice power, the largest difference of the window's spectrum over its largest
    value, the window energy, the largest bunching difference over the largest
    bunching and absolute. The absolute bunching floor that matters is the shot-noise
    level of the beam, 1/sqrt(npart) = 0.011 for 8192 particles."""
    bm, fm = hm.diag(1)
    bp, fp = hp.diag(1)
    pw_m, pw_p = fm[0][:, 0], fp[0][:, 0]
    db = float(np.max(np.abs(bm[:, 24] - bp[:, 24])))
    sm, sp = far_field_spectrum(fm[0]), far_field_spectrum(fp[0])
    return {"power_max_rel": float(np.max(np.abs(pw_m - pw_p)) / max(np.max(np.abs(pw_p)), 1e-300)),
            "spectrum_max_rel": float(np.max(np.abs(sm - sp)) / max(np.max(sp), 1e-300)),
            "energy_rel": float(abs(pw_m.sum() / pw_p.sum() - 1)) if pw_p.sum() > 0 else None,
            "bunching_max_rel": db / max(float(np.max(np.abs(bp[:, 24]))), 1e-300),
            "bunching_max_abs": db, "bunching_floor_1_over_sqrt_npart": 1.0 / np.sqrt(NPART),
            "max_slice_power_w": float(np.max(pw_p)), "max_bunching": float(np.max(bp[:, 24])),
            "after_steps": after_steps}


def resonant_companion(g4gpu, torch, shapes):
    """The workload's window at the resonant wavelength LAMBDA_RES (one slice of
    slippage per period), which lases from shot noise: the mixed form against the plain
    FP64 form after every module of the 443-step lattice, with the window energy's
    growth. Not timed."""
    lat = T.undulator_lattice(1.7, 0.015, 110, 4, LAMBDA_RES, GAMMA0, quad_k1=1.5, quad_l=0.08)
    cur = flat_top(NS)
    sp = T.slice_params(NS, GAMMA0, 2.0, 0.4e-6, 15.0, currents=cur)
    beam = g4gpu.host_load_beam(sp, 0, NPART, 4, 7, 1, LAMBDA_RES, 1.0)
    hs = []
    for prec in (g4gpu.MIXED, g4gpu.PLAIN):
        cfg = g4gpu.Config(nslice=NS, npart=NPART, ngrid=NGRID, gridmax=GRIDMAX, lambda0=LAMBDA_RES, sample=1.0,
                           gammaref=GAMMA0, precision=prec, time_run=1, device=torch.cuda.current_device())
        h = g4gpu.Handle(cfg)
        h.set_lattice(lat)
        h.load_beam(beam, cur)
        h.load_field(0, np.zeros((NS, NGRID * NGRID), dtype=np.complex128))
        if prec == g4gpu.MIXED and shapes is not None:
            h.set_launch_shapes(*shapes)
        hs.append(h)
    del beam
    out = {"lambda0": LAMBDA_RES, "modules": []}
    nlat = lat.shape[0]
    ends = [i + 1 for i in range(nlat) if lat[i, T.C["aw"]] > 0 and (i + 1 == nlat or lat[i + 1, T.C["aw"]] == 0)]
    done = 0
    for e in ends:
        for h in hs:
            h.run(done, e - done)
        done = e
        row = mixed_error(hs[0], hs[1], e)
        row["window_energy_plain"] = float(hs[1].diag(1)[1][0][:, 0].sum())
        out["modules"].append(row)
    for h in hs:
        h.close()
    e0 = out["modules"][0]["window_energy_plain"]
    out["energy_growth_module1_to_end"] = out["modules"][-1]["window_energy_plain"] / max(e0, 1e-300)
    out["power_max_rel"] = max(m["power_max_rel"] for m in out["modules"])
    out["spectrum_max_rel"] = max(m["spectrum_max_rel"] for m in out["modules"])
    out["bunching_max_rel"] = max(m["bunching_max_rel"] for m in out["modules"])
    return out


def time_form(g4gpu, torch, precision, beam, cur, lat, steps, warmup, profile=True, autotune=False, shapes=None,
              efield=None):
    cfg = g4gpu.Config(nslice=NS, npart=NPART, ngrid=NGRID, gridmax=GRIDMAX, lambda0=LAMBDA0,
                       sample=1.0, gammaref=GAMMA0, precision=precision, time_run=1,
                       device=torch.cuda.current_device())
    h = g4gpu.Handle(cfg)
    h.set_lattice(lat)
    h.load_beam(beam, cur)
    h.load_field(0, np.zeros((NS, NGRID * NGRID), dtype=np.complex128))
    if efield is not None:
        h.set_efield(*efield)
    # launch shapes picked by the library's autotuner (untimed; the state is restored)
    h.shapes = h.autotune() if autotune else None
    if shapes is not None:
        h.set_launch_shapes(*shapes)
        h.shapes = tuple(shapes)
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


# &efield of the space-charge form: the namelist's rmax and ngrid, the long-range loss
# and nz x (2 nphi + 1) short-range modes: 1 (nz 1, nphi 0) and 15 (nz 3, nphi 2)
SC_EFIELDS = ((0.0, 100, 1, 0, True), (0.0, 100, 3, 2, True))


def spacecharge_form(g4gpu, torch, beam, cur, lat, steps, warmup, peak, ms_mixed, shapes):
    """The headline window and form with space charge (&efield, EFieldSolver.cpp) on:
    per setting of SC_EFIELDS the step rate and the two space-charge kernels: the
    moments kernel (first transverse half step of the push, slice moments, radial grid
    extents) is bound by HBM: it reads gamma, x, y, px, py and writes x, y, px, py (36 B
    per particle); the field kernel (long-range loss, then per slice the radial-mode
    source in shared memory, the tridiagonal solves and the gather) by instruction
    issue: its work is counted in particle-modes (particles x modes, deposited and
    gathered)."""
    out = {"config": "headline window and lattice, mixed form, launch shapes of the headline",
           "settings": []}
    for ef in SC_EFIELDS:
        h, ms, st = time_form(g4gpu, torch, g4gpu.MIXED, beam, cur, lat, steps, warmup, shapes=shapes, efield=ef)
        h.close()
        rmax, ngr, nz, nphi, lr = ef
        modes = nz * (2 * nphi + 1) if (nz > 0 and ngr > 2) else 0
        n_m, ms_mo = st.get("sc", (0, 0.0))
        n_f, ms_fi = st.get("sc_field", (0, 0.0))
        mo_avg = ms_mo / max(n_m, 1)
        fi_avg = ms_fi / max(n_f, 1)
        alg = 36 * NS * NPART
        row = {"efield": {"rmax": rmax, "ngrid": ngr, "nz": nz, "nphi": nphi, "longrange": lr},
               "modes": modes, "value": NS * steps / (ms / 1e3), "unit": "slice-steps/s",
               "ms_per_step": ms / steps, "overhead_vs_mixed": ms / steps / ms_mixed - 1,
               "kernels": {"sc_moments": {"ms_avg": mo_avg, "alg_bytes": alg,
                                          "achieved_gbs": alg / (mo_avg / 1e3) / 1e9,
                                          "frac_hbm": alg / (mo_avg / 1e3) / 1e9 / peak},
                           "sc_field": {"ms_avg": fi_avg,
                                        "particle_modes_per_s": (NS * NPART * modes / (fi_avg / 1e3)
                                                                 if modes else None)}},
               "launches_per_step": {k: v[0] / steps for k, v in st.items() if v[0]}}
        out["settings"].append(row)
    out["value"] = out["settings"][0]["value"]
    out["unit"] = "slice-steps/s"
    return out


def cpu_baseline_sc(efield, target_seconds=8.0):
    """The oracle port with space charge on a bounded sample of the window (slices from
    its middle, full size: 8192 particles, ngrid 151), one host thread (the reference
    runs the short-range field slice after slice: the radial grid extent is carried)."""
    import g4oracle
    import build_oracle
    import g4gpu
    build_oracle.build_oracle()
    lib = g4oracle.oracle()
    lat, _, _ = workload_inputs()
    ns = 8
    cur = flat_top(NS)[NS // 2 - ns // 2:NS // 2 - ns // 2 + ns]
    sp = T.slice_params(ns, GAMMA0, 2.0, 0.4e-6, 15.0, currents=cur)
    beam = g4gpu.host_load_beam(sp, NS // 2 - ns // 2, NPART, 4, 7, 1, LAMBDA0, 1.0)
    fld = np.zeros((1, ns, NGRID * NGRID), dtype=np.complex128)
    lib.set_efield(*efield)
    try:
        t0 = time.perf_counter()
        lib.run_steps(lat[:1], GAMMA0, beam, cur, LAMBDA0, 1.0, [1], [GRIDMAX], fld, [0], time_run=1)
        dt = time.perf_counter() - t0
        nsteps = int(max(1, min(lat.shape[0], target_seconds / max(dt, 1e-6))))
        lib.set_efield(*efield)
        t0 = time.perf_counter()
        lib.run_steps(lat[:nsteps], GAMMA0, beam, cur, LAMBDA0, 1.0, [1], [GRIDMAX], fld, [0], time_run=1)
        dt = time.perf_counter() - t0
    finally:
        lib.set_efield()
    return {"value": ns * nsteps / dt, "unit": "slice-steps/s", "cores": 1, "kind": "port",
            "sample": f"{ns} slices x {nsteps} steps of the window with &efield {list(efield)}, "
                      f"plain FP64, 1 host thread, {dt:.1f} s"}


ENSEMBLE_SEED, ENSEMBLE_RUNS = 11, 64


def ensemble_runs(nrun=ENSEMBLE_RUNS, seed=ENSEMBLE_SEED):
    """The uneven ensemble: per run (nslice, npart, ngrid, taper) drawn from `seed`:
    nslice uniform in 64..1024, npart from {2048, 4096, 8192, 16384}, ngrid from
    {101, 151, 201, 255}, linear aw taper uniform in [-2 %, 0] over the 4 modules."""
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(64, 1025)), int(rng.choice([2048, 4096, 8192, 16384])),
             int(rng.choice([101, 151, 201, 255])), float(rng.uniform(-0.02, 0.0))) for _ in range(nrun)]


def ensemble_member(r, ns, npart, ngrid, taper, g4gpu):
    lat = T.undulator_lattice(1.7, 0.015, 110, 4, LAMBDA0, GAMMA0, quad_k1=1.5, quad_l=0.08, taper=taper)
    cur = flat_top(ns)
    sp = T.slice_params(ns, GAMMA0, 2.0, 0.4e-6, 15.0, currents=cur)
    beam = g4gpu.host_load_beam(sp, 0, npart, 4, ENSEMBLE_SEED + r, 1, LAMBDA0, 1.0)
    return lat, beam, cur, np.zeros((ns, ngrid * ngrid), dtype=np.complex128)


def diag_error(b, f, b0, f0):
    """Slice-power error relative to the largest slice power, the window spectrum's
    error relative to its largest value (far_field_spectrum), and bunching error
    relative to the largest bunching and absolute (bunching |<exp(i theta)>| lies in
    [0, 1]; near the shot-noise level of a quiet beam only the absolute error means
    anything), of (b, f) against (b0, f0)."""
    p, p0 = f[0][:, 0], f0[0][:, 0]
    db = float(np.max(np.abs(b[:, 24] - b0[:, 24])))
    s, s0 = far_field_spectrum(f[0]), far_field_spectrum(f0[0])
    return {"power_max_rel": float(np.max(np.abs(p - p0)) / max(np.max(np.abs(p0)), 1e-300)),
            "spectrum_max_rel": float(np.max(np.abs(s - s0)) / max(np.max(s0), 1e-300)),
            "bunching_max_rel": db / max(float(np.max(np.abs(b0[:, 24]))), 1e-300),
            "bunching_max_abs": db}


def batched_form(g4gpu, torch, steps, warmup, peak, nrun=ENSEMBLE_RUNS, nerr=4):
    """The uneven ensemble as one batch (one handle and stream per run, each run's
    steps one captured CUDA graph, launch shapes from the autotuner), mixed form.
    Timed: `steps` steps of every run after `warmup`. Error: the nerr smallest runs
    against the plain FP64 form over the same steps."""
    dev = torch.cuda.current_device()
    runs = ensemble_runs(nrun)
    cfgs = [g4gpu.Config(nslice=ns, npart=npart, ngrid=ng, gridmax=GRIDMAX, lambda0=LAMBDA0, sample=1.0,
                         gammaref=GAMMA0, precision=g4gpu.MIXED, time_run=1, device=dev)
            for (ns, npart, ng, _) in runs]
    t_load = time.perf_counter()
    b = g4gpu.Batch(cfgs)
    shapes = {}
    for r, (m, (ns, npart, ng, taper)) in enumerate(zip(b.members, runs)):
        lat, beam, cur, fld = ensemble_member(r, ns, npart, ng, taper, g4gpu)
        m.set_lattice(lat)
        m.load_beam(beam, cur)
        m.load_field(0, fld)
        shapes[f"npart {npart} ngrid {ng}"] = list(m.autotune())
    t_load = time.perf_counter() - t_load
    b.run(0, warmup)
    b.synchronize()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.run(warmup, steps)
    b.synchronize()
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    slices = sum(x[0] for x in runs)
    alg = sum(ns * (56 * npart + 16 * ng * ng) for (ns, npart, ng, _) in runs)
    # error of the smallest runs against the plain FP64 form
    order = sorted(range(nrun), key=lambda i: runs[i][0] * runs[i][1])[:nerr]
    errs = []
    for i in order:
        ns, npart, ng, taper = runs[i]
        bm, fm = b.members[i].diag(1)
        lat, beam, cur, fld = ensemble_member(i, ns, npart, ng, taper, g4gpu)
        cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ng, gridmax=GRIDMAX, lambda0=LAMBDA0, sample=1.0,
                           gammaref=GAMMA0, precision=g4gpu.PLAIN, time_run=1, device=dev)
        with g4gpu.Handle(cfg) as hp:
            hp.set_lattice(lat)
            hp.load_beam(beam, cur)
            hp.load_field(0, fld)
            hp.run(0, warmup + steps)
            bp, fp = hp.diag(1)
        errs.append(dict(run=i, nslice=ns, npart=npart, ngrid=ng, **diag_error(bm, fm, bp, fp)))
    b.close()
    value = slices * steps / (ms / 1e3)
    achieved = alg * steps / (ms / 1e3) / 1e9
    return {"value": value, "unit": "slice-steps/s", "ms_per_step": ms / steps, "runs": nrun,
            "slices": slices, "particles": int(sum(x[0] * x[1] for x in runs)),
            "draws": "nslice U{64..1024}, npart {2048..16384}, ngrid {101,151,201,255}, taper U[-2%,0], seed 11",
            "launch": "one handle + stream per run; each run's timed steps one CUDA graph (captured in the "
                      "timed region: kernels take the ring start by value, so a graph is per starting state)",
            "launch_shapes": shapes, "setup_s": t_load,
            "roofline_step": {"alg_bytes_per_step": alg, "achieved_gbs": achieved, "peak": peak,
                              "frac": achieved / peak},
            "error_vs_plain": {"runs": errs, "after_steps": warmup + steps,
                               "power_max_rel": max(e["power_max_rel"] for e in errs),
                               "spectrum_max_rel": max(e["spectrum_max_rel"] for e in errs),
                               "bunching_max_rel": max(e["bunching_max_rel"] for e in errs)}}


HARM_NS, HARM_NPART, HARM_NGRID, HARM_GRIDMAX, HARM_H = 2048, 16384, 255, 1.5e-4, (1, 3, 5)


def harmonic_fft_form(g4gpu, torch, steps, warmup, peak, nsub=256, ns=None):
    """The harmonic FFT workload, mixed form: 2048 slices x 16384 particles (nbins 8,
    shot noise seed 7, delgam 1.0, the flat-top current), fields at the 1st, 3rd and
    5th harmonic on ngrid 255 over gridmax 1.5e-4 m, FieldSolverFFT, the undulator of
    the headline workload. Error: power and bunching at harmonics 1..5 against the
    plain FP64 form on the first `nsub` slices (with the field slipping towards the
    head and zero entering at slice 0, the first slices of a window evolve exactly as
    a window of those slices alone)."""
    dev = torch.cuda.current_device()
    ns, npart, ng = ns or HARM_NS, HARM_NPART, HARM_NGRID
    nsub = min(nsub, ns)
    ncell = ng * ng
    lat, _, _ = workload_inputs(ns)
    cur = flat_top(ns)
    sp = T.slice_params(ns, GAMMA0, 1.0, 0.4e-6, 15.0, currents=cur)
    beam = g4gpu.host_load_beam(sp, 0, npart, 8, 7, 1, LAMBDA0, 1.0)
    zero = np.zeros((ns, ncell), dtype=np.complex128)

    def handle(precision, n):
        cfg = g4gpu.Config(nslice=n, npart=npart, ngrid=ng, harm=list(HARM_H), gridmax=[HARM_GRIDMAX] * 3,
                           lambda0=LAMBDA0, sample=1.0, gammaref=GAMMA0, precision=precision,
                           solver=g4gpu.SOLVER_FFT, time_run=1, device=dev)
        h = g4gpu.Handle(cfg)
        h.set_lattice(lat)
        h.load_beam(beam[:n], cur[:n])
        for k in range(len(HARM_H)):
            h.load_field(k, zero[:n])
        return h

    h = handle(g4gpu.MIXED, ns)
    nlat = lat.shape[0]
    for i in range(warmup):
        h.run(i % nlat, 1)
    h.synchronize()
    stream = torch.cuda.ExternalStream(h.stream())
    h.reset_stats()
    h.set_profiling(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        h.run((warmup + i) % nlat, 1)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    st = h.kernel_stats()
    h.set_profiling(False)
    nh = 5
    bm, fm = h.diag(nh)
    h.close()
    with handle(g4gpu.PLAIN, nsub) as hp:
        hp.run(0, warmup + steps)
        bp, fp = hp.diag(nh)
    tot = max(sum(x[1] for x in st.values()), 1e-12)
    kern = {k: {"launches": n, "ms_total": t, "ms_avg": t / n, "share": t / tot} for k, (n, t) in st.items() if n}
    # FFT solve of one field over the window: at least the field read and written and
    # the source read once (FP32 complex: 24 B per cell); the three-pass transform
    # (rows, columns, rows through global memory) moves 56 B per cell
    fft_alg = len(HARM_H) * ns * ncell * 24.0 * steps
    fft_ms = st["fft"][1]
    out = {"value": ns * steps / (ms / 1e3), "unit": "slice-steps/s", "ms_per_step": ms / steps,
           "config": f"{ns} slices x {npart} particles (nbins 8), harmonics {list(HARM_H)}, ngrid {ng}, "
                     f"gridmax {HARM_GRIDMAX} m, FieldSolverFFT, delgam 1.0, shot noise seed 7",
           "kernels": kern}
    if fft_ms > 0:
        a = fft_alg / (fft_ms / 1e3) / 1e9
        out["fft_roofline"] = {"bound": "hbm", "alg_bytes_per_cell": 24, "design_bytes_per_cell": 56,
                               "achieved_gbs": a, "peak": peak, "frac": a / peak,
                               "ms_per_field_solve": fft_ms / (steps * len(HARM_H))}
    pw, spec = {}, {}
    for k, hk in enumerate(HARM_H):
        a, b = fm[k][:nsub, 0], fp[k][:, 0]
        pw[f"h{hk}"] = float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
        sa, sb = far_field_spectrum(fm[k][:nsub]), far_field_spectrum(fp[k])
        spec[f"h{hk}"] = float(np.max(np.abs(sa - sb)) / max(np.max(sb), 1e-300))
    bun = {}
    for j in range(nh):
        a, b = bm[:nsub, 24 + 2 * j], bp[:, 24 + 2 * j]
        bun[f"h{j + 1}"] = float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
    out["error_vs_plain"] = {"slices": nsub, "after_steps": warmup + steps, "power_max_rel": pw,
                             "spectrum_max_rel": spec, "bunching_max_rel": bun}
    return out


def learned_form(g4gpu, torch, lat, beam, cur, steps, warmup, nseeds=64, train_slices=64, max_coarse=63,
                 check_every=8, tol=0.01, gamma0=GAMMA0, seed_power=0.0, time_run=1, shotnoise=1,
                 substeps=True, factor=4):
    """The coarse-step closure on the full window. Training data: fine (one-period)
    runs of a train_slices-slice window of the same beam over seeds 100..100+nseeds-1
    for the first max_coarse coarse steps (4 periods each), mixed form; the network
    (32 -> 256 -> 256 -> 256 -> 4, BF16 tensor-core GEMMs, FP32 master weights) is
    trained with Adam on the GPU. Timed: `steps` coarse steps with the closure after
    `warmup`, with the fine solve judging every check_every coarse steps (fallback
    above tol relative slice-power error). Throughput counts the fine slice-steps
    the coarse steps cover. Error: against the plain FP64 fine run. substeps: a
    coarse step pushes once over its 4 periods, then deposits and slips period by
    period from interpolated phases, then diffracts once (g4gpu_set_field_substeps);
    else it is one whole step of 4 periods. factor: the periods of a coarse step."""
    import learned
    dev = torch.cuda.current_device()
    waist, u0, c0 = 30e-6, 1.0, 1.0
    base = dict(npart=NPART, ngrid=NGRID, gridmax=GRIDMAX, lambda0=LAMBDA0, sample=1.0, gammaref=gamma0,
                precision=g4gpu.MIXED, time_run=time_run, device=dev)
    sp = T.slice_params(train_slices, gamma0, 2.0, 0.4e-6, 15.0, current=3000.0)
    # initial field of every slice: zero (SASE from shot noise) or a Gaussian seed
    if seed_power > 0:
        slice_field = g4gpu.host_gauss_hermite(T.gauss_field_par(LAMBDA0, seed_power, 30e-6), GRIDMAX, NGRID)
    else:
        slice_field = np.zeros(NGRID * NGRID, dtype=np.complex128)
    t0 = time.perf_counter()
    X, Tg, clat, fs, fc = learned.generate_training_data(
        dict(base, nslice=train_slices), lat, range(100, 100 + nseeds), sp, NPART, 4,
        np.repeat(slice_field[None, :], train_slices, axis=0), waist, u0, c0, factor=factor,
        max_coarse=max_coarse, shotnoise=shotnoise, substeps=substeps)
    t_gen = time.perf_counter() - t0
    fine_slice_steps = int(nseeds * train_slices * int(fs[max_coarse - 1] + fc[max_coarse - 1]))
    t0 = time.perf_counter()
    m = g4gpu.MLP(32, 256, 4, seed=0, device=dev)
    curve = m.train(X, Tg, epochs=8, batch=512, lr=1e-3, seed=0)
    t_train = time.perf_counter() - t0
    fld = np.repeat(slice_field[None, :], NS, axis=0)
    hf, hc = learned.make_pair(dict(base, nslice=NS), lat, clat, beam, cur, fld, m, waist, u0, c0,
                               fc if substeps else None)
    hc.run_learned(hf, 0, warmup, fs, fc, check_every=check_every, tol=tol)
    hc.synchronize()
    hf.synchronize()
    stream = torch.cuda.ExternalStream(hc.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    nchk, nfb, emax = hc.run_learned(hf, warmup, steps, fs, fc, check_every=check_every, tol=tol)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    nfine = int(fs[warmup + steps - 1] + fc[warmup + steps - 1])
    covered = nfine - int(fs[warmup])
    bl, fl = hc.diag(1)
    hf.close()
    hc.close()
    # references after the same distance: the plain FP64 fine run, and coarse steps
    # without the closure
    cfgp = g4gpu.Config(**dict(base, nslice=NS, precision=g4gpu.PLAIN))
    with g4gpu.Handle(cfgp) as hp:
        hp.set_lattice(lat)
        hp.load_beam(beam, cur)
        hp.load_field(0, fld)
        hp.run(0, nfine)
        bp, fp = hp.diag(1)
    with g4gpu.Handle(g4gpu.Config(**dict(base, nslice=NS))) as hcn:
        hcn.set_lattice(clat)
        if substeps:
            hcn.set_field_substeps(fc)
        hcn.load_beam(beam, cur)
        hcn.load_field(0, fld)
        hcn.run(0, warmup + steps)
        bn, fn = hcn.diag(1)
    m.close()
    return {"value": NS * covered / (ms / 1e3), "unit": "slice-steps/s (fine steps covered)",
            "ms_per_coarse_step": ms / steps, "coarse_steps": steps, "fine_steps_covered": covered,
            "judge": {"check_every": check_every, "tol": tol, "checks": nchk, "fallbacks": nfb,
                      "max_check_err": emax},
            "error_vs_plain": dict(diag_error(bl, fl, bp, fp), after_fine_steps=nfine,
                                   bunching_floor_1_over_sqrt_npart=1.0 / np.sqrt(NPART),
                                   bunching_note="the judge checks slice power; bunching is compared in "
                                                 "absolute terms against the shot-noise level "
                                                 "1/sqrt(npart) of the beam"),
            "coarse_without_closure_error_vs_plain": diag_error(bn, fn, bp, fp),
            "coarse_step": (f"push over {factor} periods; per period the deposition from interpolated phases "
                            f"and positions and the slippage; one diffraction over {factor} periods" if substeps
                            else f"one whole step of {factor} periods (push, field solve and slippage)"),
            "beam": f"gamma0 {gamma0}, 4096 slices x {NPART} particles, the config-0 lattice, "
                    + (f"{seed_power:g} W Gaussian seed (waist 30 um) in every slice, " if seed_power > 0
                       else "no seed, ")
                    + ("time-dependent (slippage)" if time_run else "steady state (independent slices)")
                    + (", shot noise" if shotnoise else ", quiet loading"),
            "training": {"samples": int(X.shape[0]), "fine_slice_steps": fine_slice_steps,
                         "seeds": f"100..{99 + nseeds}", "window": f"{train_slices} slices x {NPART} particles",
                         "epochs": len(curve), "loss_first": float(curve[0]), "loss_last": float(curve[-1]),
                         "generate_s": t_gen, "train_s": t_train}}


E2E_WINDOWS = 11       # timed windows of K steps
E2E_RUNS = 5           # timed whole-lattice runs


def e2e_window(g4gpu, torch, precision, beam_pinned, cur, field_pinned, lat, steps, reps, outs, shapes=None):
    """Track windows through the ABI with host buffers: upload, `steps` steps with the
    per-slice diagnostics of every step (recorded on the device, each step's record
    read back while the later steps run), download of beam and field. One warm-up
    window, `reps` timed windows (their wall times are returned), then one window with
    a synchronisation between its phases to split its time."""
    cfg = g4gpu.Config(nslice=NS, npart=NPART, ngrid=NGRID, gridmax=GRIDMAX, lambda0=LAMBDA0,
                       sample=1.0, gammaref=GAMMA0, precision=precision, time_run=1,
                       device=torch.cuda.current_device())
    h = g4gpu.Handle(cfg)
    h.set_lattice(lat)
    if shapes is not None:  # the launch shapes of the headline form (its autotuner's)
        h.set_launch_shapes(*shapes)
    out_beam, out_field = outs
    cur_np = np.ascontiguousarray(cur)
    diag_out = (np.zeros((steps, NS, len(g4gpu.DB_COLS) + 2)), np.zeros((steps, 1, NS, len(g4gpu.DF_COLS))))
    times = []
    gpu_phases = []
    d2h_diag = 0
    stream = torch.cuda.ExternalStream(h.stream())
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for rep in range(reps + 2):
        # the first window is the warm-up; the last one is split into its phases
        split = rep == reps + 1
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev[0].record(stream)
        h.load_beam_ptr(beam_pinned.data_ptr(), cur_np.ctypes.data)
        h.load_field_ptr(0, field_pinned.data_ptr())
        ev[1].record(stream)
        if split:
            h.synchronize()
            t_up = time.perf_counter()
        # the steps, with the per-slice diagnostics of every step recorded on the
        # device and read back once (g4gpu_run_diag)
        bd, fd = h.run_diag(0, steps, 1, out=diag_out)
        ev[2].record(stream)
        d2h_diag = bd.nbytes + fd.nbytes
        if split:
            t_steps = time.perf_counter()
        h.get_beam(out_beam.numpy())
        h.get_field(0, out_field.numpy().view(np.complex128).reshape(NS, NGRID * NGRID))
        ev[3].record(stream)
        t1 = time.perf_counter()
        if split:
            phases = {"upload_s": t_up - t0, "steps_with_diag_s": t_steps - t_up, "download_s": t1 - t_steps}
        elif rep > 0:
            times.append(t1 - t0)
            ev[3].synchronize()
            # device time between the phase boundaries on the handle's stream (no
            # synchronisation added inside the window)
            gpu_phases.append([ev[k].elapsed_time(ev[k + 1]) / 1e3 for k in range(3)])
    h.close()
    h2d = beam_pinned.numel() * 8 + cur_np.nbytes + field_pinned.numel() * 8
    d2h = d2h_diag + out_beam.numel() * 8 + out_field.numel() * 8
    phases["device_phases_s_per_window"] = gpu_phases
    return times, h2d, d2h, phases


def lattice_step_times(g4gpu, torch, beam, cur, lat, shapes):
    """Device time of every step of the whole lattice (CUDA events on the handle's stream
    between single-step calls), mixed form with the headline's launch shapes: how a step's
    cost moves over a run as the beam bunches and its energies part."""
    cfg = g4gpu.Config(nslice=NS, npart=NPART, ngrid=NGRID, gridmax=GRIDMAX, lambda0=LAMBDA0,
                       sample=1.0, gammaref=GAMMA0, precision=g4gpu.MIXED, time_run=1,
                       device=torch.cuda.current_device())
    nlat = lat.shape[0]
    with g4gpu.Handle(cfg) as h:
        h.set_lattice(lat)
        if shapes is not None:
            h.set_launch_shapes(*shapes)
        h.load_beam(beam, cur)
        h.load_field(0, np.zeros((NS, NGRID * NGRID), dtype=np.complex128))
        h.synchronize()
        stream = torch.cuda.ExternalStream(h.stream())
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(nlat + 1)]
        ev[0].record(stream)
        for i in range(nlat):
            h.run(i, 1)
            ev[i + 1].record(stream)
        h.synchronize()
        ms = np.array([ev[i].elapsed_time(ev[i + 1]) for i in range(nlat)])
    return {"steps": nlat, "total_s": float(ms.sum() / 1e3), "mean_ms": float(ms.mean()),
            "first_step_ms": float(ms[0]), "steps_2_to_21_mean_ms": float(ms[1:21].mean()),
            "last_20_mean_ms": float(ms[-20:].mean()), "max_ms_after_first": float(ms[1:].max())}


def cpu_sample(lib, ns):
    """ns full-size slices (8192 particles, ngrid 151) from the middle of the
    workload's window, loaded by the checker library's own bit-exact loader (the
    quiet loading and shot-noise stream of the window's slices), with zero field."""
    cur = flat_top(NS)[NS // 2 - ns // 2:NS // 2 - ns // 2 + ns]
    sp = T.slice_params(ns, GAMMA0, 2.0, 0.4e-6, 15.0, currents=cur)
    beam = lib.load_beam(sp, NS // 2 - ns // 2, NPART, 4, 7, 1, LAMBDA0, 1.0)
    return beam, cur, np.zeros((1, ns, NGRID * NGRID), dtype=np.complex128)


def cpu_baseline(nthreads, target_seconds=20.0):
    """Times the oracle port (oracle/g4oracle.c, bit-exact with the reference) on a
    bounded sample of the workload: full-size slices (8192 particles, ngrid 151), as
    many steps of the lattice as fit and then as many slices (a multiple of the
    threads) as fill about target_seconds, on all host threads."""
    import g4oracle
    import build_oracle
    build_oracle.build_oracle()
    lib = g4oracle.oracle()
    lat, _, _ = workload_inputs()
    threads = max(nthreads, 1)
    ns = threads
    beam, cur, fld = cpu_sample(lib, ns)
    kw = dict(time_run=1, nthreads=threads)
    t0 = time.perf_counter()
    lib.run_steps(lat[:1], GAMMA0, beam, cur, LAMBDA0, 1.0, [1], [GRIDMAX], fld, [0], **kw)
    dt1 = time.perf_counter() - t0
    nsteps = int(max(1, min(lat.shape[0], target_seconds / max(dt1, 1e-6))))
    ns = threads * int(max(1, round(target_seconds / max(dt1 * nsteps, 1e-6))))
    beam, cur, fld = cpu_sample(lib, ns)
    t0 = time.perf_counter()
    lib.run_steps(lat[:nsteps], GAMMA0, beam, cur, LAMBDA0, 1.0, [1], [GRIDMAX], fld, [0], **kw)
    dt = time.perf_counter() - t0
    return {"value": ns * nsteps / dt, "unit": "slice-steps/s", "cores": threads, "kind": "port",
            "sample": f"{ns} slices x {nsteps} steps of the workload (8192 particles, ngrid 151, "
                      f"plain FP64), {threads} host threads, {dt:.1f} s"}


def run_reference_arm(args):
    """The CPU implementation of the step on the host cores, on the workload's
    metric and config: the C restatement of the reference (oracle/g4oracle.c, which is
    bit-exact with the reference compiled from its own sources), all host threads,
    each step a bounded sample of the window (full-size slices, one per thread times
    REF_SLICES_PER_THREAD). The reference itself is x86 code built where its source
    tree is; that tree is not present where this arm runs, so the port stands in."""
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    import g4oracle
    import build_oracle
    build_oracle.build_oracle()
    nthreads = os.cpu_count() or 1
    lib = g4oracle.oracle()
    lat, _, _ = workload_inputs()
    ns = nthreads * REF_SLICES_PER_THREAD
    beam, cur, fld = cpu_sample(lib, ns)
    kw = dict(time_run=1, nthreads=nthreads)
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
    sample = f"{ns} full-size slices of the window per step (8192 particles, ngrid 151), {args.steps} timed steps"
    line = {"metric": METRIC, "value": value, "unit": "slice-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "form": "plain FP64 (the reference's arithmetic)",
                       "cache": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{ws}",
                       "sample_per_step": sample},
            "cpu_baseline": {"value": value, "unit": "slice-steps/s", "cores": nthreads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "slice-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


REF_SLICES_PER_THREAD = 2


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-steps", type=int, default=None, help="timed steps of the plain form")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=None,
                    help="steps of a timed e2e run (default: the whole lattice)")
    ap.add_argument("--no-full-lattice", action="store_true",
                    help="skip the mixed form's error after the whole 443-step lattice and its resonant companion")
    ap.add_argument("--nslice", type=int, default=None,
                    help="slices of the window (default 4096); smaller values are for profiling only")
    ap.add_argument("--ngrid", type=int, default=None,
                    help="grid points of the window (default 151); other values are for profiling only")
    ap.add_argument("--forms", default="mixed,plain,batched,harmonic,learned,spacecharge",
                    help="forms to time besides the mixed headline: plain, batched, harmonic, learned, "
                         "spacecharge")
    ap.add_argument("--harmonic-slices", type=int, default=None,
                    help="slices of the harmonic FFT window (default 2048); smaller values are for profiling only")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch shapes of the mixed form instead of autotuning them")
    ap.add_argument("--launch-shapes", default=None,
                    help="push_block,field_threads,field_kernel for the mixed form instead of autotuning "
                         "(for profiling captures without the tuner's trial launches)")
    args = ap.parse_args()
    global NS, NGRID
    if args.nslice:
        NS = args.nslice
    if args.ngrid:
        NGRID = args.ngrid
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
    # the end-to-end windows' host buffers, pinned once at start-up as an application
    # allocates its I/O buffers
    if rank == 0 and not args.no_e2e:
        field_pinned = torch.zeros((NS, NGRID * NGRID, 2), dtype=torch.float64).pin_memory()
        e2e_out = (torch.empty_like(beam_pinned).pin_memory(), torch.empty_like(field_pinned).pin_memory())

    peak, peak_kind = measured_peaks()
    sampler = ClockSampler(local)
    barrier(ws)
    sampler.start()
    # headline: mixed form
    fixed = tuple(int(v) for v in args.launch_shapes.split(",")) if args.launch_shapes else None
    hm, ms_m, st_m = time_form(g4gpu, torch, g4gpu.MIXED, beam, cur, lat, args.steps, args.warmup,
                               autotune=not args.no_autotune and fixed is None, shapes=fixed)
    shapes = hm.shapes
    barrier(ws)
    clocks = sampler.stop()
    ms_m = max_over_ranks(ws, ms_m)
    # end to end through the ABI, right after the headline: in the process state of a
    # single run, before the comparison runs and the other forms allocate and free their
    # handles and host buffers (after them, the same copies ran up to six times slower)
    e2e_res = {}
    if rank == 0 and not args.no_e2e:
        nrun = min(args.e2e_steps or lat.shape[0], lat.shape[0])
        for key, steps, reps, what in (
                ("e2e", nrun, E2E_RUNS, f"one whole run: upload beam+field, all {nrun} steps of the lattice with "
                                        "every step's diagnostics (g4gpu_run_diag), download"),
                ("e2e_short_window", args.steps, E2E_WINDOWS,
                 f"upload beam+field, {args.steps} steps with every step's diagnostics (g4gpu_run_diag), "
                 "download")):
            times, h2d, d2h, phases = e2e_window(g4gpu, torch, g4gpu.MIXED, beam_pinned, cur, field_pinned, lat,
                                                 steps, reps, e2e_out, shapes=shapes)
            t = statistics.median(times)
            e2e_res[key] = {"value": NS * steps / t, "unit": "slice-steps/s",
                            "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
                            "steps_per_window": steps,
                            "window": what + f"; median of {len(times)} windows after one warm-up window",
                            "window_s": t, "windows_s": times,
                            "spread": (max(times) - min(times)) / t,
                            "phases_of_one_window": phases}
        del e2e_out, field_pinned
        e2e_res["mixed_step_times_over_lattice"] = lattice_step_times(g4gpu, torch, beam, cur, lat, shapes)
    # plain FP64 form, same initial state and steps
    psteps = args.plain_steps if args.plain_steps is not None else args.steps
    do_plain = "plain" in args.forms
    if do_plain:
        hp, ms_p, st_p = time_form(g4gpu, torch, g4gpu.PLAIN, beam, cur, lat, psteps, args.warmup)
        ms_p = max_over_ranks(ws, ms_p)
    # error of the mixed form against the plain one after the same steps, and after
    # the whole lattice (both handles run on to its end)
    err = err_full = err_res = None
    if do_plain and psteps == args.steps:
        err = mixed_error(hm, hp, args.warmup + args.steps)
        if not args.no_full_lattice:
            done = args.warmup + args.steps
            nlat = lat.shape[0]
            if done < nlat:
                hm.run(done, nlat - done)
                hp.run(done, nlat - done)
            err_full = mixed_error(hm, hp, max(nlat, done))
    hm.close()
    if do_plain:
        hp.close()
    if do_plain and not args.no_full_lattice:
        err_res = resonant_companion(g4gpu, torch, shapes)

    value = job_value(ws, NS, args.steps, ms_m)
    plain_value = job_value(ws, NS, psteps, ms_p) if do_plain else None
    launches = sum(v[0] for v in st_m.values())

    def kernel_table(st, mixed):
        # the mixed form's deposition + ADI runs as one fused kernel when the slice
        # fits in shared memory, or in the shared memory of a cluster of up to four CTAs
        # (ngrid <= 333); it is accounted under the adi_x class
        fused = mixed and NGRID <= 333
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
    fp64_g, fp64_src = fp64_peak(g4gpu, torch.cuda.current_device())
    dom = max(kernels, key=lambda k: kernels[k]["ms_total"])
    dk = kernels[dom]

    line = {"metric": METRIC, "value": value, "unit": "slice-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_m / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "form": "mixed (FP32 field/solver/deposition, phase as a 64-bit fixed-point turn count)",
                       "cache": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{ws}",
                       "launch_shapes": ({"push_block": shapes[0], "field_threads": shapes[1],
                                          "field_kernel": ["one CTA per slice", "cluster pair",
                                                           "whole step per CTA"][shapes[2]],
                                          "source": "--launch-shapes" if fixed else "g4gpu_autotune"}
                                         if shapes else "defaults")},
            "forms": {"mixed": {"value": value, "ms_per_step": ms_m / args.steps},
                      "plain_fp64": ({"value": plain_value, "ms_per_step": ms_p / psteps,
                                      "steps": psteps, "kernels": kernels_plain,
                                      "fp64": fp64_roofline(kernels_plain, fp64_g, fp64_src)} if do_plain
                                     else None)},
            "value_plain_fp64": plain_value,
            "mixed_error_vs_plain": err,
            "mixed_error_vs_plain_full_lattice": err_full,
            "mixed_error_vs_plain_resonant": err_res,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": dk.get("achieved_gbs"), "peak": peak,
                         "unit": "GB/s", "frac": dk.get("frac_hbm"),
                         "traffic": (TRAFFIC_PER_SLICE[dom] * NS if dom in TRAFFIC_PER_SLICE else None),
                         "traffic_source": TRAFFIC_SOURCE,
                         "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                         "alg_bytes_per_launch": dk.get("alg_bytes"), "ms_per_launch": dk["ms_avg"]},
            "kernels": kernels, "gpu_launches": launches, "clocks": clocks}
    line.update(e2e_res)

    if "batched" in args.forms:
        line["forms"]["batched"] = batched_form(g4gpu, torch, args.steps, args.warmup, peak)
    if "harmonic" in args.forms:
        line["forms"]["harmonic_fft"] = harmonic_fft_form(g4gpu, torch, args.steps, args.warmup, peak,
                                                          ns=args.harmonic_slices)
    if "spacecharge" in args.forms:
        line["forms"]["spacecharge"] = spacecharge_form(g4gpu, torch, beam, cur, lat, args.steps, args.warmup,
                                                        peak, ms_m / args.steps, shapes)
        if rank == 0 and not args.no_cpu_baseline:
            line["forms"]["spacecharge"]["cpu_baseline"] = cpu_baseline_sc(SC_EFIELDS[0])
    if "learned" in args.forms:
        line["forms"]["learned"] = learned_form(g4gpu, torch, lat, beam, cur, args.steps, args.warmup)
        # the same closure in steady state (config 0: quiet loading, 1 kW seed, no
        # slippage), 4096 independent slices, with whole 4-period steps: valid there. In
        # the time-dependent window above a whole coarse step would slip the field 4
        # slices at once and add each slice's source coherently over 4 periods (about 4x
        # the fine run's power, in the oracle as on the GPU); its coarse steps therefore
        # push once and deposit and slip period by period.
        beam_q = g4gpu.host_load_beam(sp, 0, NPART, 4, 7, 0, LAMBDA0, 1.0)
        line["forms"]["learned_steady_state"] = learned_form(g4gpu, torch, lat, beam_q, cur, args.steps,
                                                             args.warmup, seed_power=1e3, time_run=0,
                                                             shotnoise=0, substeps=False)
        del beam_q
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
