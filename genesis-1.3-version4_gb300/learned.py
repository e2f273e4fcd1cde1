"""Learned coarse-step closure: lattice coarsening, training data, training and the
coarse-step run with the fine-step judge.

The steps:
  1. coarsen_lattice(): merges runs of up to `factor` identical undulator steps
     (one period each) into one coarse step; other steps stay as they are. Returns
     the coarse table and, per coarse step, the fine steps it covers. With
     `substeps`, the coarse handle runs a coarse step as a coarse push under the
     fine source and slippage (g4gpu_set_field_substeps): the push over the whole
     step, then period by period the deposition from interpolated phases and the
     slippage, then the diffraction of the whole step. A time-dependent window
     sampled every wavelength needs it: a whole coarse step would slip the field
     `factor` slices at once and add each slice's source coherently over the
     `factor` periods.
  2. generate_training_data(): for every seed, a window is integrated with fine
     steps; at every coarse step the state is copied to a second handle that takes
     the coarse step. The per-slice features of the starting state and the
     corrections that turn the coarse result into the fine one are recorded
     (all on the GPU: g4gpu_closure_features / g4gpu_closure_targets).
  3. MLP.train(): Adam on the GPU with the BF16 tensor-core kernels.
  4. Handle.run_learned(): coarse steps with the closure; every `check_every`
     coarse steps the fine solve of the same interval judges the slice power and
     replaces the coarse result when the error exceeds `tol`.

The teacher and judge is the non-learned fine-step method of the same arithmetic
form as the coarse handle (state copies between handles are device copies and
need equal storage).
"""
import numpy as np

import g4gpu


def coarsen_lattice(fine, factor=4, cols=g4gpu.LAT_COLS):
    """Returns (coarse_table, fine_start, fine_count)."""
    c = {k: i for i, k in enumerate(cols)}
    same = ["aw", "ax", "ay", "ku", "kx", "ky", "gradx", "grady", "qf", "qx", "qy", "helical"]
    rows, start, count = [], [], []
    i, n = 0, fine.shape[0]
    while i < n:
        r = fine[i]
        j = i + 1
        mergeable = r[c["aw"]] > 0 and r[c["cx"]] == 0 and r[c["cy"]] == 0 and r[c["phase"]] == 0
        if mergeable:
            while (j < n and j - i < factor and all(fine[j][c[k]] == r[c[k]] for k in same)
                   and fine[j][c["cx"]] == 0 and fine[j][c["cy"]] == 0 and fine[j][c["phase"]] == 0):
                j += 1
        row = r.copy()
        row[c["dz"]] = fine[i:j, c["dz"]].sum()
        row[c["slip"]] = fine[i:j, c["slip"]].sum()
        rows.append(row)
        start.append(i)
        count.append(j - i)
        i = j
    return np.array(rows), np.array(start, dtype=np.int32), np.array(count, dtype=np.int32)


def make_pair(cfg_kwargs, fine_lat, coarse_lat, beam, current, field, mlp_for_targets, waist, u0, c0,
              counts=None):
    """A fine and a coarse handle on the same window (the coarse one with a closure
    attached, which the target kernel needs for its buffers). counts: the periods of
    every coarse step, for coarse pushes under the fine source and slippage."""
    hf = g4gpu.Handle(g4gpu.Config(**cfg_kwargs))
    hc = g4gpu.Handle(g4gpu.Config(**cfg_kwargs))
    hf.set_lattice(fine_lat)
    hc.set_lattice(coarse_lat)
    if counts is not None:
        hc.set_field_substeps(counts)
    for h in (hf, hc):
        h.load_beam(beam, current)
        h.load_field(0, field)
        h.closure_attach(mlp_for_targets, waist, u0, c0)
    return hf, hc


def generate_training_data(cfg_kwargs, fine_lat, seeds, slice_params, npart, nbins, field, waist, u0, c0,
                           factor=4, max_coarse=None, shotnoise=1, substeps=False):
    """Features X [n][32] and targets T [n][4] from fine runs over `seeds` (the loading
    seed of each run; shotnoise 0 loads quiet beams); substeps: coarse pushes under the
    fine source and slippage."""
    coarse_lat, fstart, fcount = coarsen_lattice(fine_lat, factor)
    ncoarse = coarse_lat.shape[0] if max_coarse is None else min(max_coarse, coarse_lat.shape[0])
    scratch = g4gpu.MLP()
    X, T = [], []
    lam, sample = cfg_kwargs["lambda0"], cfg_kwargs["sample"]
    for seed in seeds:
        beam = g4gpu.host_load_beam(slice_params, 0, npart, nbins, seed, shotnoise, lam, sample)
        hf, hc = make_pair(cfg_kwargs, fine_lat, coarse_lat, beam, slice_params[:, 16], field, scratch, waist,
                           u0, c0, fcount if substeps else None)
        with hf, hc:
            for i in range(ncoarse):
                X.append(hf.closure_features())
                hc.copy_state_from(hf)
                hc.run(i, 1)
                hf.run(int(fstart[i]), int(fcount[i]))
                T.append(hc.closure_targets(hf))
    scratch.close()
    return np.concatenate(X), np.concatenate(T), coarse_lat, fstart, fcount


def evaluate(cfg_kwargs, fine_lat, coarse_lat, fstart, fcount, beam, current, field, mlp, waist, u0, c0,
             ncoarse=None, substeps=False):
    """Slice power and bunching after the same distance by (fine, coarse, coarse +
    closure). Returns dict of arrays."""
    ncoarse = coarse_lat.shape[0] if ncoarse is None else ncoarse
    nfine = int(fstart[ncoarse - 1] + fcount[ncoarse - 1])
    counts = fcount if substeps else None
    out = {}
    hf, hc = make_pair(cfg_kwargs, fine_lat, coarse_lat, beam, current, field, mlp, waist, u0, c0, counts)
    with hf, hc:
        hf.run(0, nfine)
        bd, fd = hf.diag(1)
        out["fine"] = (fd[0][:, 0].copy(), bd[:, 24].copy())
        hc.run(0, ncoarse)
        bd, fd = hc.diag(1)
        out["coarse"] = (fd[0][:, 0].copy(), bd[:, 24].copy())
    # coarse + closure through the driver, with no check inside the run
    hf, hc = make_pair(cfg_kwargs, fine_lat, coarse_lat, beam, current, field, mlp, waist, u0, c0, counts)
    with hf, hc:
        hc.run_learned(hf, 0, ncoarse, fstart, fcount, check_every=10 ** 9, tol=1e9)
        bd, fd = hc.diag(1)
        out["closure"] = (fd[0][:, 0].copy(), bd[:, 24].copy())
    return out


def errors(res):
    """Relative slice-power and absolute bunching errors of coarse and closure runs
    against the fine run."""
    pf, bf = res["fine"]
    scale = max(np.max(np.abs(pf)), 1e-300)
    e = {}
    for k in ("coarse", "closure"):
        p, b = res[k]
        e[k] = {"power": float(np.max(np.abs(p - pf)) / scale), "power_rms": float(np.sqrt(np.mean((p - pf) ** 2)) / scale),
                "bunching": float(np.max(np.abs(b - bf)))}
    return e
