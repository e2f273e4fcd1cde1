"""Test cases shared by the CPU and GPU tests: lattice tables, synthetic beams and
fields with the shapes of the GENESIS 1.3 v4 workloads exercised here.

The lattice tables follow the reference's unrolling (Lattice.cpp:340-516) and
slippage bookkeeping (Lattice.cpp:153-197) for the simple lattices used in the
tests: undulator modules split into steps of one period, optional quadrupoles
between modules. Column order is oracle/g4oracle.h G4_LAT_*.
"""
import math

import numpy as np

LAT_COLS = ["aw", "ax", "ay", "ku", "kx", "ky", "gradx", "grady", "qf", "qx", "qy",
            "cx", "cy", "dz", "slip", "phase", "helical", "z"]
C = {k: i for i, k in enumerate(LAT_COLS)}


def undulator_lattice(aw, lambdau, nwig, nmod, lambda0, gamma0, delz=None, helical=False,
                      kx=None, ky=None, quad_k1=0.0, quad_l=0.0, taper=0.0):
    """Per-step table for nmod undulator modules of nwig periods with an optional
    FODO quadrupole of length quad_l between modules (alternating sign of quad_k1).
    taper: linear relative change of aw from the first to the last module step."""
    delz = lambdau if delz is None else delz
    if kx is None:
        kx, ky = (0.5, 0.5) if helical else (0.0, 1.0)
    ku = 4.0 * math.asin(1) / lambdau
    rows = []
    nstep_und = int(round(lambdau * nwig / delz))
    dz_und = lambdau * nwig / nstep_und
    total_und = nmod * nstep_und
    k = 0
    for m in range(nmod):
        for i in range(nstep_und):
            r = [0.0] * len(LAT_COLS)
            awi = aw * (1.0 + taper * (k / max(total_und - 1, 1)))
            k += 1
            r[C["aw"]] = awi
            r[C["ku"]] = ku
            r[C["kx"]] = ku * ku * kx
            r[C["ky"]] = ku * ku * ky
            r[C["dz"]] = dz_und
            r[C["helical"]] = 1.0 if helical else 0.0
            rows.append(r)
        if m < nmod - 1 and quad_l > 0:
            r = [0.0] * len(LAT_COLS)
            r[C["qf"]] = quad_k1 if m % 2 == 0 else -quad_k1
            r[C["dz"]] = quad_l
            rows.append(r)
    t = np.array(rows)
    # z positions and slippage (Lattice.cpp:153-197)
    z = 0.0
    for i in range(len(t)):
        t[i, C["z"]] = z
        z += t[i, C["dz"]]
    lz = 0.0
    for i in range(len(t)):
        a = t[i, C["aw"]]
        if a > 0:
            tmp = 2 * gamma0 * gamma0 * lambda0 / (1 + a * a)
            t[i, C["slip"]] = t[i, C["dz"]] / tmp
            if lz > 0 and i > 0:
                t[i - 1, C["slip"]] += math.floor(lz / 2 / gamma0 / gamma0 / lambda0) + 1
                lz = 0.0
        else:
            lz += t[i, C["dz"]]
            t[i, C["slip"]] = 0.0
    t[-1, C["slip"]] += math.floor(lz / 2 / gamma0 / gamma0 / lambda0) + 1
    return t


def slice_params(ns, gamma, delgam, emit_n, beta, alpha=0.0, current=3000.0, currents=None):
    """[ns][17] slice parameter rows for the quiet loader (oracle/g4oracle.h)."""
    sp = np.zeros((ns, 17))
    sp[:, 0] = gamma
    sp[:, 1] = delgam
    sp[:, 2] = emit_n
    sp[:, 3] = emit_n
    sp[:, 4] = beta
    sp[:, 5] = beta
    sp[:, 6] = alpha
    sp[:, 7] = alpha
    sp[:, 16] = current if currents is None else currents
    return sp


def flat_top_current(ns, lambda0, sample, peak, edge_sigma):
    """Flat-top current with Gaussian edges of rms length edge_sigma [m]."""
    s = np.arange(ns) * lambda0 * sample
    s0, s1 = s[0] + 3 * edge_sigma, s[-1] - 3 * edge_sigma
    cur = np.full(ns, peak)
    lo = s < s0
    hi = s > s1
    cur[lo] = peak * np.exp(-0.5 * ((s[lo] - s0) / edge_sigma) ** 2)
    cur[hi] = peak * np.exp(-0.5 * ((s[hi] - s1) / edge_sigma) ** 2)
    return cur


def gauss_field_par(lambda0, power, w0, harm=1, phase=0.0, z0=0.0):
    """Gauss-Hermite parameter vector (oracle/g4oracle.h orc_gauss_hermite)."""
    return np.array([lambda0, power, phase, z0, w0, 0, 0, 0, 0, 0, 0, harm], dtype=np.float64)


# Config 0/1 physics (planar undulator, FODO between modules)
CFG0 = dict(aw=1.7, lambdau=0.015, nwig=110, nmod=4, lambda0=1e-10, gamma0=11357.8,
            quad_k1=1.5, quad_l=0.08, current=3000.0, delgam=2.0, emit_n=0.4e-6, beta=15.0,
            npart=8192, nbins=4, ngrid=151, gridmax=1e-4, power=1e3, w0=30e-6)
# Example1 of the reference (helical, lasing)
EX1 = dict(aw=0.84853, lambdau=0.015, lambda0=1e-10, gamma0=11357.82, current=3000.0,
           delgam=1.0, emit_n=4e-7, npart=8192, nbins=8, ngrid=255, gridmax=2e-4, power=5e3,
           w0=30e-6)
