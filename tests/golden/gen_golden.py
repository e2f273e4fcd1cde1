"""Generates the golden fixtures of tests/golden/ from the GENESIS 1.3 v4 reference
itself, compiled from its own sources (oracle/ref_build/Makefile -> oracle/_ref/).

Run where the reference tree is present, naming it in G4_REFERENCE_DIR:
    G4_REFERENCE_DIR=<tree> python oracle/build_oracle.py <tree>
    G4_REFERENCE_DIR=<tree> python tests/golden/gen_golden.py

Fixtures (numpy .npz):
  streams.npz    ran2, Hammersley, inverse erfc, Bessel J_n and fc(h) values
  loading.npz    quiet-loaded / shot-noise slices and Gauss-Hermite seed fields
  steps.npz      integration steps of small windows: input state, lattice table and
                 the reference's output state for single stages and full steps
  example1.npz   the reference's Example1 deck (examples/Example1-SteadyState):
                 lattice table, loaded beam, per-step power / bunching / energy
  config0.npz    the 443-step steady-state deck of the planar FODO configuration:
                 lattice table, loaded beam, per-step power / bunching / energy
  spacecharge.npz integration steps with space charge (&efield): short-range modes,
                 the long-range loss, both; input state, parameters and output state

  wakes.npz      the reference's single-particle wakes (resistive round and flat pipe,
                 geometric, roughness) for several &wake settings, and integration steps
                 with wakes (Collective::update / apply) on windows of sample 1 and 3

  chicane.npz    integration steps through a chicane between two undulator modules
                 (TrackBeam::applyChicane and applyR56), time-dependent and steady state
  one4one.npz    one4one windows (slices of different particle counts) sorted after the
                 push (Beam::sort), every step and every third step with space charge
  incoherent.npz incoherent synchrotron radiation (&sponrad): the energy loss over planar
                 and helical lattices, and loss with spread over one step of a larger
                 window (with the same window's step without it)
  fft.npz        the FFT field solver (FieldSolverFFT) over whole lattices, unfiltered
                 and filtered, odd and even grids, harmonics 1, 3, 5 on ngrid 255; the
                 far-field pointing and divergence of DiagField (filter "fft"). The
                 reference is built with -DFFTW on oracle/ref_build's FFTW stand-in
                 (FFTW's documented DFT evaluated directly), as FFTW is not installed

`python tests/golden/gen_golden.py spacecharge` (or `wakes`, `chicane`, `one4one`,
`incoherent`, `fft`) regenerates only that file.

The reference's CI check of Example1 (examples/Example1-SteadyState/TEST_power.py)
expects a final power of 0.932785e9 W within 30 %; example1.npz records what the
compiled reference produces here.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import g4cases as T  # noqa: E402
import g4oracle as G  # noqa: E402
from rawio import read_raw  # noqa: E402

# the reference source tree (its example decks are read from there)
REF_DIR = os.environ.get("G4_REFERENCE_DIR")
GENESIS = os.path.join(ROOT, "oracle", "_ref", "genesis4")


def gen_streams(r):
    d = {}
    for s in (1, 7, 11, 123456789):
        d[f"ran2_{s}"] = r.ran2(s, 64)
    for b in range(6):
        for st in (0, 12345, 987654321):
            d[f"ham_{b}_{st}"] = r.hammersley(b, st, 64)
    x = np.linspace(1e-12, 2 - 1e-12, 1001)
    d["inverfc_x"] = x
    d["inverfc_y"] = r.inverfc(x)
    xs = np.array([-9.0, -3.0, 0.0, 0.1, 0.3, 1.0, 2.5, 7.9, 8.1, 15.0])
    d["bessel_x"] = xs
    d["bessel_j"] = np.array([[r.besselj(n, v) for v in xs] for n in range(5)])
    aws = np.array([0.5, 0.84853, 1.7, 3.0])
    d["fc_aw"] = aws
    d["fc"] = np.array([[[r.fc(a, hel, h) for h in range(1, 8)] for hel in (0, 1)] for a in aws])
    np.savez_compressed(os.path.join(HERE, "streams.npz"), **d)


def loading_cases():
    sp0 = T.slice_params(4, 11357.8, 2.0, 0.4e-6, 15.0)
    sp1 = T.slice_params(4, 11357.8, 1.0, 0.4e-6, 15.0, alpha=0.3)
    sp2 = T.slice_params(3, 11357.8, 2.0, 0.4e-6, 12.0)
    sp2[:, 8] = 1e-6
    sp2[:, 11] = 0.1
    sp2[:, 12] = [0.05, 0.2, 0.0]    # bunch (both branches of QuietLoading.cpp:248-258)
    sp2[:, 13] = 0.4
    sp2[:, 14] = [0.5, 0.0, 1.0]     # emod
    sp2[:, 15] = 0.1
    cur = T.flat_top_current(4, 1e-10, 1.0, 3000.0, 0.8e-10)
    sp3 = T.slice_params(4, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur)
    return [
        dict(name="quiet_nb4", sp=sp0, islice0=0, npart=64, nbins=4, seed=1, sn=0),
        dict(name="shot_nb4", sp=sp0, islice0=0, npart=64, nbins=4, seed=7, sn=1),
        dict(name="shot_nb8", sp=sp1, islice0=10, npart=128, nbins=8, seed=11, sn=1),
        dict(name="bunch_emod", sp=sp2, islice0=3, npart=32, nbins=4, seed=5, sn=0),
        dict(name="shot_profile", sp=sp3, islice0=100, npart=64, nbins=4, seed=7, sn=1),
    ]


def gh_cases():
    return [
        dict(name="gh_fund", par=T.gauss_field_par(1e-10, 1e3, 30e-6), gridmax=1e-4, ngrid=21),
        dict(name="gh_h3", par=np.array([1e-10, 2e2, 0.3, 0.5, 20e-6, 1e-6, -2e-6, 1e-5, 0, 1, 2, 3.0]),
             gridmax=1.5e-4, ngrid=17),
    ]


def gen_loading(r):
    d = {}
    for c in loading_cases():
        d[c["name"] + "_sp"] = c["sp"]
        d[c["name"] + "_args"] = np.array([c["islice0"], c["npart"], c["nbins"], c["seed"], c["sn"]])
        d[c["name"]] = r.load_beam(c["sp"], c["islice0"], c["npart"], c["nbins"], c["seed"], c["sn"], 1e-10, 1.0)
    for c in gh_cases():
        d[c["name"] + "_par"] = c["par"]
        d[c["name"] + "_grid"] = np.array([c["gridmax"], c["ngrid"]])
        d[c["name"]] = r.gauss_hermite(c["par"], c["gridmax"], c["ngrid"])
    np.savez_compressed(os.path.join(HERE, "loading.npz"), **d)


def step_cases(r):
    """Small windows that exercise every branch of the step."""
    cases = []
    # planar FODO, time dependent, shot noise
    lat = T.undulator_lattice(1.7, 0.015, 8, 2, 1e-10, 11357.8, quad_k1=1.5, quad_l=0.08)
    cur = np.array([3000.0, 2500.0, 1000.0, 3000.0])
    part = r.load_beam(T.slice_params(4, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur), 0, 64, 4, 7, 1, 1e-10, 1.0)
    gh = r.gauss_hermite(T.gauss_field_par(1e-10, 1e5, 20e-6), 6e-5, 25)
    fld = np.stack([gh * (1 + 0.2j * k) for k in range(4)])[None]
    cases.append(dict(name="planar", lat=lat, gammaref=11357.8, part=part, cur=cur, harm=[1],
                      gridmax=[6e-5], fields=fld, first=[0], time_run=1, periodic=0))
    # helical undulator with corrector kicks, a phase shift and an offset/gradient
    lat = T.undulator_lattice(0.84853, 0.015, 6, 2, 1e-10, 11357.82, helical=True, quad_k1=2.0, quad_l=0.08)
    lat[3, T.C["cx"]] = 2e-6
    lat[5, T.C["cy"]] = -1e-6
    lat[2, T.C["phase"]] = 0.7
    lat[:6, T.C["ax"]] = 2e-6
    lat[:6, T.C["gradx"]] = 3.0
    lat[6, T.C["qx"]] = 1e-5
    part = r.load_beam(T.slice_params(3, 11357.82, 1.0, 0.4e-6, 10.0), 2, 64, 8, 3, 1, 1e-10, 1.0)
    gh = r.gauss_hermite(T.gauss_field_par(1e-10, 5e3, 30e-6), 8e-5, 21)
    fld = np.stack([gh * (1 - 0.1j * k) for k in range(3)])[None]
    cases.append(dict(name="helical", lat=lat, gammaref=11357.82, part=part, cur=np.full(3, 3000.0),
                      harm=[1], gridmax=[8e-5], fields=fld, first=[1], time_run=1, periodic=0))
    # two harmonics (1 and 3) with their own grids; periodic window
    lat = T.undulator_lattice(1.7, 0.015, 6, 2, 1e-10, 11357.8, quad_k1=1.5, quad_l=0.08)
    part = r.load_beam(T.slice_params(5, 11357.8, 2.0, 0.4e-6, 15.0), 0, 48, 4, 9, 1, 1e-10, 1.0)
    g1 = r.gauss_hermite(T.gauss_field_par(1e-10, 1e5, 20e-6), 6e-5, 19)
    g3 = r.gauss_hermite(T.gauss_field_par(1e-10, 1e3, 12e-6, harm=3), 4e-5, 19)
    fld = np.stack([np.stack([g1 * (1 + 0.3j * k) for k in range(5)]),
                    np.stack([g3 * (1 - 0.2j * k) for k in range(5)])])
    cases.append(dict(name="harm13", lat=lat, gammaref=11357.8, part=part, cur=np.full(5, 2000.0),
                      harm=[1, 3], gridmax=[6e-5, 4e-5], fields=fld, first=[0, 2], time_run=1,
                      periodic=1))
    # steady state single slice, particles partly off the grid
    lat = T.undulator_lattice(1.7, 0.015, 10, 1, 1e-10, 11357.8)
    part = r.load_beam(T.slice_params(1, 11357.8, 2.0, 4e-6, 15.0), 0, 96, 4, 1, 0, 1e-10, 1.0)
    gh = r.gauss_hermite(T.gauss_field_par(1e-10, 1e6, 15e-6), 3e-5, 15)
    cases.append(dict(name="steady", lat=lat, gammaref=11357.8, part=part, cur=np.array([3000.0]),
                      harm=[1], gridmax=[3e-5], fields=gh[None, None], first=[0], time_run=0,
                      periodic=0))
    return cases


def gen_steps(r):
    d = {}
    for c in step_cases(r):
        n = c["name"]
        for k in ("lat", "part", "cur", "harm", "gridmax", "fields", "first"):
            d[f"{n}_{k}"] = np.asarray(c[k])
        d[f"{n}_args"] = np.array([c["gammaref"], c["time_run"], c["periodic"]])
        for stages in (1, 2, 4, 7):
            # single stages over the first step, the full step over the whole lattice
            lat = c["lat"][:1] if stages != 7 else c["lat"]
            out = r.run_steps(lat, c["gammaref"], c["part"], c["cur"], 1e-10, 1.0, c["harm"],
                              c["gridmax"], c["fields"], c["first"], time_run=c["time_run"],
                              periodic=c["periodic"], stages=stages)
            d[f"{n}_s{stages}_part"] = out[0]
            d[f"{n}_s{stages}_fields"] = out[1]
            d[f"{n}_s{stages}_first"] = out[2]
    np.savez_compressed(os.path.join(HERE, "steps.npz"), **d)


def sc_cases(r):
    """Windows with space charge: the short-range field (radial grid grown from rmax 0),
    the long-range loss, and both in steady state with a fixed radial grid."""
    cases = []
    lat = T.undulator_lattice(1.7, 0.015, 6, 2, 1e-10, 11357.8, quad_k1=1.5, quad_l=0.08)
    cur = np.array([3000.0, 2500.0, 1000.0, 3000.0])
    part = r.load_beam(T.slice_params(4, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur), 0, 64, 4, 7, 1, 1e-10, 1.0)
    gh = r.gauss_hermite(T.gauss_field_par(1e-10, 1e5, 20e-6), 6e-5, 25)
    fld = np.stack([gh * (1 + 0.2j * k) for k in range(4)])[None]
    base = dict(lat=lat, gammaref=11357.8, part=part, cur=cur, harm=[1], gridmax=[6e-5], fields=fld, first=[0],
                time_run=1, periodic=0)
    cases.append(dict(base, name="short", efield=[0.0, 24, 2, 1, 0]))
    cases.append(dict(base, name="long", efield=[0.0, 0, 0, 0, 1]))
    cases.append(dict(base, name="both", efield=[0.0, 16, 1, 2, 1]))
    lat1 = T.undulator_lattice(1.7, 0.015, 10, 1, 1e-10, 11357.8)
    part1 = r.load_beam(T.slice_params(1, 11357.8, 2.0, 0.4e-6, 15.0), 0, 96, 4, 1, 0, 1e-10, 1.0)
    gh1 = r.gauss_hermite(T.gauss_field_par(1e-10, 1e6, 15e-6), 6e-5, 21)
    cases.append(dict(name="steady", lat=lat1, gammaref=11357.8, part=part1, cur=np.array([3000.0]), harm=[1],
                      gridmax=[6e-5], fields=gh1[None, None], first=[0], time_run=0, periodic=0,
                      efield=[5e-5, 30, 3, 2, 1]))
    return cases


def gen_space_charge(r):
    d = {}
    for c in sc_cases(r):
        n = c["name"]
        for k in ("lat", "part", "cur", "harm", "gridmax", "fields", "first", "efield"):
            d[f"{n}_{k}"] = np.asarray(c[k])
        d[f"{n}_args"] = np.array([c["gammaref"], c["time_run"], c["periodic"]])
        rmax, ngrid, nz, nphi, longrange = c["efield"]
        r.set_efield(rmax, int(ngrid), int(nz), int(nphi), bool(longrange))
        out = r.run_steps(c["lat"], c["gammaref"], c["part"], c["cur"], 1e-10, 1.0, c["harm"], c["gridmax"],
                          c["fields"], c["first"], time_run=c["time_run"], periodic=c["periodic"], stages=7)
        r.set_efield()
        d[f"{n}_out_part"] = out[0]
        d[f"{n}_out_fields"] = out[1]
        d[f"{n}_out_first"] = out[2]
    np.savez_compressed(os.path.join(HERE, "spacecharge.npz"), **d)


WAKE_SETS = {
    "cu_round": dict(radius=2.5e-3, conductivity=5.813e7, relaxation=8.1e-6, roundpipe=True),
    "al_flat": dict(radius=3.0e-3, conductivity=3.571e7, relaxation=2.4e-6, roundpipe=False),
    "geo_round": dict(radius=2.5e-3, gap=1e-3, lgap=0.5, roundpipe=True),
    "geo_flat": dict(radius=2.5e-3, gap=2e-3, lgap=1.5, roundpipe=False),
    "rough": dict(radius=2.5e-3, hrough=1e-7, lrough=1e-4),
    "all": dict(radius=2.0e-3, conductivity=5.813e7, relaxation=8.1e-6, roundpipe=True, gap=1e-3, lgap=0.5,
                hrough=1e-7, lrough=1e-4),
}
WAKE_NS, WAKE_DS = 200, 1e-10


def wake_cases(r):
    """Windows with wakes: the single-particle wakes of the "all" setting scaled so that
    each changes gamma by about 1e-3 over the lattice (like the FEL interaction of these
    windows; over a few slices the unscaled wakes are too weak to see), an external loss
    per slice; windows of sample 1 (4 slices, 4 fine points) and sample 3 (5 slices,
    15 fine points, current ramp), and a transient wake."""
    res, geo, rou = r.single_wakes(64, WAKE_DS, **WAKE_SETS["all"])
    res, geo, rou = res * 1e2, geo * 30.0, rou * 1e3
    lat = T.undulator_lattice(1.7, 0.015, 6, 2, 1e-10, 11357.8, quad_k1=1.5, quad_l=0.08)
    cases = []
    cur = np.array([3000.0, 2500.0, 1000.0, 3000.0])
    part = r.load_beam(T.slice_params(4, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur), 0, 64, 4, 7, 1, 1e-10, 1.0)
    gh = r.gauss_hermite(T.gauss_field_par(1e-10, 1e5, 20e-6), 6e-5, 25)
    fld = np.stack([gh * (1 + 0.2j * k) for k in range(4)])[None]
    base = dict(lat=lat, gammaref=11357.8, part=part, cur=cur, harm=[1], gridmax=[6e-5], fields=fld, first=[0],
                time_run=1, periodic=0, sample=1.0)
    ext = np.array([-2000.0, 500.0, 0.0, 1500.0])
    cases.append(dict(base, name="s1", wake=dict(ext=ext, res=res[:4], geo=geo[:4], rou=rou[:4], ds=WAKE_DS,
                                                 ztrans=0.0, radius=2.0e-3, transient=False)))
    cases.append(dict(base, name="s1_transient", wake=dict(ext=0 * ext, res=res[:4], geo=geo[:4], rou=rou[:4],
                                                           ds=WAKE_DS, ztrans=-1.0, radius=2.0e-3, transient=True)))
    cur5 = np.linspace(500.0, 3500.0, 5)
    part5 = r.load_beam(T.slice_params(5, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur5), 0, 48, 4, 3, 1, 1e-10, 3.0)
    fld5 = np.stack([gh * (1 - 0.1j * k) for k in range(5)])[None]
    cases.append(dict(base, name="s3", part=part5, cur=cur5, fields=fld5, sample=3.0,
                      wake=dict(ext=np.linspace(-1000.0, 1000.0, 5), res=res[:15], geo=geo[:15], rou=rou[:15],
                                ds=WAKE_DS, ztrans=0.0, radius=2.0e-3, transient=False)))
    return cases


def gen_wakes(r):
    d = {}
    for name, kw in WAKE_SETS.items():
        res, geo, rou = r.single_wakes(WAKE_NS, WAKE_DS, **kw)
        d[f"single_{name}_res"], d[f"single_{name}_geo"], d[f"single_{name}_rou"] = res, geo, rou
        d[f"single_{name}_par"] = np.array([kw.get("radius", 2.5e-3), kw.get("conductivity", 0.0),
                                            kw.get("relaxation", 0.0), float(kw.get("roundpipe", True)),
                                            kw.get("gap", 0.0), kw.get("lgap", 1.0), kw.get("hrough", 0.0),
                                            kw.get("lrough", 1.0)])
    d["single_ns_ds"] = np.array([WAKE_NS, WAKE_DS])
    for c in wake_cases(r):
        n = c["name"]
        for k in ("lat", "part", "cur", "harm", "gridmax", "fields", "first"):
            d[f"{n}_{k}"] = np.asarray(c[k])
        w = c["wake"]
        for k in ("ext", "res", "geo", "rou"):
            d[f"{n}_wake_{k}"] = np.asarray(w[k])
        d[f"{n}_wake_par"] = np.array([w["ds"], w["ztrans"], w["radius"], float(w["transient"])])
        d[f"{n}_args"] = np.array([c["gammaref"], c["time_run"], c["periodic"], c["sample"]])
        r.set_wake(**w)
        out = r.run_steps(c["lat"], c["gammaref"], c["part"], c["cur"], 1e-10, c["sample"], c["harm"],
                          c["gridmax"], c["fields"], c["first"], time_run=c["time_run"], periodic=c["periodic"],
                          stages=7)
        r.set_wake()
        d[f"{n}_out_part"] = out[0]
        d[f"{n}_out_fields"] = out[1]
        d[f"{n}_out_first"] = out[2]
    np.savez_compressed(os.path.join(HERE, "wakes.npz"), **d)


CHICANE = [0.01, 0.1, 0.3, 1.0]  # angle, lb, ld, lt


def chicane_lattice(nwig):
    """Two undulator modules of nwig periods with a chicane step between them (aw 0, the
    chicane's length, a small slippage of its own; the table takes any values)."""
    und = T.undulator_lattice(1.7, 0.015, nwig, 2, 1e-10, 11357.8)
    row = np.zeros(len(T.LAT_COLS))
    row[T.C["dz"]] = CHICANE[3]
    row[T.C["slip"]] = 2.0
    lat = np.vstack([und[:nwig], row, und[nwig:]])
    z = 0.0
    for i in range(lat.shape[0]):
        lat[i, T.C["z"]] = z
        z += lat[i, T.C["dz"]]
    chic = np.zeros((lat.shape[0], 4))
    chic[nwig] = CHICANE
    return lat, chic


def chicane_cases(r):
    lat, chic = chicane_lattice(6)
    cur = np.array([3000.0, 2500.0, 1000.0, 3000.0])
    part = r.load_beam(T.slice_params(4, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur), 0, 64, 4, 7, 1, 1e-10, 1.0)
    gh = r.gauss_hermite(T.gauss_field_par(1e-10, 1e5, 20e-6), 6e-5, 25)
    fld = np.stack([gh * (1 + 0.2j * k) for k in range(4)])[None]
    cases = [dict(name="td", lat=lat, chic=chic, gammaref=11357.8, part=part, cur=cur, harm=[1], gridmax=[6e-5],
                  fields=fld, first=[0], time_run=1, periodic=0)]
    lat1, chic1 = chicane_lattice(5)
    part1 = r.load_beam(T.slice_params(1, 11357.8, 2.0, 0.4e-6, 15.0), 0, 96, 4, 1, 0, 1e-10, 1.0)
    gh1 = r.gauss_hermite(T.gauss_field_par(1e-10, 1e6, 15e-6), 6e-5, 21)
    cases.append(dict(name="steady", lat=lat1, chic=chic1, gammaref=11357.8, part=part1, cur=np.array([3000.0]),
                      harm=[1], gridmax=[6e-5], fields=gh1[None, None], first=[0], time_run=0, periodic=0))
    return cases


def gen_chicane(r):
    d = {}
    for c in chicane_cases(r):
        n = c["name"]
        for k in ("lat", "chic", "part", "cur", "harm", "gridmax", "fields", "first"):
            d[f"{n}_{k}"] = np.asarray(c[k])
        d[f"{n}_args"] = np.array([c["gammaref"], c["time_run"], c["periodic"]])
        r.set_chicanes(c["chic"])
        out = r.run_steps(c["lat"], c["gammaref"], c["part"], c["cur"], 1e-10, 1.0, c["harm"], c["gridmax"],
                          c["fields"], c["first"], time_run=c["time_run"], periodic=c["periodic"], stages=7)
        r.set_chicanes()
        d[f"{n}_out_part"] = out[0]
        d[f"{n}_out_fields"] = out[1]
        d[f"{n}_out_first"] = out[2]
    np.savez_compressed(os.path.join(HERE, "chicane.npz"), **d)


# resonant at lambda0 1e-10 with aw 1.7 and lambdau 0.015: the phases stay near their
# slices, and sorting moves only the particles that cross a slice boundary
O4O_GAMMA = 17081.0


def o4o_window(r, ns=6, cap=96, seed=3):
    """A one4one window: slices of 50..80 particles (capacity cap), uniform phases, with
    some phases pushed outside their slice (moved by the first sort) and a few outside
    the window (dropped by it)."""
    rng = np.random.default_rng(seed)
    cur = np.full(ns, 2500.0)
    part = r.load_beam(T.slice_params(ns, O4O_GAMMA, 2.0, 0.4e-6, 15.0, currents=cur), 0, cap, 1, 5, 0, 1e-10, 1.0)
    counts = rng.integers(50, 81, ns).astype(np.int32)
    for i in range(ns):
        k = rng.choice(counts[i], size=counts[i] // 8, replace=False)
        part[i, k, 1] += rng.uniform(-7.0, 7.0, k.size)
        part[i, counts[i]:, :] = 0.0
    part[0, 0, 1] = -0.5                      # s < 0: leaves the window
    part[ns - 1, 1, 1] = 2 * np.pi + 0.25     # beyond the window's end
    return part, counts, cur


def o4o_cases(r):
    lat = T.undulator_lattice(1.7, 0.015, 12, 1, 1e-10, O4O_GAMMA)
    part, counts, cur = o4o_window(r)
    gh = r.gauss_hermite(T.gauss_field_par(1e-10, 1e5, 20e-6), 6e-5, 25)
    fld = np.stack([gh * (1 + 0.2j * k) for k in range(part.shape[0])])[None]
    base = dict(lat=lat, gammaref=O4O_GAMMA, part=part, cur=cur, counts=counts, harm=[1], gridmax=[6e-5],
                fields=fld, first=[0], time_run=1, periodic=0)
    return [dict(base, name="every", every=1, efield=[0.0, 0, 0, 0, 0]),
            dict(base, name="third", every=3, efield=[0.0, 16, 1, 1, 1])]


def gen_one4one(r):
    d = {}
    for c in o4o_cases(r):
        n = c["name"]
        for k in ("lat", "part", "cur", "counts", "harm", "gridmax", "fields", "first", "efield"):
            d[f"{n}_{k}"] = np.asarray(c[k])
        d[f"{n}_args"] = np.array([c["gammaref"], c["time_run"], c["periodic"], c["every"]])
        r.set_counts(c["counts"], c["every"])
        rmax, ngr, nz, nphi, lr = c["efield"]
        r.set_efield(rmax, int(ngr), int(nz), int(nphi), bool(lr))
        out = r.run_steps(c["lat"], c["gammaref"], c["part"], c["cur"], 1e-10, 1.0, c["harm"], c["gridmax"],
                          c["fields"], c["first"], time_run=c["time_run"], periodic=c["periodic"], stages=7)
        d[f"{n}_out_counts"] = r.get_counts(len(c["counts"]))
        r.set_counts()
        r.set_efield()
        d[f"{n}_out_part"] = out[0]
        d[f"{n}_out_fields"] = out[1]
        d[f"{n}_out_first"] = out[2]
    np.savez_compressed(os.path.join(HERE, "one4one.npz"), **d)


def gen_incoherent(r):
    d = {}
    cur = np.array([3000.0, 2500.0, 1000.0, 3000.0])
    gh = r.gauss_hermite(T.gauss_field_par(1e-10, 1e5, 20e-6), 6e-5, 25)
    fld = np.stack([gh * (1 + 0.2j * k) for k in range(4)])[None]
    cases = []
    for name, helical, npart, nwig, loss, spread in (("loss", False, 64, 6, 1, 0), ("loss_helical", True, 64, 6, 1, 0),
                                                     ("spread", False, 1024, 1, 1, 1)):
        lat = T.undulator_lattice(1.7, 0.015, nwig, 1, 1e-10, 11357.8, helical=helical)
        part = r.load_beam(T.slice_params(4, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur), 0, npart, 4, 7, 1, 1e-10,
                           1.0)
        cases.append((name, lat, part, loss, spread))
    for name, lat, part, loss, spread in cases:
        d[f"{name}_lat"], d[f"{name}_part"] = lat, part
        d[f"{name}_isr"] = np.array([1234, loss, spread, 4])
        r.set_incoherent(1234, bool(loss), bool(spread), 4)
        out = r.run_steps(lat, 11357.8, part, cur, 1e-10, 1.0, [1], [6e-5], fld, [0], time_run=1, stages=7)
        r.set_incoherent(1234, False, False, 4)
        base = r.run_steps(lat, 11357.8, part, cur, 1e-10, 1.0, [1], [6e-5], fld, [0], time_run=1, stages=7)
        d[f"{name}_out_part"], d[f"{name}_out_fields"] = out[0], out[1]
        d[f"{name}_base_part"] = base[0]
    d["cur"], d["fields"] = cur, fld
    np.savez_compressed(os.path.join(HERE, "incoherent.npz"), **d)


# ngrid of the FFT-solver windows: odd and even, every register radix of the engine's
# transform plans (25 = 5 5, 32 = 16 2, 45 = 15 3, 22 = 2 11) and a generic prime stage
# (38 = 2 19)
FFT_GRIDS = (25, 32, 45, 22, 38)
FFT_FILTER = (0.7, 0.9, 0.3)


def fft_cases(r):
    """Windows for the reference's FieldSolverFFT (built on the FFTW stand-in): two
    harmonics (1, 3) on their own grids, the unfiltered and the filtered source (xcut
    0.7, ycut 0.9, sigmoid 0.3) on every grid of FFT_GRIDS; and config 3's layout at a
    reduced size: harmonics 1, 3, 5 on ngrid 255 over gridmax 1.5e-4 m, nbins 8 shot
    noise, delgam 1.0. The windows are periodic (the field slipping out of the head
    re-enters at the tail): at 2.26 slices of slippage per step a zero-filled window
    of a few slices would be emptied within two steps, and every solve would then
    transform a zero field."""
    cases = []
    lat = T.undulator_lattice(1.7, 0.015, 6, 2, 1e-10, 11357.8, quad_k1=1.5, quad_l=0.08)
    part = r.load_beam(T.slice_params(5, 11357.8, 2.0, 0.4e-6, 15.0), 0, 64, 4, 7, 1, 1e-10, 1.0)
    for n in FFT_GRIDS:
        g1 = r.gauss_hermite(T.gauss_field_par(1e-10, 1e5, 20e-6), 6e-5, n)
        g3 = r.gauss_hermite(T.gauss_field_par(1e-10, 1e3, 12e-6, harm=3), 4e-5, n)
        fld = np.stack([np.stack([g1 * (1 + 0.3j * k) for k in range(5)]),
                        np.stack([g3 * (1 - 0.2j * k) for k in range(5)])])
        for solver in (1, 2):
            cases.append(dict(name=f"n{n}_s{solver}", lat=lat, part=part, cur=np.full(5, 3000.0), harm=[1, 3],
                              gridmax=[6e-5, 4e-5], fields=fld, solver=solver,
                              filt=FFT_FILTER if solver == 2 else (1.0, 1.0, 1.0)))
    ns, ng, gm, harm = 3, 255, 1.5e-4, [1, 3, 5]
    lat = T.undulator_lattice(1.7, 0.015, 5, 2, 1e-10, 11357.8, quad_k1=1.5, quad_l=0.08)
    part = r.load_beam(T.slice_params(ns, 11357.8, 1.0, 0.4e-6, 15.0), 0, 256, 8, 7, 1, 1e-10, 1.0)
    fld = harm255_fields(r.gauss_hermite, ns, ng, gm, harm)
    cases.append(dict(name="harm255", lat=lat, part=part, cur=np.full(ns, 3000.0), harm=harm, gridmax=[gm] * 3,
                      fields=fld, solver=1, filt=(1.0, 1.0, 1.0)))
    return cases


def harm255_fields(gauss_hermite, ns=3, ng=255, gm=1.5e-4, harm=(1, 3, 5)):
    """Initial fields of the harm255 case from a Gauss-Hermite loader (the reference's,
    or one bit-exact with it): they are rebuilt rather than stored."""
    return np.stack([np.stack([gauss_hermite(T.gauss_field_par(1e-10, 1e5 / h ** 2, 25e-6, harm=h), gm, ng)
                               * np.exp(1j * (0.4 * k + h)) for k in range(ns)]) for h in harm])


# cells of the ngrid-255 output fields kept in fft.npz (every 29th: 2243 per slice)
HARM255_CELLS = slice(0, None, 29)


def far_field(ng, ns=6):
    """A Gaussian beam off axis with a transverse tilt that changes from slice to slice
    (rebuilt by the tests rather than stored)."""
    x = np.arange(ng) - 0.5 * (ng - 1)
    g = np.exp(-((x[None, :] - 2.0) ** 2 + (x[:, None] + 1.0) ** 2) / (0.05 * ng * ng))
    return np.stack([(g * np.exp(1j * (0.2 + 0.05 * s) * x[None, :] - 1j * 0.03 * s * x[:, None])).ravel() * 1e4
                     for s in range(ns)])


# (ngrid, harmonic, ring start) of the far-field cases: odd and even grids
FAR_FIELD_CASES = ((45, 1, 0), (32, 3, 2), (51, 1, 5), (21, 5, 1))


def gen_fft(r):
    """fft.npz: the reference's FFT field solver (FieldSolverFFT.cpp:9-167) over whole
    lattices, and its far-field diagnostics (Diagnostic.cpp:718-996 with filter "fft"),
    both built against the FFTW stand-in of oracle/ref_build."""
    d = {}
    for c in fft_cases(r):
        n = c["name"]
        big = n == "harm255"
        for k in ("lat", "part", "cur", "harm", "gridmax", "filt"):
            d[f"{n}_{k}"] = np.asarray(c[k])
        if not big:  # one input field per grid, shared by the unfiltered and filtered case
            d[f"{n.split('_')[0]}_fields"] = np.asarray(c["fields"])
        d[f"{n}_solver"] = np.array(c["solver"])
        nf = len(c["harm"])
        out = r.run_steps(c["lat"], 11357.8, c["part"], c["cur"], 1e-10, 1.0, c["harm"], c["gridmax"],
                          c["fields"], [0] * nf, time_run=1, periodic=1, stages=7, solver=c["solver"],
                          filt=c["filt"])
        d[f"{n}_out_part"], d[f"{n}_out_first"] = out[0], out[2]
        d[f"{n}_out_fields"] = out[1][:, :, HARM255_CELLS] if big else out[1]
        # the far-field columns of the solved fields
        for k in range(nf):
            sl, gl = r.diag_field_all(out[1][k], c["gridmax"][k], 1e-10, 1.0, c["harm"][k], int(out[2][k]))
            d[f"{n}_diag{k}"], d[f"{n}_global{k}"] = sl, gl
    for ng, harm, first in FAR_FIELD_CASES:
        d[f"ff{ng}_diag"], d[f"ff{ng}_global"] = r.diag_field_all(far_field(ng), 6e-5, 1e-10, 1.0, harm, first)
    np.savez_compressed(os.path.join(HERE, "fft.npz"), **d)


LAT_FROM_OUT = {"aw": "aw", "ax": "ax", "ay": "ay", "ku": "ku", "kx": "kx", "ky": "ky",
                "gradx": "gradx", "grady": "grady", "qf": "qf", "qx": "qx", "qy": "qy",
                "cx": "cx", "cy": "cy", "dz": "dz", "slip": "slippage", "phase": "phaseshift",
                "z": "z"}


def run_deck(name, deck, lattice, helical):
    """Runs the reference's genesis4 on a deck; returns lattice table, loaded beam, outputs."""
    with tempfile.TemporaryDirectory() as tmp:
        with open(os.path.join(tmp, name + ".in"), "w") as f:
            f.write(deck)
        with open(os.path.join(tmp, name + ".lat"), "w") as f:
            f.write(lattice)
        subprocess.run([GENESIS, name + ".in"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        out = read_raw(os.path.join(tmp, name + ".out.h5.raw"))
        par = read_raw(os.path.join(tmp, name + "_init.par.h5.raw"))
    latg = out["Lattice"]
    nz = latg["aw"].size
    tab = np.zeros((nz, len(T.LAT_COLS)))
    for k, src in LAT_FROM_OUT.items():
        tab[:, T.C[k]] = latg[src][:nz]
    tab[:, T.C["helical"]] = np.where(tab[:, T.C["aw"]] > 0, float(helical), 0.0)
    beam = np.stack([par[k]["particles"].reshape(-1, 6) for k in sorted(par)])
    cur = np.array([par[k]["current"][0] for k in sorted(par)])
    return tab, beam, cur, out


def gen_example1():
    ex = os.path.join(REF_DIR, "examples", "Example1-SteadyState")
    deck = open(os.path.join(ex, "Example1.in")).read()
    lattice = open(os.path.join(ex, "Example1.lat")).read()
    # dump the loaded beam before tracking: &write after &beam
    deck = deck.replace("&track", "&write\nbeam=Example1_init\n&end\n\n&track", 1)
    tab, beam, cur, out = run_deck("Example1", deck, lattice, helical=True)
    np.savez_compressed(os.path.join(HERE, "example1.npz"), lat=tab, beam=beam, current=cur,
                        gammaref=11357.82, lambda0=1e-10, gridmax=2e-4, ngrid=255, power0=5e3,
                        waist=30e-6, power=out["Field"]["power"], bunching=out["Beam"]["bunching"],
                        energy=out["Beam"]["energy"], xsize=out["Beam"]["xsize"],
                        fieldxsize=out["Field"]["xsize"])


CONFIG0_DECK = """&setup
rootname=cfg0
lattice=cfg0.lat
beamline=FEL
lambda0=1e-10
gamma0=11357.8
delz=0.015
shotnoise=0
nbins=4
npart=8192
seed=1
&end

&field
power=1e3
dgrid=1e-4
ngrid=151
waist_size=30e-6
&end

&beam
current=3000
delgam=2.0
ex=0.4e-6
ey=0.4e-6
betax=15
betay=15
alphax=0
alphay=0
&end

&write
beam=cfg0_init
&end

&track
&end
"""
CONFIG0_LAT = """UND: UNDULATOR = {lambdau=0.015, nwig=110, aw=1.7};
QF: QUADRUPOLE = {l=0.08, k1=1.5};
QD: QUADRUPOLE = {l=0.08, k1=-1.5};
FEL: LINE = {UND,QF,UND,QD,UND,QF,UND};
"""


def gen_config0():
    tab, beam, cur, out = run_deck("cfg0", CONFIG0_DECK, CONFIG0_LAT, helical=False)
    np.savez_compressed(os.path.join(HERE, "config0.npz"), lat=tab, beam=beam, current=cur,
                        gammaref=11357.8, lambda0=1e-10, gridmax=1e-4, ngrid=151, power0=1e3,
                        waist=30e-6, power=out["Field"]["power"], bunching=out["Beam"]["bunching"],
                        energy=out["Beam"]["energy"])


def main():
    if not REF_DIR:
        sys.exit("set G4_REFERENCE_DIR to the reference source tree")
    r = G.reference()
    if r is None or not os.path.exists(GENESIS):
        sys.exit("the reference checker is not built: run oracle/build_oracle.py with the reference present")
    if sys.argv[1:] == ["spacecharge"]:
        gen_space_charge(r)
        return
    if sys.argv[1:] == ["wakes"]:
        gen_wakes(r)
        return
    if sys.argv[1:] == ["chicane"]:
        gen_chicane(r)
        return
    if sys.argv[1:] == ["one4one"]:
        gen_one4one(r)
        return
    if sys.argv[1:] == ["incoherent"]:
        gen_incoherent(r)
        return
    if sys.argv[1:] == ["fft"]:
        gen_fft(r)
        return
    gen_space_charge(r)
    gen_wakes(r)
    gen_chicane(r)
    gen_one4one(r)
    gen_incoherent(r)
    gen_fft(r)
    gen_streams(r)
    gen_loading(r)
    gen_steps(r)
    gen_example1()
    gen_config0()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
