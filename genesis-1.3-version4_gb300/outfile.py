"""The reference's output file (.out.h5) from the engine's diagnostics.

Diagnostic::writeToOutputFile (src/Core/Diagnostic.cpp:136-240) writes the groups
  Lattice  the per-step lattice vectors and zplot (the output positions), 1-D;
  Global   gamma0, lambdaref, sample, slen, one4one, time, scan, s and frequency, 1-D;
  Beam     per output step and slice [nz][ns]: energy, energyspread, positions and sizes,
           bunching and bunchingphase (bunchingN / bunchingphaseN for harmonics N), the
           auxiliary extremes, current, Twiss values; Global/* per output step [nz];
  Field    (FieldN for harmonic N) power, positions and sizes, near- and far-field
           intensity and phase, far-field pointing and divergence [nz][ns]; Global/* [nz];
           gridspacing, dgrid, ngrid [1];
every dataset with the string attribute "unit" (DiagBeam::getTags and DiagField::getTags,
Diagnostic.cpp:283-372, 661-715), with the output filter's defaults (Setup.cpp:155-164)
except that the Global values are always written; the auxiliary fields (efield,
wakefield, LSCfield, SSCfield) are not. Values come from g4gpu_run_diag / g4gpu_diag
(per-slice records), g4gpu_diag_fft (far field) and g4gpu_diag_global (window values);
the file itself from the engine's HDF5 encoder (g4gpu_h5_*).
"""
import numpy as np

import g4gpu

# our beam record columns -> (dataset, unit) of the reference
BEAM_UNITS = {"energy": "mc^2", "energyspread": "mc^2", "xposition": "m", "xsize": "m", "yposition": "m",
              "ysize": "m", "pxposition": "rad", "pyposition": "rad", "emitx": "m", "emity": "m", "betax": "m",
              "betay": "m", "alphax": "rad", "alphay": "rad", "xmin": "m", "xmax": "m", "pxmin": "rad",
              "pxmax": "rad", "ymin": "m", "ymax": "m", "pymin": "rad", "pymax": "rad", "emin": "mc^2",
              "emax": "mc^2"}
FIELD_UNITS = {"power": "W", "xposition": "m", "xsize": "m", "yposition": "m", "ysize": "m",
               "intensity-nearfield": "W/m^2", "phase-nearfield": "rad", "intensity-farfield": "W/rad^2",
               "phase-farfield": "rad", "xpointing": "rad", "xdivergence": "rad", "ypointing": "rad",
               "ydivergence": "rad"}
BEAM_GLOBAL_UNITS = {"energy": "mc^2", "energyspread": "mc^2", "xposition": "m", "xsize": "m",
                     "yposition": "m", "ysize": "m"}
FIELD_GLOBAL_UNITS = {"energy": "J", "xposition": "m", "xsize": "m", "yposition": "m", "ysize": "m",
                      "intensity-nearfield": "W/m^2", "intensity-farfield": "W/rad^2", "xpointing": "rad",
                      "xdivergence": "rad", "ypointing": "rad", "ydivergence": "rad"}
# lattice table column -> (dataset, unit), Diagnostic.cpp:150-171
LATTICE = [("z", "z", "m"), ("dz", "dz", "m"), ("aw", "aw", " "), ("ax", "ax", "m"), ("ay", "ay", "m"),
           ("ku", "ku", "m^{-1}"), ("kx", "kx", " "), ("ky", "ky", " "), ("qf", "qf", "m^{-2}"),
           ("qx", "qx", "m"), ("qy", "qy", "m"), ("cx", "cx", "rad"), ("cy", "cy", "rad"),
           ("gradx", "gradx", "m^{-1}"), ("grady", "grady", "m^{-1}"), ("slip", "slippage", " "),
           ("phase", "phaseshift", "rad")]


def write_out(path, cfg, lattice, zout, beam, field, current, fft=None, chicanes=None, nharm=1, time_run=None):
    """Writes the reference's .out.h5 layout.

    cfg: g4gpu.Config of the run; lattice: [nsteps][18] table; zout [nz]: the output
    positions; beam [nz][ns][24 + 2 nharm] and field [nz][nfield][ns][9] (g4gpu_run_diag
    records); current [ns] (A); fft [nz][nfield][ns][4] or None; chicanes [nsteps][4]
    (angle in rad, lb, ld, lt) or None."""
    ns, nf = cfg.nslice, cfg.nfield
    beam = np.asarray(beam, dtype=np.float64)
    field = np.asarray(field, dtype=np.float64)
    nz = beam.shape[0]
    with g4gpu.H5Writer(path) as w:
        # Lattice
        w.dataset("Lattice/zplot", np.asarray(zout, dtype=np.float64), "m")
        lat = np.asarray(lattice, dtype=np.float64)
        for col, name, unit in LATTICE:
            w.dataset("Lattice/" + name, lat[:, _lat_col(col)], unit)
        ch = np.zeros((lat.shape[0], 4)) if chicanes is None else np.asarray(chicanes, dtype=np.float64)
        # the reference stores Undulator::chic_angle, the bend angle in rad, under the
        # unit "degree" (Diagnostic.cpp:168)
        w.dataset("Lattice/chic_angle", ch[:, 0], "degree")
        for k, name in ((1, "chic_lb"), (2, "chic_ld"), (3, "chic_lt")):
            w.dataset("Lattice/" + name, ch[:, k], "m")
        # Global (Diagnostic.cpp:173-201)
        slicelength = cfg.lambda0 * cfg.sample
        tr = cfg.time_run if time_run is None else time_run
        w.dataset("Global/gamma0", [cfg.gammaref], "mc^2")
        w.dataset("Global/lambdaref", [cfg.lambda0], "m")
        w.dataset("Global/sample", [cfg.sample], " ")
        w.dataset("Global/slen", [slicelength * ns], "m")
        w.dataset("Global/one4one", [0.0], " ")
        w.dataset("Global/time", [1.0 if tr else 0.0], " ")
        w.dataset("Global/scan", [0.0], " ")
        w.dataset("Global/s", np.arange(ns) * slicelength, "m")
        e0 = 1239.842e-9 / cfg.lambda0
        df = 0.0 if ns == 1 else e0 * cfg.lambda0 / slicelength / ns
        w.dataset("Global/frequency", e0 + np.arange(ns) * df - 0.5 * df * ns, "eV")
        # Beam
        for k, name in enumerate(g4gpu.DB_COLS):
            w.dataset("Beam/" + name, beam[:, :, k], BEAM_UNITS[name])
        for h in range(nharm):
            sfx = "" if h == 0 else str(h + 1)
            w.dataset(f"Beam/bunching{sfx}", beam[:, :, len(g4gpu.DB_COLS) + 2 * h], " ")
            w.dataset(f"Beam/bunchingphase{sfx}", beam[:, :, len(g4gpu.DB_COLS) + 2 * h + 1], "rad")
        cur = np.asarray(current, dtype=np.float64)
        w.dataset("Beam/current", np.tile(cur, (nz, 1)), "A")  # per output step (filter current on)
        bg = np.array([g4gpu.diag_global(cfg, nharm, cur, beam[i], None)[0] for i in range(nz)])
        for k, name in enumerate(g4gpu.DBG_COLS):
            w.dataset("Beam/Global/" + name, bg[:, k], BEAM_GLOBAL_UNITS[name])
        # Field, FieldN
        for k in range(nf):
            h = int(cfg.harm[k])
            grp = "Field" if h == 1 else f"Field{h}"
            for c, name in enumerate(g4gpu.DF_COLS):
                w.dataset(f"{grp}/{name}", field[:, k, :, c], FIELD_UNITS[name])
            if fft is not None:
                ff = np.asarray(fft, dtype=np.float64)
                for c, name in enumerate(g4gpu.DFFT_COLS):
                    w.dataset(f"{grp}/{name}", ff[:, k, :, c], FIELD_UNITS[name])
            fg = np.array([g4gpu.diag_global(cfg, nharm, cur, None, field[i], None if fft is None else
                                             np.asarray(fft)[i])[1][k] for i in range(nz)])
            for c, name in enumerate(g4gpu.DFG_COLS):
                if fft is None and name in g4gpu.DFFT_COLS:
                    continue
                w.dataset(f"{grp}/Global/{name}", fg[:, c], FIELD_GLOBAL_UNITS[name])
            dgrid = 2 * cfg.gridmax[k] / (cfg.ngrid - 1)
            w.dataset(f"{grp}/gridspacing", [dgrid], "m")
            w.dataset(f"{grp}/dgrid", [cfg.gridmax[k]], "m")
            w.dataset(f"{grp}/ngrid", [float(cfg.ngrid)], " ")
        # Meta (Output::writeMeta, the version record)
        for name, v in (("Major", 4), ("Minor", 6), ("Revision", 14), ("Beta", 0)):
            w.dataset(f"Meta/Version/{name}", [float(v)], " ")


_LAT = ["aw", "ax", "ay", "ku", "kx", "ky", "gradx", "grady", "qf", "qx", "qy", "cx", "cy", "dz", "slip", "phase",
        "helical", "z"]


def _lat_col(name):
    return _LAT.index(name)


def write_fld(path, cfg, ifld, field, first, s0=0.0):
    """The reference's field dump (.fld.h5, WriteFieldHDF5::writeMain,
    src/IO/writeFieldHDF5.cpp:42-130): Meta/Version, wavelength, slicespacing, refposition,
    gridsize (m), gridpoints and slicecount (int), and per slice in window order
    sliceNNNNNN/field-real and field-imag, the field scaled by dgrid eev / ks / sqrt(vacimp)
    (sqrt(W) per cell). field [nslice][ngrid^2] complex in storage order with ring start
    `first` (g4gpu_get_field)."""
    ns, ng = cfg.nslice, cfg.ngrid
    h = int(cfg.harm[ifld])
    xlambda = cfg.lambda0 / h
    dgrid = 2 * cfg.gridmax[ifld] / (ng - 1)
    ks = 4.0 * np.arcsin(1.0) / xlambda
    scl = dgrid * 510998.95069 / ks / np.sqrt(376.73)
    f = np.asarray(field).reshape(ns, ng * ng)
    with g4gpu.H5Writer(path) as w:
        for name, v in (("Major", 4), ("Minor", 6), ("Revision", 14), ("Beta", 0)):
            w.dataset(f"Meta/Version/{name}", [float(v)], " ")
        w.dataset("wavelength", [xlambda], "m")
        w.dataset("slicespacing", [cfg.lambda0 * cfg.sample], "m")
        w.dataset("refposition", [s0], "m")
        w.dataset("gridsize", [dgrid], "m")
        w.dataset_int("gridpoints", [ng])
        w.dataset_int("slicecount", [ns])
        for i in range(ns):
            s = f[(i + int(first)) % ns]
            w.dataset(f"slice{i + 1:06d}/field-real", scl * s.real, " ")
            w.dataset(f"slice{i + 1:06d}/field-imag", scl * s.imag, " ")


def write_par(path, cfg, particles, current, nbins, counts=None, s0=0.0):
    """The reference's particle dump (.par.h5, WriteBeamHDF5::writeMain,
    src/IO/writeBeamHDF5.cpp:14-188): Meta/Version, slicelength (the reference length),
    slicespacing, refposition (m), beamletsize, slicecount, one4one (int), and per slice
    sliceNNNNNN/current (A), gamma, theta (rad), x, y (m), px, py (rad). particles
    [nslice][npart][6] (g4gpu_get_beam), counts per slice for one4one windows."""
    ns = cfg.nslice
    p = np.asarray(particles).reshape(ns, -1, 6)
    cur = np.asarray(current, dtype=np.float64)
    with g4gpu.H5Writer(path) as w:
        for name, v in (("Major", 4), ("Minor", 6), ("Revision", 14), ("Beta", 0)):
            w.dataset(f"Meta/Version/{name}", [float(v)], " ")
        w.dataset("slicelength", [cfg.lambda0], "m")
        w.dataset("slicespacing", [cfg.lambda0 * cfg.sample], "m")
        w.dataset("refposition", [s0], "m")
        w.dataset_int("beamletsize", [nbins])
        w.dataset_int("slicecount", [ns])
        w.dataset_int("one4one", [1 if counts is not None else 0])
        for i in range(ns):
            n = p.shape[1] if counts is None else int(counts[i])
            g = f"slice{i + 1:06d}"
            w.dataset(f"{g}/current", [cur[i]], "A")
            for c, (name, unit) in enumerate((("gamma", " "), ("theta", "rad"), ("x", "m"), ("y", "m"),
                                               ("px", "rad"), ("py", "rad"))):
                w.dataset(f"{g}/{name}", p[i, :n, c], unit)
