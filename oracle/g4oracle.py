"""ctypes bindings for the CPU checker libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py, never by the product path.

Two libraries share one calling convention:
  * liborc   — oracle/g4oracle.c, the plain-C FP64 restatement (built by
               oracle/build_oracle.py; travels to every machine);
  * libg4ref — the GENESIS 1.3 v4 reference compiled from its own sources by
               oracle/ref_build/Makefile (only where the reference is present).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libg4ref.so")

# lattice table columns (oracle/g4oracle.h G4_LAT_*)
LAT_COLS = ["aw", "ax", "ay", "ku", "kx", "ky", "gradx", "grady", "qf", "qx", "qy",
            "cx", "cy", "dz", "slip", "phase", "helical", "z"]
LAT_NCOL = len(LAT_COLS)
LAT = {k: i for i, k in enumerate(LAT_COLS)}

DB_COLS = ["energy", "energyspread", "xposition", "xsize", "yposition", "ysize",
           "pxposition", "pyposition", "emitx", "emity", "betax", "betay", "alphax",
           "alphay", "xmin", "xmax", "pxmin", "pxmax", "ymin", "ymax", "pymin", "pymax",
           "emin", "emax"]
DF_COLS = ["power", "xposition", "xsize", "yposition", "ysize", "intensity-nearfield",
           "phase-nearfield", "intensity-farfield", "phase-farfield"]

_P = ctypes.POINTER
_d = ctypes.c_double
_i = ctypes.c_int
_pd = _P(ctypes.c_double)
_pi = _P(ctypes.c_int)


def _ptr(a, t=_pd):
    return a.ctypes.data_as(t)


class _Lib:
    def __init__(self, path, prefix):
        self.path = path
        self.lib = ctypes.CDLL(path)
        self.p = prefix
        L = self.lib
        f = getattr(L, prefix + "run_steps")
        f.restype = _i
        self.has_accuslip = prefix == "orc_"
        if self.has_accuslip:
            f.argtypes = [_i, _pd, _d, _i, _i, _pd, _pd, _d, _d, _i, _pi, _i, _pd, _pd, _pi,
                          _pd, _i, _i, _i, _i, _pd, _i]
        else:
            f.argtypes = [_i, _pd, _d, _i, _i, _pd, _pd, _d, _d, _i, _pi, _i, _pd, _pd, _pi,
                          _i, _i, _i]
        getattr(L, prefix + "ran2").argtypes = [_i, _i, _pd]
        getattr(L, prefix + "hammersley").argtypes = [_i, _i, _i, _pd]
        getattr(L, prefix + "inverfc").argtypes = [_i, _pd, _pd]
        getattr(L, prefix + "besselj").argtypes = [_i, _d]
        getattr(L, prefix + "besselj").restype = _d
        getattr(L, prefix + "fc").argtypes = [_d, _i, _i]
        getattr(L, prefix + "fc").restype = _d
        getattr(L, prefix + "load_beam").argtypes = [_i, _i, _i, _i, _i, _i, _d, _d, _pd, _pd]
        getattr(L, prefix + "gauss_hermite").argtypes = [_pd, _d, _i, _pd]
        if prefix == "g4ref_":
            L.g4ref_set_solver.argtypes = [_i, _pd]
            L.g4ref_diag_field.argtypes = [_i, _i, _d, _d, _d, _i, _pd, _i, _pd, _pd]
            L.g4ref_diag_field.restype = _i
        if prefix == "orc_":
            L.orc_diag_beam.argtypes = [_i, _i, _pd, _i, _pd]
            L.orc_diag_field.argtypes = [_i, _i, _d, _d, _i, _pd, _i, _pd]
            L.orc_diag_field_fft.argtypes = [_i, _i, _d, _d, _i, _pd, _i, _pd]
            L.orc_diag_global_beam.argtypes = [_i, _i, _pd, _pd, _pd]
            L.orc_diag_global_field.argtypes = [_i, _i, _d, _d, _i, _d, _pd, _pd]
            L.orc_deposit_source.argtypes = [_pd, _i, _i, _i, _pd, _pd, _d, _i, _i, _d, _pd]
            L.orc_adi_advance.argtypes = [_i, _i, _i, _d, _d, _d, _pd, _pd]

    def set_incoherent(self, seed=1234, do_loss=False, do_spread=False, nbins=1):
        """Incoherent synchrotron radiation (&sponrad) of the following run_steps calls."""
        f = getattr(self.lib, self.p + "set_incoherent")
        f.argtypes = [_i, _i, _i, _i]
        f(int(seed), int(bool(do_loss)), int(bool(do_spread)), int(nbins))

    def set_counts(self, counts=None, sort_every=0):
        """One4one window of the following run_steps calls: particles per slice (None
        clears), and a sort after the push of every sort_every-th step."""
        f = getattr(self.lib, self.p + "set_one4one" if self.p == "g4ref_" else self.p + "set_counts")
        f.argtypes = [_i, _pi, _i]
        if counts is None:
            f(0, None, 0)
            return
        c = np.ascontiguousarray(counts, dtype=np.int32)
        f(int(c.size), _ptr(c, _pi), int(sort_every))

    def get_counts(self, ns):
        out = np.zeros(ns, dtype=np.int32)
        f = getattr(self.lib, self.p + "get_counts")
        f.argtypes = [_i, _pi]
        f(int(ns), _ptr(out, _pi))
        return out

    def sort(self, particles, counts, current, reflength, sample):
        """Beam::sort of a one4one window (oracle only): returns (particles, counts,
        current, lost)."""
        part = np.array(particles, dtype=np.float64, order="C", copy=True)
        cnt = np.array(counts, dtype=np.int32, copy=True)
        cur = np.array(current, dtype=np.float64, copy=True)
        self.lib.orc_sort.argtypes = [_i, _i, _pd, _pi, _pd, _d, _d]
        lost = self.lib.orc_sort(part.shape[0], part.shape[1], _ptr(part), _ptr(cnt, _pi), _ptr(cur),
                                 float(reflength), float(sample))
        return part, cnt, cur, lost

    def set_chicanes(self, table=None):
        """Chicanes [nsteps][4] (angle, lb, ld, lt) of the following run_steps calls'
        lattice rows; None clears them."""
        f = getattr(self.lib, self.p + "set_chicanes")
        f.argtypes = [_i, _pd]
        if table is None:
            f(0, None)
            return
        t = np.ascontiguousarray(table, dtype=np.float64).reshape(-1, 4)
        self._chic_keep = t
        f(int(t.shape[0]), _ptr(t))

    def set_wake(self, ext=None, res=None, geo=None, rou=None, ds=1e-10, ztrans=0.0, radius=2.5e-3,
                 transient=False):
        """Wakes (&wake) for the following run_steps calls: external loss per slice (eV/m)
        and the single-particle wakes on the fine grid; no arguments switch them off."""
        f = getattr(self.lib, self.p + "set_wake")
        f.argtypes = [_i, _i, _i, _d, _pd, _pd, _pd, _pd, _d, _d, _i]
        if ext is None:
            f(0, 0, 0, 0.0, None, None, None, None, 0.0, 0.0, 0)
            return
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ext, res, geo, rou)]
        self._wake_keep = arrs
        f(1, int(arrs[1].size), int(arrs[0].size), float(ds), *[_ptr(a) for a in arrs], float(ztrans),
          float(radius), int(bool(transient)))

    def single_wakes(self, ns, ds, radius=2.5e-3, conductivity=0.0, relaxation=0.0, roundpipe=True, gap=0.0,
                     lgap=1.0, hrough=0.0, lrough=1.0):
        """The reference's single-particle wakes (resistive, geometric, roughness) on ns
        points spaced ds; compiled reference only."""
        f = getattr(self.lib, self.p + "single_wakes")
        f.argtypes = [_i, _d, _d, _d, _d, _i, _d, _d, _d, _d, _pd, _pd, _pd]
        out = [np.zeros(ns) for _ in range(3)]
        f(int(ns), float(ds), float(radius), float(conductivity), float(relaxation), int(bool(roundpipe)),
          float(gap), float(lgap), float(hrough), float(lrough), *[_ptr(a) for a in out])
        return tuple(out)

    def set_efield(self, rmax=0.0, ngrid=0, nz=0, nphi=0, longrange=False):
        """Space charge (&efield) for the following run_steps calls; the defaults switch it off."""
        f = getattr(self.lib, self.p + "set_efield")
        f.argtypes = [_d, _i, _i, _i, _i]
        f(float(rmax), int(ngrid), int(nz), int(nphi), int(bool(longrange)))

    def ran2(self, seed, n):
        out = np.zeros(n)
        getattr(self.lib, self.p + "ran2")(seed, n, _ptr(out))
        return out

    def hammersley(self, base_index, start, n):
        out = np.zeros(n)
        getattr(self.lib, self.p + "hammersley")(base_index, start, n, _ptr(out))
        return out

    def inverfc(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros_like(x)
        getattr(self.lib, self.p + "inverfc")(x.size, _ptr(x), _ptr(out))
        return out

    def besselj(self, n, x):
        return getattr(self.lib, self.p + "besselj")(n, x)

    def fc(self, aw, helical, h):
        return getattr(self.lib, self.p + "fc")(aw, int(helical), h)

    def load_beam(self, slicepar, islice0, npart, nbins, seed, shotnoise, lam, sample):
        slicepar = np.ascontiguousarray(slicepar, dtype=np.float64).reshape(-1, 17)
        ns = slicepar.shape[0]
        out = np.zeros((ns, npart, 6))
        getattr(self.lib, self.p + "load_beam")(ns, islice0, npart, nbins, seed, int(shotnoise),
                                                lam, sample, _ptr(slicepar), _ptr(out))
        return out

    def gauss_hermite(self, par, gridmax, ngrid):
        par = np.ascontiguousarray(par, dtype=np.float64)
        out = np.zeros((ngrid * ngrid, 2))
        getattr(self.lib, self.p + "gauss_hermite")(_ptr(par), gridmax, ngrid, _ptr(out))
        return out[:, 0] + 1j * out[:, 1]

    def run_steps(self, lat, gammaref, particles, current, reflength, sample, harm, gridmax,
                  fields, first, time_run=True, periodic=False, stages=7, solver=0,
                  filt=None, nthreads=1, accuslip=None):
        """Runs the steps of `lat` in place on copies; returns (particles, fields, first, accuslip)."""
        lat = np.ascontiguousarray(lat, dtype=np.float64).reshape(-1, LAT_NCOL)
        part = np.array(particles, dtype=np.float64, order="C", copy=True)
        ns, npart = part.shape[0], part.shape[1]
        cur = np.ascontiguousarray(current, dtype=np.float64)
        harm = np.ascontiguousarray(harm, dtype=np.int32)
        nfld = harm.size
        gm = np.ascontiguousarray(gridmax, dtype=np.float64).reshape(nfld)
        f = np.array(fields, dtype=np.complex128, order="C", copy=True).reshape(nfld, ns, -1)
        ngrid = int(round(np.sqrt(f.shape[2])))
        fv = f.view(np.float64)
        fst = np.ascontiguousarray(first, dtype=np.int32).reshape(nfld).copy()
        fn = getattr(self.lib, self.p + "run_steps")
        if self.has_accuslip:
            acc = np.zeros(nfld) if accuslip is None else np.array(accuslip, dtype=np.float64)
            fl = np.ones(3) if filt is None else np.ascontiguousarray(filt, dtype=np.float64)
            rc = fn(lat.shape[0], _ptr(lat), gammaref, ns, npart, _ptr(part), _ptr(cur),
                    reflength, sample, nfld, _ptr(harm, _pi), ngrid, _ptr(gm), _ptr(fv),
                    _ptr(fst, _pi), _ptr(acc), int(time_run), int(periodic), stages, solver,
                    _ptr(fl), nthreads)
        else:
            # the reference's FieldSolverFFT runs on the FFTW stand-in of oracle/ref_build
            fl = np.ones(3) if filt is None else np.ascontiguousarray(filt, dtype=np.float64)
            acc = None
            self.lib.g4ref_set_solver(int(solver), _ptr(fl))
            try:
                rc = fn(lat.shape[0], _ptr(lat), gammaref, ns, npart, _ptr(part), _ptr(cur),
                        reflength, sample, nfld, _ptr(harm, _pi), ngrid, _ptr(gm), _ptr(fv),
                        _ptr(fst, _pi), int(time_run), int(periodic), stages)
            finally:
                self.lib.g4ref_set_solver(0, None)
        if rc != 0:
            raise RuntimeError(f"{self.p}run_steps failed: {rc}")
        return part, f, fst, acc

    def diag_field_all(self, field, gridmax, reflength, sample, harm, first):
        """The reference's DiagField::getValues with every filter on (reference build
        only): per slice [ns][13] by window slice (DF_COLS, then xpointing, xdivergence,
        ypointing, ydivergence) and the window values [11] (energy, x/y position and
        size, mean near- and far-field intensity, far-field pointing and divergence)."""
        f = np.ascontiguousarray(field, dtype=np.complex128)
        ns = f.shape[0]
        ngrid = int(round(np.sqrt(f.shape[1])))
        out = np.zeros((ns, 13))
        glob = np.zeros(11)
        rc = self.lib.g4ref_diag_field(ns, ngrid, gridmax, reflength, sample, harm, _ptr(f.view(np.float64)),
                                       int(first), _ptr(out), _ptr(glob))
        if rc != 0:
            raise RuntimeError(f"g4ref_diag_field failed: {rc}")
        return out, glob

    def diag_beam(self, particles, nharm):
        part = np.ascontiguousarray(particles, dtype=np.float64)
        ns, npart = part.shape[0], part.shape[1]
        out = np.zeros((ns, len(DB_COLS) + 2 * nharm))
        self.lib.orc_diag_beam(ns, npart, _ptr(part), nharm, _ptr(out))
        return out

    def diag_field(self, field, gridmax, lambda0, harm, first):
        f = np.ascontiguousarray(field, dtype=np.complex128)
        ns = f.shape[0]
        ngrid = int(round(np.sqrt(f.shape[1])))
        out = np.zeros((ns, len(DF_COLS)))
        self.lib.orc_diag_field(ns, ngrid, gridmax, lambda0, harm, _ptr(f.view(np.float64)),
                                int(first), _ptr(out))
        return out

    def diag_global_beam(self, particles, current):
        """Window values of the beam [6] (energy, energyspread, x/y position and size)."""
        part = np.ascontiguousarray(particles, dtype=np.float64)
        out = np.zeros(6)
        self.lib.orc_diag_global_beam(part.shape[0], part.shape[1], _ptr(part),
                                      _ptr(np.ascontiguousarray(current, dtype=np.float64)), _ptr(out))
        return out

    def diag_global_field(self, field, gridmax, lambda0, harm, sample):
        """Window values of one field [11] (energy J, x/y position and size, mean near-
        and far-field intensity, far-field pointing and divergence)."""
        f = np.ascontiguousarray(field, dtype=np.complex128)
        ns = f.shape[0]
        ngrid = int(round(np.sqrt(f.shape[1])))
        out = np.zeros(11)
        self.lib.orc_diag_global_field(ns, ngrid, gridmax, lambda0, harm, sample, _ptr(f.view(np.float64)),
                                       _ptr(out))
        return out

    def diag_field_fft(self, field, gridmax, lambda0, harm, first):
        """Far-field xpointing, xdivergence, ypointing, ydivergence [ns][4] by window slice."""
        f = np.ascontiguousarray(field, dtype=np.complex128)
        ns = f.shape[0]
        ngrid = int(round(np.sqrt(f.shape[1])))
        out = np.zeros((ns, 4))
        self.lib.orc_diag_field_fft(ns, ngrid, gridmax, lambda0, harm, _ptr(f.view(np.float64)),
                                    int(first), _ptr(out))
        return out

    def deposit_source(self, lat, istep, particles, current, reflength, harm, ngrid, gridmax):
        """Source term [ns][ngrid^2] complex of one field at lattice step istep."""
        lat = np.ascontiguousarray(lat, dtype=np.float64).reshape(-1, LAT_NCOL)
        part = np.ascontiguousarray(particles, dtype=np.float64)
        ns, npart = part.shape[0], part.shape[1]
        cur = np.ascontiguousarray(current, dtype=np.float64)
        out = np.zeros((ns, ngrid * ngrid), dtype=np.complex128)
        self.lib.orc_deposit_source(_ptr(lat), istep, ns, npart, _ptr(part), _ptr(cur), reflength,
                                    harm, ngrid, gridmax, _ptr(out.view(np.float64)))
        return out

    def adi_advance(self, field, source, first, delz, dgrid, xks):
        """One ADI step of every slice of `field` [ns][ngrid^2] (storage order) with
        `source` [ns][ngrid^2] in beam-slice order, or None; returns a new array."""
        f = np.array(field, dtype=np.complex128, order="C", copy=True)
        ns, ngrid = f.shape[0], int(round(np.sqrt(f.shape[1])))
        src = None if source is None else np.ascontiguousarray(source, dtype=np.complex128)
        self.lib.orc_adi_advance(ns, ngrid, int(first), delz, dgrid, xks, _ptr(f.view(np.float64)),
                                 None if src is None else _ptr(src.view(np.float64)))
        return f


_oracle = None
_ref = None


def oracle(path=None):
    global _oracle
    if _oracle is None or (path and _oracle.path != path):
        _oracle = _Lib(path or ORACLE_SO, "orc_")
    return _oracle


def reference(path=None):
    """The compiled reference checker, or None where it was not built."""
    global _ref
    p = path or REF_SO
    if _ref is None:
        if not os.path.exists(p):
            return None
        _ref = _Lib(p, "g4ref_")
    return _ref
