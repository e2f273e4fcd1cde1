"""Python binding of the GB300 engine's C ABI (include/g4gpu.h) via ctypes.

This module is a thin wrapper: every call goes to lib/libg4gpu.so, which runs
the undulator step as CUDA kernels on the GPU. There is no CPU fallback; if the
library is missing, load_library() raises.

Usage:
    import g4gpu
    cfg = g4gpu.Config(nslice=..., npart=..., ngrid=..., ...)
    with g4gpu.Handle(cfg) as h:
        h.set_lattice(table)              # [nsteps][LAT_NCOL]
        h.load_beam(particles, current)   # [ns][np][6], [ns]
        h.load_field(0, field, first=0)   # [ns][ngrid*ngrid] complex
        h.run(0, nsteps)
        beam_diag, field_diag = h.diag(nharm=1)
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libg4gpu.so")

MAX_FIELDS = 8
MAX_HARM = 16
PLAIN, MIXED = 0, 1
SOLVER_ADI, SOLVER_FFT = 0, 1
STAGE_PUSH, STAGE_FIELD, STAGE_SLIP, STAGE_ALL = 1, 2, 4, 7
ERR_ARG, ERR_CUDA, ERR_STATE, ERR_DEVICE, ERR_NOMEM = 1, 2, 3, 4, 5

LAT_COLS = ["aw", "ax", "ay", "ku", "kx", "ky", "gradx", "grady", "qf", "qx", "qy",
            "cx", "cy", "dz", "slip", "phase", "helical", "z"]
LAT_NCOL = len(LAT_COLS)
DB_COLS = ["energy", "energyspread", "xposition", "xsize", "yposition", "ysize",
           "pxposition", "pyposition", "emitx", "emity", "betax", "betay", "alphax",
           "alphay", "xmin", "xmax", "pxmin", "pxmax", "ymin", "ymax", "pymin", "pymax",
           "emin", "emax"]
DF_COLS = ["power", "xposition", "xsize", "yposition", "ysize", "intensity-nearfield",
           "phase-nearfield", "intensity-farfield", "phase-farfield"]
DFFT_COLS = ["xpointing", "xdivergence", "ypointing", "ydivergence"]
G4GPU_DPI_FIELD, G4GPU_DPI_BEAM = 0, 1
DBG_COLS = ["energy", "energyspread", "xposition", "xsize", "yposition", "ysize"]
DFG_COLS = ["energy", "xposition", "xsize", "yposition", "ysize", "intensity-nearfield",
            "intensity-farfield", "xpointing", "xdivergence", "ypointing", "ydivergence"]
KERNEL_CLASSES = ["push", "adi_x", "adi_y", "fft", "slip", "diag", "misc", "sc", "sc_field", "step"]

# exported symbols of include/g4gpu.h
ABI_SYMBOLS = [
    "g4gpu_config_defaults", "g4gpu_create", "g4gpu_destroy", "g4gpu_last_error",
    "g4gpu_set_lattice", "g4gpu_load_beam", "g4gpu_get_beam", "g4gpu_load_field",
    "g4gpu_get_field", "g4gpu_set_efield", "g4gpu_run", "g4gpu_synchronize", "g4gpu_diag", "g4gpu_run_diag", "g4gpu_diag_fft", "g4gpu_diag_global", "g4gpu_get_config",
    "g4gpu_dpi_open", "g4gpu_dpi_kind", "g4gpu_dpi_nobj", "g4gpu_dpi_multi", "g4gpu_dpi_obj_name",
    "g4gpu_dpi_info", "g4gpu_dpi_field", "g4gpu_dpi_beam", "g4gpu_dpi_field_from", "g4gpu_dpi_beam_from",
    "g4gpu_dpi_close", "g4gpu_get_stream",
    "g4gpu_set_profiling", "g4gpu_kernel_stats", "g4gpu_reset_stats", "g4gpu_device_bytes",
    "g4gpu_measure_fp64_rate", "g4gpu_slip_shifts", "g4gpu_slip_count", "g4gpu_slice_bytes",
    "g4gpu_shift_out", "g4gpu_shift_in",
    "g4gpu_host_load_beam", "g4gpu_host_gauss_hermite", "g4gpu_host_fc", "g4gpu_host_single_wakes",
    "g4gpu_set_wake", "g4gpu_set_chicanes", "g4gpu_load_beam_counts", "g4gpu_get_counts", "g4gpu_sort",
    "g4gpu_apply_slippage", "g4gpu_set_incoherent", "g4gpu_h5_create", "g4gpu_h5_dataset", "g4gpu_h5_dataset_int",
    "g4gpu_h5_close",
    "g4gpu_set_graph_mode", "g4gpu_autotune", "g4gpu_batch_create", "g4gpu_batch_destroy",
    "g4gpu_batch_member", "g4gpu_batch_run", "g4gpu_batch_synchronize",
    "g4gpu_mlp_create", "g4gpu_mlp_destroy", "g4gpu_mlp_last_error", "g4gpu_mlp_num_params",
    "g4gpu_mlp_get_params", "g4gpu_mlp_set_params", "g4gpu_mlp_set_normalization", "g4gpu_mlp_forward",
    "g4gpu_mlp_gradients", "g4gpu_mlp_train", "g4gpu_closure_attach", "g4gpu_closure_features",
    "g4gpu_closure_apply", "g4gpu_closure_targets", "g4gpu_copy_state", "g4gpu_run_learned",
    "g4gpu_set_field_substeps",
    "g4gpu_adi_advance_noalloc", "g4gpu_set_launch_shapes",
]
CLOSURE_NIN, CLOSURE_NOUT = 32, 4
NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024
NOALLOC_MAX_NGRID = 168


class G4Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"g4gpu error {code}: {msg}")
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [
        ("nslice", ctypes.c_int), ("npart", ctypes.c_int), ("ngrid", ctypes.c_int),
        ("nfield", ctypes.c_int), ("harm", ctypes.c_int * MAX_FIELDS),
        ("gridmax", ctypes.c_double * MAX_FIELDS), ("lambda0", ctypes.c_double),
        ("sample", ctypes.c_double), ("gammaref", ctypes.c_double),
        ("precision", ctypes.c_int), ("solver", ctypes.c_int), ("source_filter", ctypes.c_int),
        ("xcut", ctypes.c_double), ("ycut", ctypes.c_double), ("sigmoid", ctypes.c_double),
        ("time_run", ctypes.c_int), ("periodic", ctypes.c_int), ("device", ctypes.c_int),
    ]

    def __init__(self, **kw):
        super().__init__()
        _lib().g4gpu_config_defaults(ctypes.byref(self))
        harm = kw.pop("harm", None)
        gridmax = kw.pop("gridmax", None)
        for k, v in kw.items():
            if not hasattr(self, k):
                raise TypeError(f"unknown config field {k}")
            setattr(self, k, v)
        if harm is not None:
            harm = list(np.atleast_1d(harm))
            self.nfield = len(harm)
            for i, h in enumerate(harm):
                self.harm[i] = int(h)
        if gridmax is not None:
            gm = list(np.atleast_1d(gridmax))
            if len(gm) == 1 and self.nfield > 1:
                gm = gm * self.nfield
            for i, g in enumerate(gm):
                self.gridmax[i] = float(g)


_LIB = None


def load_library(path=None):
    """Loads lib/libg4gpu.so; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} is missing: build it with genesis-1.3-version4_gb300/build.py")
    L = ctypes.CDLL(p)
    P = ctypes.POINTER
    d, i, vp, pd = ctypes.c_double, ctypes.c_int, ctypes.c_void_p, P(ctypes.c_double)
    L.g4gpu_config_defaults.argtypes = [P(Config)]
    L.g4gpu_config_defaults.restype = None
    L.g4gpu_create.argtypes = [P(Config), P(vp)]
    L.g4gpu_destroy.argtypes = [vp]
    L.g4gpu_destroy.restype = None
    L.g4gpu_last_error.argtypes = [vp]
    L.g4gpu_last_error.restype = ctypes.c_char_p
    L.g4gpu_set_lattice.argtypes = [vp, i, pd]
    L.g4gpu_load_beam.argtypes = [vp, vp, vp]
    L.g4gpu_get_beam.argtypes = [vp, vp]
    L.g4gpu_load_field.argtypes = [vp, i, vp, i, d]
    L.g4gpu_get_field.argtypes = [vp, i, vp, P(i), pd]
    L.g4gpu_set_efield.argtypes = [vp, d, i, i, i, i]
    L.g4gpu_run.argtypes = [vp, i, i, i]
    L.g4gpu_synchronize.argtypes = [vp]
    L.g4gpu_diag.argtypes = [vp, i, vp, vp]
    L.g4gpu_run_diag.argtypes = [vp, i, i, i, vp, vp]
    L.g4gpu_diag_fft.argtypes = [vp, vp]
    L.g4gpu_measure_fp64_rate.argtypes = [i, pd]
    L.g4gpu_slip_shifts.argtypes = [pd, d, d, P(i)]
    L.g4gpu_slip_count.argtypes = [vp, i, d, P(i), P(i)]
    L.g4gpu_slice_bytes.argtypes = [vp]
    L.g4gpu_slice_bytes.restype = ctypes.c_size_t
    L.g4gpu_shift_out.argtypes = [vp, i, i, vp]
    L.g4gpu_shift_in.argtypes = [vp, i, vp]
    L.g4gpu_diag_global.argtypes = [P(Config), i, vp, vp, vp, vp, vp, vp]
    L.g4gpu_get_config.argtypes = [vp, P(Config)]
    L.g4gpu_dpi_open.argtypes = [ctypes.c_char_p, ctypes.c_char_p, i, P(vp), ctypes.c_char_p, i]
    for nm in ("g4gpu_dpi_kind", "g4gpu_dpi_nobj", "g4gpu_dpi_multi"):
        getattr(L, nm).argtypes = [vp]
    L.g4gpu_dpi_obj_name.argtypes = [vp, i, ctypes.c_char_p, i]
    L.g4gpu_dpi_info.argtypes = [vp, ctypes.c_char_p, i]
    L.g4gpu_dpi_field.argtypes = [vp, i, i, i, d, d, i, vp, i, vp]
    L.g4gpu_dpi_beam.argtypes = [vp, i, i, i, vp, vp]
    L.g4gpu_dpi_field_from.argtypes = [vp, vp, i, i, vp]
    L.g4gpu_dpi_beam_from.argtypes = [vp, vp, i, vp]
    L.g4gpu_dpi_close.argtypes = [vp]
    L.g4gpu_dpi_close.restype = None
    L.g4gpu_get_stream.argtypes = [vp, P(vp)]
    L.g4gpu_set_profiling.argtypes = [vp, i]
    L.g4gpu_kernel_stats.argtypes = [vp, P(ctypes.c_longlong), pd]
    L.g4gpu_reset_stats.argtypes = [vp]
    L.g4gpu_device_bytes.argtypes = [vp]
    L.g4gpu_device_bytes.restype = ctypes.c_size_t
    L.g4gpu_host_load_beam.argtypes = [i, i, i, i, i, i, d, d, pd, pd]
    L.g4gpu_host_gauss_hermite.argtypes = [pd, d, i, pd]
    L.g4gpu_host_fc.argtypes = [d, i, i]
    L.g4gpu_host_fc.restype = d
    L.g4gpu_host_single_wakes.argtypes = [i, d, d, d, d, i, d, d, d, d, pd, pd, pd]
    L.g4gpu_set_wake.argtypes = [vp, i, d, pd, pd, pd, pd, d, d, i]
    L.g4gpu_set_chicanes.argtypes = [vp, i, pd]
    L.g4gpu_set_field_substeps.argtypes = [vp, i, ctypes.POINTER(ctypes.c_int)]
    L.g4gpu_load_beam_counts.argtypes = [vp, vp, vp, P(i)]
    L.g4gpu_get_counts.argtypes = [vp, P(i)]
    L.g4gpu_sort.argtypes = [vp, P(i)]
    L.g4gpu_apply_slippage.argtypes = [vp, i, d]
    L.g4gpu_set_incoherent.argtypes = [vp, i, i, i, i]
    L.g4gpu_h5_create.argtypes = [ctypes.c_char_p, P(vp)]
    L.g4gpu_h5_dataset.argtypes = [vp, ctypes.c_char_p, i, P(ctypes.c_longlong), pd, ctypes.c_char_p]
    L.g4gpu_h5_dataset_int.argtypes = [vp, ctypes.c_char_p, i, P(i)]
    L.g4gpu_h5_close.argtypes = [vp]
    L.g4gpu_set_graph_mode.argtypes = [vp, i]
    L.g4gpu_autotune.argtypes = [vp, P(i), P(i), P(i)]
    L.g4gpu_set_launch_shapes.argtypes = [vp, i, i, i]
    L.g4gpu_batch_create.argtypes = [i, P(Config), P(vp)]
    L.g4gpu_batch_destroy.argtypes = [vp]
    L.g4gpu_batch_destroy.restype = None
    L.g4gpu_batch_member.argtypes = [vp, i]
    L.g4gpu_batch_member.restype = vp
    L.g4gpu_batch_run.argtypes = [vp, i, i, i]
    L.g4gpu_batch_synchronize.argtypes = [vp]
    pf = P(ctypes.c_float)
    L.g4gpu_mlp_create.argtypes = [i, i, i, i, i, P(vp)]
    L.g4gpu_mlp_destroy.argtypes = [vp]
    L.g4gpu_mlp_destroy.restype = None
    L.g4gpu_mlp_last_error.argtypes = [vp]
    L.g4gpu_mlp_last_error.restype = ctypes.c_char_p
    L.g4gpu_mlp_num_params.argtypes = [vp]
    L.g4gpu_mlp_num_params.restype = ctypes.c_size_t
    L.g4gpu_mlp_get_params.argtypes = [vp, pf]
    L.g4gpu_mlp_set_params.argtypes = [vp, pf]
    L.g4gpu_mlp_set_normalization.argtypes = [vp, pf, pf, pf, pf]
    L.g4gpu_mlp_forward.argtypes = [vp, pf, i, pf]
    L.g4gpu_mlp_gradients.argtypes = [vp, pf, pf, i, pf, pf]
    L.g4gpu_mlp_train.argtypes = [vp, pf, pf, i, i, i, ctypes.c_float, i, pf]
    L.g4gpu_closure_attach.argtypes = [vp, vp, d, d, d]
    L.g4gpu_closure_features.argtypes = [vp, pf]
    L.g4gpu_closure_apply.argtypes = [vp, pf]
    L.g4gpu_closure_targets.argtypes = [vp, vp, pf]
    L.g4gpu_copy_state.argtypes = [vp, vp]
    L.g4gpu_run_learned.argtypes = [vp, vp, i, i, P(i), P(i), i, d, P(i), P(i), pd]
    L.g4gpu_adi_advance_noalloc.argtypes = [vp, vp, i, i, i, d, d, d, i, vp]
    for name in ABI_SYMBOLS:
        if not hasattr(L, name):
            raise ImportError(f"{p} does not export {name}")
    _LIB = L
    return L


def _lib():
    return load_library()


def _pd(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _vp(a):
    return ctypes.c_void_p(a.ctypes.data)


def host_load_beam(slicepar, islice0, npart, nbins, seed, shotnoise, lambda0, sample, out=None):
    """Quiet loading + shot noise on the host, bit-exact with the reference.
    `out` may be a preallocated C-contiguous float64 array [ns][npart][6]."""
    sp = np.ascontiguousarray(slicepar, dtype=np.float64).reshape(-1, 17)
    if out is None:
        out = np.zeros((sp.shape[0], npart, 6))
    elif out.shape != (sp.shape[0], npart, 6) or out.dtype != np.float64 or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous float64 array [ns][npart][6]")
    rc = _lib().g4gpu_host_load_beam(sp.shape[0], islice0, npart, nbins, seed, int(shotnoise),
                                     lambda0, sample, _pd(sp), _pd(out))
    if rc:
        raise G4Error(rc, "host_load_beam: invalid arguments")
    return out


def host_gauss_hermite(par, gridmax, ngrid):
    par = np.ascontiguousarray(par, dtype=np.float64)
    out = np.zeros((ngrid * ngrid, 2))
    rc = _lib().g4gpu_host_gauss_hermite(_pd(par), gridmax, ngrid, _pd(out))
    if rc:
        raise G4Error(rc, "host_gauss_hermite: invalid arguments")
    return out[:, 0] + 1j * out[:, 1]


def slip_shifts(accuslip, slippage, sample):
    """Control::applySlippage's bookkeeping on the host (g4gpu_slip_shifts): returns
    (shifts, direction, new accumulated slippage)."""
    acc = ctypes.c_double(float(accuslip))
    dr = ctypes.c_int()
    n = _lib().g4gpu_slip_shifts(ctypes.byref(acc), float(slippage), float(sample), ctypes.byref(dr))
    if n < 0:
        raise ValueError("invalid slippage arguments")
    return n, dr.value, acc.value


def host_fc(aw, helical, h):
    return _lib().g4gpu_host_fc(aw, int(helical), h)


class H5Writer:
    """An HDF5 file of FP64 datasets with a "unit" attribute each (the reference's output
    layout), written at close: w.dataset("Beam/energy", array, "mc^2")."""

    def __init__(self, path):
        self.L = _lib()
        self.f = ctypes.c_void_p()
        rc = self.L.g4gpu_h5_create(os.fsencode(path), ctypes.byref(self.f))
        if rc:
            raise G4Error(rc, f"cannot create {path}")

    def dataset(self, path, data, unit=" "):
        a = np.ascontiguousarray(data, dtype=np.float64)
        if a.ndim == 0:
            a = a.reshape(1)
        dims = (ctypes.c_longlong * a.ndim)(*a.shape)
        rc = self.L.g4gpu_h5_dataset(self.f, path.encode(), a.ndim, dims, _pd(a), unit.encode())
        if rc:
            raise G4Error(rc, f"h5 dataset {path}: bad path, shape or a duplicate name")

    def dataset_int(self, path, data):
        a = np.ascontiguousarray(data, dtype=np.int32).ravel()
        rc = self.L.g4gpu_h5_dataset_int(self.f, path.encode(), a.size, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        if rc:
            raise G4Error(rc, f"h5 dataset {path}: bad path or a duplicate name")

    def close(self):
        if self.f:
            rc = self.L.g4gpu_h5_close(self.f)
            self.f = None
            if rc:
                raise G4Error(rc, "h5 file could not be written")

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def host_single_wakes(ns, ds, radius=2.5e-3, conductivity=0.0, relaxation=0.0, roundpipe=True, gap=0.0, lgap=1.0,
                      hrough=0.0, lrough=1.0):
    """Single-particle wakes (resistive, geometric, roughness) on ns points spaced ds,
    with the &wake namelist's parameters and defaults."""
    out = [np.zeros(int(ns)) for _ in range(3)]
    rc = _lib().g4gpu_host_single_wakes(int(ns), float(ds), float(radius), float(conductivity), float(relaxation),
                                        int(bool(roundpipe)), float(gap), float(lgap), float(hrough), float(lrough),
                                        *[_pd(a) for a in out])
    if rc:
        raise G4Error(rc, "host_single_wakes: invalid arguments")
    return tuple(out)


class Handle:
    """One time window resident on the GPU (g4gpu_handle)."""

    def __init__(self, cfg):
        self.L = _lib()
        self.cfg = cfg
        h = ctypes.c_void_p()
        rc = self.L.g4gpu_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc:
            raise G4Error(rc, self.L.g4gpu_last_error(None).decode())
        self.h = h

    def _check(self, rc):
        if rc:
            raise G4Error(rc, self.L.g4gpu_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.g4gpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ncell(self):
        return self.cfg.ngrid * self.cfg.ngrid

    def set_lattice(self, table):
        t = np.ascontiguousarray(table, dtype=np.float64).reshape(-1, LAT_NCOL)
        self._check(self.L.g4gpu_set_lattice(self.h, t.shape[0], _pd(t)))
        self.nsteps = t.shape[0]

    def load_beam(self, particles, current):
        """particles: host array [ns][np][6] (any memory, pinned is fastest)."""
        p = particles if (isinstance(particles, np.ndarray) and particles.flags.c_contiguous and
                          particles.dtype == np.float64) else np.ascontiguousarray(particles, np.float64)
        c = np.ascontiguousarray(current, dtype=np.float64)
        if p.size != self.cfg.nslice * self.cfg.npart * 6 or c.size != self.cfg.nslice:
            raise ValueError("particle or current array has the wrong size")
        self._check(self.L.g4gpu_load_beam(self.h, _vp(p), _vp(c)))

    def load_beam_counts(self, particles, current, counts):
        """A one4one window: particles [ns][np][6] of which the first counts[is] of every
        slice are used (np is a slice's capacity)."""
        p = np.ascontiguousarray(particles, np.float64)
        c = np.ascontiguousarray(current, dtype=np.float64)
        n = np.ascontiguousarray(counts, dtype=np.int32)
        if p.size != self.cfg.nslice * self.cfg.npart * 6 or c.size != self.cfg.nslice or n.size != self.cfg.nslice:
            raise ValueError("particle, current or count array has the wrong size")
        self._check(self.L.g4gpu_load_beam_counts(self.h, _vp(p), _vp(c), n.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))

    def get_counts(self):
        n = np.zeros(self.cfg.nslice, dtype=np.int32)
        self._check(self.L.g4gpu_get_counts(self.h, n.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return n

    def set_incoherent(self, seed=1234, do_loss=False, do_spread=False, nbins=1):
        """Incoherent synchrotron radiation (&sponrad) for the following steps."""
        self._check(self.L.g4gpu_set_incoherent(self.h, int(seed), int(bool(do_loss)), int(bool(do_spread)),
                                                int(nbins)))

    def apply_slippage(self, ifld, slippage):
        """Control::applySlippage of field ifld outside the step loop."""
        self._check(self.L.g4gpu_apply_slippage(self.h, int(ifld), float(slippage)))

    # ---- a window sharded over ranks (one handle per rank) ----
    def slip_count(self, ifld, slippage):
        """(shifts, direction) the step's slippage yields for field ifld
        (g4gpu_slip_count: Control::applySlippage's bookkeeping)."""
        n, dr = ctypes.c_int(), ctypes.c_int()
        self._check(self.L.g4gpu_slip_count(self.h, int(ifld), float(slippage), ctypes.byref(n), ctypes.byref(dr)))
        return n.value, dr.value

    def slice_bytes(self):
        return int(self.L.g4gpu_slice_bytes(self.h))

    def shift_out(self, ifld, direction, send_ptr):
        """Copies the slice leaving this block to the device address send_ptr (0: none)
        and frees its slot for the entering slice."""
        self._check(self.L.g4gpu_shift_out(self.h, int(ifld), int(direction),
                                           ctypes.c_void_p(send_ptr) if send_ptr else None))

    def shift_in(self, ifld, recv_ptr):
        """Fills the entering slice from the device address recv_ptr (0: zeros)."""
        self._check(self.L.g4gpu_shift_in(self.h, int(ifld), ctypes.c_void_p(recv_ptr) if recv_ptr else None))

    def sort(self):
        """Beam::sort for the window (one4one); returns the field shift (0)."""
        sh = ctypes.c_int(0)
        self._check(self.L.g4gpu_sort(self.h, ctypes.byref(sh)))
        return sh.value

    def load_beam_ptr(self, particles_ptr, current_ptr):
        """Same as load_beam with raw host pointers (e.g. pinned torch tensors)."""
        self._check(self.L.g4gpu_load_beam(self.h, ctypes.c_void_p(particles_ptr),
                                           ctypes.c_void_p(current_ptr)))

    def get_beam(self, out=None):
        if out is None:
            out = np.empty((self.cfg.nslice, self.cfg.npart, 6))
        self._check(self.L.g4gpu_get_beam(self.h, _vp(out)))
        return out

    def load_field(self, ifld, field, first=0, accuslip=0.0):
        f = np.ascontiguousarray(field, dtype=np.complex128)
        if f.size != self.cfg.nslice * self.ncell:
            raise ValueError("field array has the wrong size")
        self._check(self.L.g4gpu_load_field(self.h, ifld, _vp(f), int(first), float(accuslip)))

    def load_field_ptr(self, ifld, ptr, first=0, accuslip=0.0):
        self._check(self.L.g4gpu_load_field(self.h, ifld, ctypes.c_void_p(ptr), int(first), float(accuslip)))

    def get_field(self, ifld, out=None):
        if out is None:
            out = np.empty((self.cfg.nslice, self.ncell), dtype=np.complex128)
        first = ctypes.c_int()
        acc = ctypes.c_double()
        self._check(self.L.g4gpu_get_field(self.h, ifld, _vp(out), ctypes.byref(first), ctypes.byref(acc)))
        return out, first.value, acc.value

    def slippage_state(self, ifld):
        first = ctypes.c_int()
        acc = ctypes.c_double()
        self._check(self.L.g4gpu_get_field(self.h, ifld, None, ctypes.byref(first), ctypes.byref(acc)))
        return first.value, acc.value

    def run(self, istep0, nsteps, stages=STAGE_ALL):
        self._check(self.L.g4gpu_run(self.h, istep0, nsteps, stages))

    def synchronize(self):
        self._check(self.L.g4gpu_synchronize(self.h))

    def diag(self, nharm=1, beam=True, field=True):
        ns = self.cfg.nslice
        b = np.zeros((ns, len(DB_COLS) + 2 * nharm)) if beam else None
        f = np.zeros((self.cfg.nfield, ns, len(DF_COLS))) if field else None
        self._check(self.L.g4gpu_diag(self.h, nharm, _vp(b) if beam else None,
                                      _vp(f) if field else None))
        return b, f

    def diag_fft(self):
        """Far-field xpointing, xdivergence, ypointing, ydivergence [nfield][nslice][4]
        (g4gpu_diag_fft)."""
        out = np.zeros((self.cfg.nfield, self.cfg.nslice, len(DFFT_COLS)))
        self._check(self.L.g4gpu_diag_fft(self.h, _vp(out)))
        return out

    def run_diag(self, istep0, nsteps, nharm=1, beam=True, field=True, out=None):
        """Runs nsteps steps from istep0 and returns the per-slice diagnostics after
        every step: beam [nsteps][nslice][cols], field [nsteps][nfield][nslice][cols]
        (g4gpu_run_diag). `out` may pass preallocated (beam, field) arrays."""
        ns = self.cfg.nslice
        if out is not None:
            b, f = out
        else:
            b = np.zeros((nsteps, ns, len(DB_COLS) + 2 * nharm)) if beam else None
            f = np.zeros((nsteps, self.cfg.nfield, ns, len(DF_COLS))) if field else None
        self._check(self.L.g4gpu_run_diag(self.h, int(istep0), int(nsteps), nharm,
                                          _vp(b) if b is not None else None,
                                          _vp(f) if f is not None else None))
        return b, f

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self.L.g4gpu_get_stream(self.h, ctypes.byref(s)))
        return s.value

    def set_profiling(self, on):
        self._check(self.L.g4gpu_set_profiling(self.h, int(on)))

    def kernel_stats(self):
        n = len(KERNEL_CLASSES)
        la = (ctypes.c_longlong * n)()
        ms = (ctypes.c_double * n)()
        self._check(self.L.g4gpu_kernel_stats(self.h, la, ms))
        return {k: (int(la[i]), float(ms[i])) for i, k in enumerate(KERNEL_CLASSES)}

    def reset_stats(self):
        self._check(self.L.g4gpu_reset_stats(self.h))

    def device_bytes(self):
        return int(self.L.g4gpu_device_bytes(self.h))

    def set_field_substeps(self, counts):
        """Periods per lattice step (g4gpu_set_field_substeps): a step of c > 1 periods
        pushes once over its length and deposits and slips period by period, then
        diffracts once."""
        cnt = np.ascontiguousarray(counts, dtype=np.int32).ravel()
        self._check(self.L.g4gpu_set_field_substeps(self.h, int(cnt.size),
                                                    cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))

    def set_chicanes(self, table):
        """Chicanes of the lattice steps: [nsteps][4] angle, lb, ld, lt (zero angle: none)."""
        t = np.ascontiguousarray(table, dtype=np.float64).reshape(-1, 4)
        self._check(self.L.g4gpu_set_chicanes(self.h, int(t.shape[0]), _pd(t)))

    def set_wake(self, ext=None, res=None, geo=None, rou=None, ds=None, ztrans=0.0, radius=2.5e-3,
                 transient=False):
        """Wakes for the following steps: external loss per slice (eV/m) and the
        single-particle wakes on the fine grid (nslice * sample points spaced ds, the
        reference length by default); ext None switches them off."""
        if ext is None:
            self._check(self.L.g4gpu_set_wake(self.h, 0, 0.0, None, None, None, None, 0.0, 0.0, 0))
            return
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ext, res, geo, rou)]
        if arrs[0].size != self.cfg.nslice or not (arrs[1].size == arrs[2].size == arrs[3].size):
            raise ValueError("ext needs nslice values and res, geo, rou one length")
        ds = self.cfg.lambda0 if ds is None else ds
        self._check(self.L.g4gpu_set_wake(self.h, int(arrs[1].size), float(ds), *[_pd(a) for a in arrs],
                                          float(ztrans), float(radius), int(bool(transient))))

    def set_efield(self, rmax=0.0, ngrid=100, nz=0, nphi=0, longrange=False):
        """Space charge for the following steps (&efield: rmax, ngrid, nz, nphi,
        longrange, with the namelist's defaults); nz = 0 and longrange False switch it
        off. Resets the radial grid extent to rmax."""
        self._check(self.L.g4gpu_set_efield(self.h, float(rmax), int(ngrid), int(nz), int(nphi),
                                            int(bool(longrange))))

    def set_graph_mode(self, on):
        self._check(self.L.g4gpu_set_graph_mode(self.h, int(on)))

    def closure_attach(self, mlp, waist, u0=1.0, c0=1.0):
        self._mlp = mlp  # keep the network alive while attached
        self._check(self.L.g4gpu_closure_attach(self.h, mlp.m, waist, u0, c0))

    def closure_features(self):
        out = np.zeros((self.cfg.nslice, CLOSURE_NIN), dtype=np.float32)
        self._check(self.L.g4gpu_closure_features(self.h, _pf(out)))
        return out

    def closure_apply(self, corr):
        corr = np.ascontiguousarray(corr, dtype=np.float32)
        self._check(self.L.g4gpu_closure_apply(self.h, _pf(corr)))

    def closure_targets(self, fine):
        out = np.zeros((self.cfg.nslice, CLOSURE_NOUT), dtype=np.float32)
        self._check(self.L.g4gpu_closure_targets(self.h, fine.h, _pf(out)))
        return out

    def copy_state_from(self, other):
        self._check(self.L.g4gpu_copy_state(self.h, other.h))

    def run_learned(self, fine, istep0, ncoarse, fine_start, fine_count, check_every=8, tol=0.01):
        fs = np.ascontiguousarray(fine_start, dtype=np.int32)
        fc = np.ascontiguousarray(fine_count, dtype=np.int32)
        nchk, nfb = ctypes.c_int(), ctypes.c_int()
        emax = ctypes.c_double()
        self._check(self.L.g4gpu_run_learned(self.h, fine.h, istep0, ncoarse,
                                             fs.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                             fc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), check_every, tol,
                                             ctypes.byref(nchk), ctypes.byref(nfb), ctypes.byref(emax)))
        return nchk.value, nfb.value, emax.value

    def set_launch_shapes(self, push_block, field_threads, field_kernel):
        self._check(self.L.g4gpu_set_launch_shapes(self.h, push_block, field_threads, field_kernel))

    def autotune(self):
        """(push threads per block, field kernel threads per CTA, field kernel: 0 one
        CTA per slice, 1 a cluster pair)"""
        pb, ft, fk = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self.L.g4gpu_autotune(self.h, ctypes.byref(pb), ctypes.byref(ft), ctypes.byref(fk)))
        return pb.value, ft.value, fk.value


def diag_global(cfg, nharm, current=None, beam_diag=None, field_diag=None, fft_diag=None):
    """Window ("Global/") values from one state's per-slice diagnostics
    (g4gpu_diag_global): (beam [6] or None, field [nfield][11] or None)."""
    L = _lib()
    c = np.ascontiguousarray(current, dtype=np.float64) if current is not None else None
    bd = np.ascontiguousarray(beam_diag, dtype=np.float64) if beam_diag is not None else None
    fd = np.ascontiguousarray(field_diag, dtype=np.float64) if field_diag is not None else None
    qd = np.ascontiguousarray(fft_diag, dtype=np.float64) if fft_diag is not None else None
    bg = np.zeros(len(DBG_COLS)) if bd is not None else None
    fg = np.zeros((cfg.nfield, len(DFG_COLS))) if fd is not None else None
    rc = L.g4gpu_diag_global(ctypes.byref(cfg), nharm, _vp(c) if c is not None else None,
                             _vp(bd) if bd is not None else None, _vp(fd) if fd is not None else None,
                             _vp(qd) if qd is not None else None, _vp(bg) if bg is not None else None,
                             _vp(fg) if fg is not None else None)
    if rc != 0:
        raise G4Error(rc, "g4gpu_diag_global: bad arguments")
    return bg, fg


class Plugin:
    """A diagnostic plugin (DPI) built against the reference's plugin interface.
    field()/beam() return {object name: [nslice] values by window slice}."""

    def __init__(self, libfile, parameter="", verbose=0):
        self.L = _lib()
        self.p = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        rc = self.L.g4gpu_dpi_open(os.fsencode(libfile), parameter.encode(), int(verbose), ctypes.byref(self.p),
                                   err, 512)
        if rc != 0:
            raise G4Error(rc, err.value.decode())
        self.kind = self.L.g4gpu_dpi_kind(self.p)
        self.multi = bool(self.L.g4gpu_dpi_multi(self.p))
        buf = ctypes.create_string_buffer(512)
        self.names = []
        for k in range(self.L.g4gpu_dpi_nobj(self.p)):
            self.L.g4gpu_dpi_obj_name(self.p, k, buf, 512)
            self.names.append(buf.value.decode())
        self.L.g4gpu_dpi_info(self.p, buf, 512)
        self.info = buf.value.decode()

    def _named(self, out):
        return {nm: out[k] for k, nm in enumerate(self.names)}

    def field(self, field, first, iz, harm, ngrid, dgrid, xlambda):
        f = np.ascontiguousarray(field, dtype=np.complex128)
        ns = f.shape[0]
        out = np.zeros((len(self.names), ns))
        rc = self.L.g4gpu_dpi_field(self.p, int(iz), int(harm), int(ngrid), float(dgrid), float(xlambda), ns,
                                    _vp(f), int(first), _vp(out))
        if rc != 0:
            raise G4Error(rc, "g4gpu_dpi_field")
        return self._named(out)

    def beam(self, particles, iz):
        part = np.ascontiguousarray(particles, dtype=np.float64)
        out = np.zeros((len(self.names), part.shape[0]))
        rc = self.L.g4gpu_dpi_beam(self.p, int(iz), part.shape[0], part.shape[1], _vp(part), _vp(out))
        if rc != 0:
            raise G4Error(rc, "g4gpu_dpi_beam")
        return self._named(out)

    def field_from(self, handle, ifld, iz):
        out = np.zeros((len(self.names), handle.cfg.nslice))
        handle._check(self.L.g4gpu_dpi_field_from(self.p, handle.h, int(ifld), int(iz), _vp(out)))
        return self._named(out)

    def beam_from(self, handle, iz):
        out = np.zeros((len(self.names), handle.cfg.nslice))
        handle._check(self.L.g4gpu_dpi_beam_from(self.p, handle.h, int(iz), _vp(out)))
        return self._named(out)

    def close(self):
        if self.p:
            self.L.g4gpu_dpi_close(self.p)
            self.p = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def adi_advance_noalloc(field_ptr, source_ptr, nslice, ngrid, first, delz, dgrid, xks, device=0,
                        stream=None):
    """One single-precision ADI step of nslice field slices at device address
    field_ptr ([nslice][ngrid^2] complex float, in place) with the source at
    source_ptr (beam-slice order, or None), allocating no device memory
    (g4gpu_adi_advance_noalloc). Returns after the step has finished."""
    L = _lib()
    rc = L.g4gpu_adi_advance_noalloc(ctypes.c_void_p(field_ptr),
                                     ctypes.c_void_p(source_ptr) if source_ptr else None,
                                     nslice, ngrid, first, delz, dgrid, xks, device,
                                     ctypes.c_void_p(stream) if stream else None)
    if rc:
        raise G4Error(rc, L.g4gpu_last_error(None).decode())


def _pf(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class MLP:
    """BF16 tensor-core MLP of the learned closure (g4gpu_mlp)."""

    def __init__(self, nin=CLOSURE_NIN, width=256, nout=CLOSURE_NOUT, seed=0, device=0):
        self.L = _lib()
        m = ctypes.c_void_p()
        rc = self.L.g4gpu_mlp_create(nin, width, nout, seed, device, ctypes.byref(m))
        if rc:
            raise G4Error(rc, self.L.g4gpu_last_error(None).decode())
        self.m = m
        self.nin, self.width, self.nout = nin, width, nout

    def _check(self, rc):
        if rc:
            raise G4Error(rc, self.L.g4gpu_mlp_last_error(self.m).decode())

    @property
    def num_params(self):
        return int(self.L.g4gpu_mlp_num_params(self.m))

    def get_params(self):
        out = np.zeros(self.num_params, dtype=np.float32)
        self._check(self.L.g4gpu_mlp_get_params(self.m, _pf(out)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.L.g4gpu_mlp_set_params(self.m, _pf(p)))

    def set_normalization(self, fmean, fstd, oshift, oscale):
        a = [np.ascontiguousarray(x, dtype=np.float32) for x in (fmean, fstd, oshift, oscale)]
        self._check(self.L.g4gpu_mlp_set_normalization(self.m, *[_pf(x) for x in a]))

    def forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.nout), dtype=np.float32)
        self._check(self.L.g4gpu_mlp_forward(self.m, _pf(X), X.shape[0], _pf(Y)))
        return Y

    def gradients(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        self._check(self.L.g4gpu_mlp_gradients(self.m, _pf(X), _pf(T), X.shape[0], _pf(g), _pf(loss)))
        return g, float(loss[0])

    def train(self, X, T, epochs=10, batch=1024, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        curve = np.zeros(epochs, dtype=np.float32)
        self._check(self.L.g4gpu_mlp_train(self.m, _pf(X), _pf(T), X.shape[0], epochs, batch, lr, seed,
                                           _pf(curve)))
        return curve

    def close(self):
        if getattr(self, "m", None):
            self.L.g4gpu_mlp_destroy(self.m)
            self.m = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Member(Handle):
    """A handle owned by a Batch (not destroyed on its own)."""

    def __init__(self, L, h, cfg):
        self.L = L
        self.cfg = cfg
        self.h = ctypes.c_void_p(h)

    def close(self):
        self.h = None


class Batch:
    """An ensemble of independent runs (g4gpu_batch)."""

    def __init__(self, cfgs):
        self.L = _lib()
        n = len(cfgs)
        arr = (Config * n)(*cfgs)
        b = ctypes.c_void_p()
        rc = self.L.g4gpu_batch_create(n, arr, ctypes.byref(b))
        if rc:
            raise G4Error(rc, self.L.g4gpu_last_error(None).decode())
        self.b = b
        self.members = [_Member(self.L, self.L.g4gpu_batch_member(b, i), cfgs[i]) for i in range(n)]

    def run(self, istep0, nsteps, stages=STAGE_ALL):
        rc = self.L.g4gpu_batch_run(self.b, istep0, nsteps, stages)
        if rc:
            raise G4Error(rc, self.L.g4gpu_last_error(None).decode())

    def synchronize(self):
        rc = self.L.g4gpu_batch_synchronize(self.b)
        if rc:
            raise G4Error(rc, self.L.g4gpu_last_error(None).decode())

    def close(self):
        if getattr(self, "b", None):
            for m in self.members:
                m.h = None
            self.L.g4gpu_batch_destroy(self.b)
            self.b = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
