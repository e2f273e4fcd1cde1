/* g4gpu.h — C ABI of the GB300 engine for the GENESIS 1.3 v4 undulator step.
 *
 * One handle owns one time window (or, with the batch entry points, an ensemble of
 * independent runs) resident in GPU memory: particles in structure-of-arrays form,
 * the complex radiation field of every harmonic, and the per-step lattice tables.
 * Every call returns 0 on success or a G4GPU_ERR_* code; g4gpu_last_error() gives
 * the message. No call traps the device: kernels that detect an inconsistency
 * (an index outside the grid) set a device flag that the next synchronising call
 * reports as G4GPU_ERR_DEVICE.
 *
 * What each entry point replaces in the reference (GENESIS 1.3 v4.6.14, paths
 * within svenreiche/Genesis-1.3-Version4) is cited beside it. The integration step
 * g4gpu_run() replaces the body of the step loop in src/Core/Gencore.cpp:102-147:
 * Beam::track (src/Core/Beam.cpp:296-311), Field::track for every field
 * (src/Core/Field.cpp:177-185 → FieldSolver::advance, include/FieldSolver.h:20-26)
 * and Control::applySlippage (src/Core/Control.cpp:158-276).
 *
 * Array conventions:
 *   particles  [nslice][npart][6] doubles (gamma, theta, x, y, px, py) — the
 *              reference's Particle record (include/Particle.h:6-13) per slice
 *   current    [nslice] doubles, Beam::current (include/Beam.h)
 *   field      [nslice][ngrid*ngrid][2] doubles (re, im) in storage order; window
 *              slice j sits in storage slot (j + first) % nslice (include/Field.h:57-59)
 *   lattice    [nsteps][G4GPU_LAT_NCOL] doubles, one row per integration step, the
 *              per-step vectors of the reference's Undulator (include/Undulator.h:58-62)
 */
#ifndef G4GPU_H
#define G4GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define G4GPU_ABI_VERSION 1
#define G4GPU_MAX_FIELDS 8
#define G4GPU_MAX_HARM 16

/* status codes */
#define G4GPU_OK 0
#define G4GPU_ERR_ARG 1     /* invalid argument or configuration */
#define G4GPU_ERR_CUDA 2    /* a CUDA runtime call failed */
#define G4GPU_ERR_STATE 3   /* call out of order (e.g. run before load) */
#define G4GPU_ERR_DEVICE 4  /* a kernel raised the device error flag */
#define G4GPU_ERR_NOMEM 5   /* device allocation failed */

/* arithmetic of the step */
#define G4GPU_PLAIN 0 /* FP64 everywhere, the reference's arithmetic */
#define G4GPU_MIXED 1 /* FP32 field, solver, deposition and transverse optics; the
                         accumulated phase as a 64-bit fixed-point turn count (exact
                         accumulation, 2 pi / 2^32 resolution); FP64 diagnostic reductions */

/* field solver (Field::initSolver, src/Core/Field.cpp:72-83) */
#define G4GPU_SOLVER_ADI 0 /* FieldSolverADI, src/Core/FieldSolverADI.cpp */
#define G4GPU_SOLVER_FFT 1 /* FieldSolverFFT, src/Core/FieldSolverFFT.cpp */

/* stage bits for g4gpu_run */
#define G4GPU_STAGE_PUSH 1  /* Beam::track */
#define G4GPU_STAGE_FIELD 2 /* Field::track of every field */
#define G4GPU_STAGE_SLIP 4  /* Control::applySlippage of every field */
#define G4GPU_STAGE_ALL 7

/* lattice table columns: Undulator per-step vectors (include/Undulator.h:58-62);
 * the column set and order are also those of oracle/g4oracle.h */
enum {
  G4GPU_LAT_AW, G4GPU_LAT_AX, G4GPU_LAT_AY, G4GPU_LAT_KU, G4GPU_LAT_KX, G4GPU_LAT_KY,
  G4GPU_LAT_GRADX, G4GPU_LAT_GRADY, G4GPU_LAT_QF, G4GPU_LAT_QX, G4GPU_LAT_QY,
  G4GPU_LAT_CX, G4GPU_LAT_CY, G4GPU_LAT_DZ, G4GPU_LAT_SLIP, G4GPU_LAT_PHASE,
  G4GPU_LAT_HELICAL, G4GPU_LAT_Z, G4GPU_LAT_NCOL
};

/* per-slice beam diagnostic columns (DiagBeam::getValues, src/Core/Diagnostic.cpp:373-563);
 * g4gpu_diag writes these, then |b_h| and arg(b_h) for h = 1..nharm */
enum {
  G4GPU_DB_ENERGY, G4GPU_DB_ENERGYSPREAD, G4GPU_DB_XPOS, G4GPU_DB_XSIZE, G4GPU_DB_YPOS,
  G4GPU_DB_YSIZE, G4GPU_DB_PXPOS, G4GPU_DB_PYPOS, G4GPU_DB_EMITX, G4GPU_DB_EMITY,
  G4GPU_DB_BETAX, G4GPU_DB_BETAY, G4GPU_DB_ALPHAX, G4GPU_DB_ALPHAY, G4GPU_DB_XMIN,
  G4GPU_DB_XMAX, G4GPU_DB_PXMIN, G4GPU_DB_PXMAX, G4GPU_DB_YMIN, G4GPU_DB_YMAX,
  G4GPU_DB_PYMIN, G4GPU_DB_PYMAX, G4GPU_DB_EMIN, G4GPU_DB_EMAX, G4GPU_DB_NCOL
};
/* per-slice field diagnostic columns (DiagField::getValues, src/Core/Diagnostic.cpp:718-902),
 * indexed by window slice */
enum {
  G4GPU_DF_POWER, G4GPU_DF_XPOS, G4GPU_DF_XSIZE, G4GPU_DF_YPOS, G4GPU_DF_YSIZE,
  G4GPU_DF_NF_INT, G4GPU_DF_NF_PHI, G4GPU_DF_FF_INT, G4GPU_DF_FF_PHI, G4GPU_DF_NCOL
};
/* Window ("Global/") values of g4gpu_diag_global: the beam's (DiagBeam,
 * src/Core/Diagnostic.cpp:551-606) ... */
enum {
  G4GPU_DBG_ENERGY, G4GPU_DBG_ENERGYSPREAD, G4GPU_DBG_XPOS, G4GPU_DBG_XSIZE, G4GPU_DBG_YPOS, G4GPU_DBG_YSIZE,
  G4GPU_DBG_NCOL
};
/* ... and a field's (DiagField, src/Core/Diagnostic.cpp:902-975): energy [J], centroid
 * and size, mean near- and far-field intensity, far-field pointing and divergence */
enum {
  G4GPU_DFG_ENERGY, G4GPU_DFG_XPOS, G4GPU_DFG_XSIZE, G4GPU_DFG_YPOS, G4GPU_DFG_YSIZE, G4GPU_DFG_NF_INT,
  G4GPU_DFG_FF_INT, G4GPU_DFG_XPOINT, G4GPU_DFG_XDIV, G4GPU_DFG_YPOINT, G4GPU_DFG_YDIV, G4GPU_DFG_NCOL
};
/* Columns of g4gpu_diag_fft: far-field pointing and divergence [rad]
 * (DiagField with FFTW, src/Core/Diagnostic.cpp:786-847, filter "fft") */
enum {
  G4GPU_DFFT_XPOINT, G4GPU_DFFT_XDIV, G4GPU_DFFT_YPOINT, G4GPU_DFFT_YDIV, G4GPU_DFFT_NCOL
};

typedef struct {
  int nslice;    /* slices in the time window (Time::getNodeNSlice, src/Main/GenTime.cpp:64-86) */
  int npart;     /* macro particles per slice (&setup npart) */
  int ngrid;     /* transverse grid points per dimension (&field ngrid), >= 3 */
  int nfield;    /* number of radiation fields (harmonics), 1..G4GPU_MAX_FIELDS */
  int harm[G4GPU_MAX_FIELDS];       /* harmonic of each field (Field::harm) */
  double gridmax[G4GPU_MAX_FIELDS]; /* half width of each grid (&field dgrid, Field::gridmax) */
  double lambda0;  /* reference wavelength (&setup lambda0) */
  double sample;   /* slice spacing in units of lambda0 (&time sample) */
  double gammaref; /* reference energy (&setup gamma0, Undulator::getGammaRef) */
  int precision;   /* G4GPU_PLAIN or G4GPU_MIXED */
  int solver;      /* G4GPU_SOLVER_ADI or G4GPU_SOLVER_FFT (&track fft_fieldsolver) */
  int source_filter;    /* &track source_filter (FFT solver only) */
  double xcut, ycut, sigmoid; /* &track xcut, ycut, sigmoid */
  int time_run;    /* time-dependent run: slippage is applied (Control::timerun) */
  int periodic;    /* &track periodic: the window wraps instead of zero-filling */
  int device;      /* CUDA device ordinal */
} g4gpu_config;

typedef struct g4gpu_ctx *g4gpu_handle;

/* Fills *cfg with the reference's defaults (Setup.cpp:7-47, Track.cpp:4-15). */
void g4gpu_config_defaults(g4gpu_config *cfg);

/* Creates a handle and allocates the device arrays for cfg.
 * Replaces the allocation in Beam::init (src/Core/Beam.cpp:221-238) and
 * Field::init (src/Core/Field.cpp:34-70) plus Field::initSolver (Field.cpp:72-83). */
int g4gpu_create(const g4gpu_config *cfg, g4gpu_handle *out);

/* Releases the handle and its device memory. */
void g4gpu_destroy(g4gpu_handle h);

/* Message of the last failed call on h (or of the last failed g4gpu_create when h
 * is NULL); never NULL. */
const char *g4gpu_last_error(g4gpu_handle h);

/* Uploads the per-step lattice tables and precomputes the per-step constants
 * (coupling fc(h) of Undulator::fc, src/Core/Undulator.cpp:141-167; transverse
 * focusing of TrackBeam::track, src/Core/TrackBeam.cpp:17-64; ADI coefficients of
 * FieldSolverADI::init, src/Core/FieldSolverADI.cpp:125-182). Replaces the
 * Undulator produced by Lattice::generateLattice (src/Lattice/Lattice.cpp:53-149). */
int g4gpu_set_lattice(g4gpu_handle h, int nsteps, const double *table);

/* Copies particles (host, AoS) and slice currents to the device. */
int g4gpu_load_beam(g4gpu_handle h, const double *particles, const double *current);
/* Copies the particles of the device back (host, AoS). */
int g4gpu_get_beam(g4gpu_handle h, double *particles);

/* One4one windows (&setup one4one, Beam::init with one4one, src/Core/Beam.cpp:22-40):
 * slices hold different numbers of particles, counts[nslice] in [0, npart], npart being
 * then a slice's capacity; particles [nslice][npart][6] with the first counts[is]
 * records of every slice used. g4gpu_load_beam returns the handle to full slices. */
int g4gpu_load_beam_counts(g4gpu_handle h, const double *particles, const double *current, const int *counts);
/* Particles per slice (npart in every slice unless the window is one4one). */
int g4gpu_get_counts(g4gpu_handle h, int *counts);
/* Beam::sort for one rank (src/Core/Beam.cpp:81-94, Sorting::globalSort / localSort,
 * src/Util/Sorting.cpp:55-145, 198-474): particles outside the window leave it, the
 * others move to the slice their phase lies in, the slices' currents follow their
 * counts, and the wake is formed again. *shift (may be NULL) receives the field shift
 * the reference returns, always 0 (its centre shift is off). Synchronous. A full window
 * (no counts) is left alone, as the reference skips sorting outside one4one runs.
 * G4GPU_ERR_STATE when a slice would exceed npart (the particles without room are lost).
 * Arrivals are placed behind a slice's staying particles in an order that varies from
 * run to run (atomic slot assignment), and so does which of them are lost on overflow;
 * the particles of a slice that does not overflow are the same set every run.
 * The reference sorts at marker steps between the push and the field solve
 * (Gencore.cpp:121-132): g4gpu_run(h, i, 1, G4GPU_STAGE_PUSH), g4gpu_sort, then
 * g4gpu_run(h, i, 1, G4GPU_STAGE_FIELD | G4GPU_STAGE_SLIP). */
int g4gpu_sort(g4gpu_handle h, int *shift);

/* Control::applySlippage (src/Core/Control.cpp:158-276) of field ifld by `slippage`
 * wavelengths outside the step loop, as Gencore::run does after a sort that returned a
 * shift (Gencore.cpp:125-131): the ring start moves and entering slices are cleared
 * unless the window is periodic; nothing for a steady-state run. Asynchronous. */
int g4gpu_apply_slippage(g4gpu_handle h, int ifld, double slippage);

/* ---- a window sharded over ranks -----------------------------------------------
 * The reference splits the time window into contiguous blocks of slices, one block per
 * MPI rank (Time::finishInit, src/Main/GenTime.cpp:74-77). The step's only exchange is
 * the slippage (Control::applySlippage, src/Core/Control.cpp:183-275): per slice shift
 * every rank sends the slice leaving its block to the next rank (the previous one when
 * the slippage runs backwards) and receives the entering slice from the other
 * neighbour; rank 0 (the last rank, backwards) fills it with zeros unless the window
 * is periodic, when the ring closes. A handle per rank holds its block (cfg.nslice of
 * its slices, its part of the currents and particles); its steps run with the stages
 * PUSH | FIELD, and each step's slippage of field ifld is g4gpu_slip_count, then per
 * shift g4gpu_shift_out, the caller's transfer between the ranks (NCCL, MPI, a peer
 * copy: the engine takes no part in it), g4gpu_shift_in. The transfers must be ordered
 * after g4gpu_shift_out and before g4gpu_shift_in on the handle's stream. */

/* The accumulated-slippage bookkeeping of Control::applySlippage (Control.cpp:161-186)
 * on the host, without a handle: adds `slippage` to *accuslip, takes one `sample` off
 * it per shift while |*accuslip| > 0.8 sample, and returns the number of shifts, with
 * *direction = +1 (towards the head of the window) or -1. -1 for invalid arguments. */
int g4gpu_slip_shifts(double *accuslip, double slippage, double sample, int *direction);
/* The same on field ifld of h (its accumulated slippage); *nshift = 0 for a steady-
 * state run. No device work. */
int g4gpu_slip_count(g4gpu_handle h, int ifld, double slippage, int *nshift, int *direction);
/* Bytes of one field slice on the device: ngrid^2 complex values of the handle's
 * precision (16 B plain, 8 B mixed). */
size_t g4gpu_slice_bytes(g4gpu_handle h);
/* One slice shift of field ifld, first half: copies the slice leaving the block
 * (window slice nslice - 1 for direction +1, window slice 0 for -1) to `send`
 * (g4gpu_slice_bytes of device or host memory; may be NULL) and moves the ring start
 * so that its storage slot becomes the entering slice. Asynchronous on the handle's
 * stream (synchronise before a host buffer is read). */
int g4gpu_shift_out(g4gpu_handle h, int ifld, int direction, void *send);
/* Second half: fills the entering slice from `recv` (device or host memory, as
 * `send`), or with zeros when recv is NULL. Asynchronous (a host buffer must stay
 * unchanged until the handle's stream has passed the copy). G4GPU_ERR_STATE without a
 * g4gpu_shift_out. */
int g4gpu_shift_in(g4gpu_handle h, int ifld, const void *recv);

/* Copies field ifld (host, storage order) to the device with ring start `first`
 * and accumulated slippage `accuslip` (Field::first, Field::accuslip). */
int g4gpu_load_field(g4gpu_handle h, int ifld, const double *field, int first, double accuslip);
/* Copies field ifld back (storage order) with its ring start and slippage. */
int g4gpu_get_field(g4gpu_handle h, int ifld, double *field, int *first, double *accuslip);

/* Incoherent synchrotron radiation for the following steps: &sponrad (seed, doLoss,
 * doSpread, src/Main/SponRad.cpp:19-36) with the beam's beamlet size nbins (particles
 * sharing one random draw; one4one windows draw per particle). Every undulator step then
 * adds -loss + spread (2u - 1) to gamma after the integration (Incoherent::apply,
 * src/Core/Incoherent.cpp:31-80). The loss is exact; the draws u come from a counter-based
 * generator (Philox-4x32-10 on seed, step, slice and beamlet) instead of the reference's
 * sequential ran2 stream, which it seeds per MPI rank: the same distribution, not the same
 * numbers. Each call restarts the stream; do_loss = do_spread = 0 switches it off. */
int g4gpu_set_incoherent(g4gpu_handle h, int seed, int do_loss, int do_spread, int nbins);

/* Chicanes of the lattice steps: table [nsteps][4] with the bend angle, dipole length lb,
 * dipole spacing ld and total length lt of the chicane a step covers (0 angle: none), as
 * Undulator::chic_angle, chic_lb, chic_ld, chic_lt hold them after
 * Lattice::generateLattice converted the delay to the angle (src/Lattice/Lattice.cpp:
 * 105-128); nsteps must be the lattice's. A chicane step applies the chicane's transfer
 * matrix before its first half step (TrackBeam::applyChicane, src/Core/TrackBeam.cpp:
 * 131-244) and the R56 phase shift after the integration (TrackBeam::applyR56, :260-277).
 * g4gpu_set_lattice clears them. */
int g4gpu_set_chicanes(g4gpu_handle h, int nsteps, const double *table);

/* Space charge for the following steps: the &efield namelist (src/Main/EField.cpp:19-39)
 * as Beam::initEField passes it to EFieldSolver::init (src/Core/EFieldSolver.cpp:27-48).
 * rmax: initial extent of the radial grid (it grows to 1.5 times a slice's extreme
 * radius whenever a slice exceeds it, slice after slice and step after step, as in
 * EFieldSolver::analyseBeam); ngrid: radial grid points; nz, nphi: longitudinal and
 * azimuthal modes of the short-range field (l = 1..nz, m = -nphi..nphi); longrange:
 * the long-range loss from every slice's current and size. The short-range part runs
 * when nz > 0 and ngrid > 2; all zero switches space charge off. Each call resets the
 * grid extent to rmax. Replaces EFieldSolver::longRange and shortRange
 * (EFieldSolver.cpp:56-272) in BeamSolver::advance (src/Core/BeamSolver.cpp:43-61). */
int g4gpu_set_efield(g4gpu_handle h, double rmax, int ngrid, int nz, int nphi, int longrange);

/* Wakes for the following steps: Collective::initWake (src/Core/Collective.cpp:39-107)
 * as the &wake namelist (src/Main/Wake.cpp:47-135) calls it. ns_hr fine points spaced
 * ds cover the window (nslice * sample of them, ds the reference length); ext
 * [nslice]: the external loss of every slice (eV/m, &wake loss); res, geo, rou
 * [ns_hr]: the single-particle wakes (g4gpu_host_single_wakes). ztrans, radius,
 * transient are kept as the reference keeps them; its transient cut is computed but
 * not applied, so they do not change the result. The wake of every slice
 * (Collective::update, Collective.cpp:132-187) is computed on the device from the
 * window's current, here and on every later g4gpu_load_beam, and every step adds
 * loss * dz / eev to each particle's gamma after the energy-phase integration
 * (Collective::apply, Collective.cpp:109-129). ext = NULL switches wakes off. */
int g4gpu_set_wake(g4gpu_handle h, int ns_hr, double ds, const double *ext, const double *res, const double *geo,
                   const double *rou, double ztrans, double radius, int transient);

/* Runs integration steps istep0 .. istep0+nsteps-1 of the lattice on the device,
 * each made of the stages selected by `stages` in the order of Gencore.cpp:118-147.
 * Asynchronous: returns once the work is queued on the handle's stream. */
int g4gpu_run(g4gpu_handle h, int istep0, int nsteps, int stages);

/* Waits for the handle's stream and reports any device error flag. */
int g4gpu_synchronize(g4gpu_handle h);

/* Per-slice diagnostics of the current state, reduced on the device in FP64.
 * beam_out [nslice][G4GPU_DB_NCOL + 2*nharm] (may be NULL),
 * field_out [nfield][nslice][G4GPU_DF_NCOL] indexed by window slice (may be NULL).
 * Replaces Diagnostic::calc (src/Core/Diagnostic.cpp:262-277) for these columns. */
int g4gpu_diag(g4gpu_handle h, int nharm, double *beam_out, double *field_out);

/* Far-field pointing and divergence of every slice of every field: the forward 2-D
 * FFT of the slice, its power-weighted moments on the shifted frequency map, scaled by
 * xlambda / (ngrid dgrid). out [nfield][nslice][G4GPU_DFFT_NCOL] by window slice.
 * Replaces the FFTW part of DiagField::getValues (src/Core/Diagnostic.cpp:786-847).
 * Uses the handle's scratch field array (allocated on the first call where the
 * handle has none). */
int g4gpu_diag_fft(g4gpu_handle h, double *out);

/* The handle's configuration (as created). */
int g4gpu_get_config(g4gpu_handle h, g4gpu_config *cfg);

/* ---- diagnostic plugins (DPI) --------------------------------------------------
 * Shared libraries built against the reference's plugin interface
 * (include/DiagnosticPlugin.h, DiagnosticHookS.h, data version 2023092701): field
 * plugins export factory/destroy, beam plugins factory_beamdiag/destroy_beamdiag.
 * Replaces LibraryInterface (src/Core/DiagnosticHookLI.cpp) and the feeding of
 * DiagFieldHook / DiagBeamHook (src/Core/DiagnosticHook.cpp:110-262,
 * DiagnosticHookBeam.cpp) for a single rank. */
typedef struct g4gpu_dpi_s *g4gpu_dpi;
enum { G4GPU_DPI_FIELD = 0, G4GPU_DPI_BEAM = 1 };
/* Loads the plugin, creates its object and reads its output names (get_infos with
 * `parameter`); err (errlen bytes) receives a message on failure. */
int g4gpu_dpi_open(const char *libfile, const char *parameter, int verbose, g4gpu_dpi *out, char *err,
                   int errlen);
int g4gpu_dpi_kind(g4gpu_dpi p);   /* G4GPU_DPI_FIELD or G4GPU_DPI_BEAM */
int g4gpu_dpi_nobj(g4gpu_dpi p);   /* number of output objects */
int g4gpu_dpi_multi(g4gpu_dpi p);  /* 1: a field plugin that takes all slices at once */
int g4gpu_dpi_obj_name(g4gpu_dpi p, int i, char *buf, int n);
int g4gpu_dpi_info(g4gpu_dpi p, char *buf, int n);
/* A field plugin on host data: field [nslice][ngrid^2] complex in storage order with
 * ring start `first`; out [nobj][nslice] by window slice (as the reference stores
 * /Field/<prefix>/<object>). */
int g4gpu_dpi_field(g4gpu_dpi p, int iz, int harm, int ngrid, double dgrid, double xlambda, int nslice,
                    const double *field, int first, double *out);
/* A beam plugin on host data: particles [nslice][npart][6]; out [nobj][nslice]. */
int g4gpu_dpi_beam(g4gpu_dpi p, int iz, int nslice, int npart, const double *particles, double *out);
/* The same on the handle's current state (field ifld, or the beam), copied from the device. */
int g4gpu_dpi_field_from(g4gpu_dpi p, g4gpu_handle h, int ifld, int iz, double *out);
int g4gpu_dpi_beam_from(g4gpu_dpi p, g4gpu_handle h, int iz, double *out);
void g4gpu_dpi_close(g4gpu_dpi p);

/* The window values from one state's per-slice diagnostics, on the host (no handle,
 * no device): beam_diag [nslice][G4GPU_DB_NCOL + 2*nharm] with the slices' current
 * [nslice] gives beam_global[G4GPU_DBG_NCOL] (current-weighted, as DiagBeam);
 * field_diag [nfield][nslice][G4GPU_DF_NCOL] and fft_diag
 * [nfield][nslice][G4GPU_DFFT_NCOL] (may be NULL: the far-field columns are then 0)
 * give field_global[nfield][G4GPU_DFG_NCOL] (power-weighted; the far-field moments
 * weighted by the slices' power too, which is the far field's up to the constant n^2).
 * The sums the reference forms are rebuilt from the per-slice moments, so the values
 * agree with it to rounding. Pairs of inputs and outputs may be NULL together. */
int g4gpu_diag_global(const g4gpu_config *cfg, int nharm, const double *current, const double *beam_diag,
                      const double *field_diag, const double *fft_diag, double *beam_global,
                      double *field_global);

/* Runs steps istep0 .. istep0+nsteps-1 (all stages, as g4gpu_run) and records after
 * every step the per-slice diagnostics g4gpu_diag would return at that point:
 * beam_out [nsteps][nslice][G4GPU_DB_NCOL + 2*nharm], field_out
 * [nsteps][nfield][nslice][G4GPU_DF_NCOL] (either may be NULL). Each step's record is
 * formed on the device, copied back as soon as it is complete and finished on the
 * host while the device runs the later steps; the reference keeps them in memory the
 * same way (Diagnostic::calc after every output step in Gencore::run,
 * src/Core/Gencore.cpp:102-160; written by Output::writeGroup at the end).
 * Synchronous: returns when the steps and all records are done; a device error raised
 * during any step fails the call with G4GPU_ERR_DEVICE, and beam_out and field_out
 * are then undefined (records of every step may already have been written). */
int g4gpu_run_diag(g4gpu_handle h, int istep0, int nsteps, int nharm, double *beam_out, double *field_out);

/* The CUDA stream (cudaStream_t) every kernel of h is queued on. */
int g4gpu_get_stream(g4gpu_handle h, void **stream);

/* Kernel accounting. With profiling on, every launch is bracketed by CUDA events
 * on the handle's stream; g4gpu_kernel_stats returns per kernel class
 * (G4GPU_K_*) the launch count and the summed device time in milliseconds of the
 * launches since the last reset. The launch counter runs always. */
enum { G4GPU_K_PUSH, G4GPU_K_ADI_X, G4GPU_K_ADI_Y, G4GPU_K_FFT, G4GPU_K_SLIP, G4GPU_K_DIAG,
       G4GPU_K_MISC, G4GPU_K_SC, G4GPU_K_SC_FIELD,
       G4GPU_K_STEP, /* the whole step of a slice in one kernel (launch shape field_kernel 2) */
       G4GPU_K_NCLASS };
int g4gpu_set_profiling(g4gpu_handle h, int on);
int g4gpu_kernel_stats(g4gpu_handle h, long long *launches, double *ms);
int g4gpu_reset_stats(g4gpu_handle h);

/* Bytes of device memory held by h. */
size_t g4gpu_device_bytes(g4gpu_handle h);

/* The FP64 instruction rate of a device, measured: a kernel of independent FP64
 * fused multiply-add chains (eight per thread, eight CTAs of 256 threads per SM)
 * timed by CUDA events, best of three launches after one warm-up. *instr_per_s
 * receives FP64 instructions per second (an FMA counts once; DADD and DMUL issue
 * at the same rate). This is the peak of the plain FP64 form's roofline: its push
 * and ADI sweeps are bound by the FP64 pipe. Synchronous; allocates and frees a
 * small output buffer. No reference counterpart. */
int g4gpu_measure_fp64_rate(int device, double *instr_per_s);

/* ---- CUDA graphs, launch-shape tuning, batched ensembles ------------------- */

/* With graph mode on, g4gpu_run captures each step range into one CUDA graph the
 * first time it runs from a given ring state (Field::first / accuslip) and replays
 * the graph afterwards: one launch per range instead of several per step. Results
 * are identical to direct launches. Per-kernel event timing is not collected for
 * graph launches (the launch counter is). No reference counterpart (the reference
 * has no GPU path); it serves the Gencore.cpp:102-160 loop over a lattice. */
int g4gpu_set_graph_mode(g4gpu_handle h, int on);

/* Times the candidate launch shapes of the step kernels on the handle's own data
 * (one step per candidate; beam and field are restored afterwards) and keeps the
 * fastest: threads per block of the push, threads per CTA of the fused field
 * kernel, and the fused field kernel itself (0: one CTA per slice, 1: a cluster of
 * two CTAs per slice, each holding half the rows, 2: the whole step of a slice in
 * one CTA, push, deposition and ADI, for one-field windows without space charge;
 * steps it does not apply to run kernel 0). Grids too large for one CTA (ngrid > 168)
 * run on the smallest cluster of 2 to 4 CTAs whose bands of rows fit shared memory
 * (up to ngrid 333), beyond that on the tiled two-pass ADI. Choices are cached per
 * (precision, npart, ngrid, nfield, solver) for the life of the process. Requires
 * the lattice, beam and fields to be loaded. *push_block, *field_threads and
 * *field_kernel (each may be NULL) receive the choice. No reference counterpart. */
int g4gpu_autotune(g4gpu_handle h, int *push_block, int *field_threads, int *field_kernel);
/* Sets the launch shapes g4gpu_autotune would choose: push_block a multiple of 32 in
 * [32, 512], field_threads a multiple of 32 in [2 ngrid, 1024] (mixed ADI form), and
 * field_kernel 0, 1 or 2; other values are rejected with G4GPU_ERR_ARG. The pair kernel
 * runs only where its segmented solves apply, the whole-step kernel only on one-field
 * windows without space charge; elsewhere the single-CTA field kernel does. No
 * reference counterpart. */
int g4gpu_set_launch_shapes(g4gpu_handle h, int push_block, int field_threads, int field_kernel);

/* A batch owns nrun independent handles (one time window each, with its own
 * sizes, lattice and stream), e.g. an ensemble of runs of uneven slice counts,
 * particle counts and grids. Members are loaded through g4gpu_batch_member and
 * the usual calls; g4gpu_batch_run advances every member over steps
 * istep0 .. istep0+nsteps-1 of its own lattice (clipped to its length) as one
 * captured graph per member, launched back to back so that the members run
 * concurrently on the GPU. Replaces running nrun separate reference jobs. */
typedef struct g4gpu_batch_ctx *g4gpu_batch;
int g4gpu_batch_create(int nrun, const g4gpu_config *cfgs, g4gpu_batch *out);
void g4gpu_batch_destroy(g4gpu_batch b);
g4gpu_handle g4gpu_batch_member(g4gpu_batch b, int i);
int g4gpu_batch_run(g4gpu_batch b, int istep0, int nsteps, int stages);
int g4gpu_batch_synchronize(g4gpu_batch b);

/* ---- learned coarse-step closure ----------------------------------------------
 * No reference counterpart: the reference integrates every undulator period
 * (src/Core/Gencore.cpp:102-160). A small MLP (nin -> width -> width -> width ->
 * nout, ReLU) with BF16 tensor-core forward and backward kernels (FP32 accumulate,
 * FP32 master weights, Adam) corrects coarse integration steps; the non-learned
 * fine-step solve is its fallback and its judge (g4gpu_run_learned). */
typedef struct g4gpu_mlp_ctx *g4gpu_mlp;
int g4gpu_mlp_create(int nin, int width, int nout, int seed, int device, g4gpu_mlp *out);
void g4gpu_mlp_destroy(g4gpu_mlp m);
const char *g4gpu_mlp_last_error(g4gpu_mlp m);
/* parameter vector: per layer W [n_out_padded][n_in_padded] then b [n_out_padded],
 * layer widths padded to multiples of 16 */
size_t g4gpu_mlp_num_params(g4gpu_mlp m);
int g4gpu_mlp_get_params(g4gpu_mlp m, float *out);
int g4gpu_mlp_set_params(g4gpu_mlp m, const float *in);
/* input normalisation (x - fmean) / fstd and output de-normalisation y * oscale + oshift */
int g4gpu_mlp_set_normalization(g4gpu_mlp m, const float *fmean, const float *fstd, const float *oshift,
                                const float *oscale);
int g4gpu_mlp_forward(g4gpu_mlp m, const float *X, int n, float *Y);
/* gradients of the mean squared error of the normalised outputs over n rows */
int g4gpu_mlp_gradients(g4gpu_mlp m, const float *X, const float *T, int n, float *grads, float *loss);
/* fits the normalisation to (X, T), then Adam over shuffled mini-batches */
int g4gpu_mlp_train(g4gpu_mlp m, const float *X, const float *T, int n, int epochs, int batch, float lr,
                    int seed, float *loss_per_epoch);

/* Attaches a network (32 features -> 4 corrections) to a handle: per-slice features
 * are the bunching at harmonics 1-3, mean and rms energy, the on-axis field, and
 * the projections of field 0 on 16 Gauss-Hermite modes of the given waist; the
 * corrections are a phase and an energy shift of the slice's particles and a
 * complex factor on the slice's field. u0, c0 scale the field features. */
int g4gpu_closure_attach(g4gpu_handle h, g4gpu_mlp m, double waist, double u0, double c0);
int g4gpu_closure_features(g4gpu_handle h, float *out);    /* [nslice][32] */
int g4gpu_closure_apply(g4gpu_handle h, const float *corr); /* [nslice][4] */
/* training targets [nslice][4]: the corrections turning the coarse state of hc into
 * the fine state of hf after the same interval (hc needs an attached closure) */
int g4gpu_closure_targets(g4gpu_handle hc, g4gpu_handle hf, float *out);
/* device copy of beam, fields and ring state between handles of the same shape */
int g4gpu_copy_state(g4gpu_handle dst, g4gpu_handle src);
/* Coarse pushes under a fine source and slippage, for the closure's coarse steps.
 * counts[nsteps] (nsteps the lattice's): a lattice step i with counts[i] = c > 1 is a
 * coarse step standing for c identical undulator periods of length dz/c (its dz and
 * slippage are the c periods' sums, as a coarsened lattice table gives them). It runs:
 *   1. the push of Beam::track over the whole dz (one RK4 step, BeamSolver.cpp:89-141);
 *   2. c source sub-steps: the deposition of FieldSolverADI::advance for a period
 *      (FieldSolverADI.cpp:19-51, scaled to dz/c), from every particle's phase and
 *      position interpolated linearly between the start and the end of the push at
 *      the end of period j, added to the field as the Crank-Nicolson step adds it
 *      without diffraction (twice the source), each followed by Control::applySlippage
 *      of dz/c (Control.cpp:158-276);
 *   3. one FieldSolverADI::ADI step (FieldSolverADI.cpp:60-122) over dz with no source:
 *      the diffraction of the c periods. The transverse diffraction acts alike on every
 *      slice, so it commutes with the slippage; splitting it from the sources errs by
 *      the diffraction of a source over c periods, (c dz / Rayleigh length) relative.
 * So the pusher takes coarse steps while the source and the slippage keep the period's
 * resolution: a time-dependent window sampled every wavelength keeps each slice's
 * source spread over the c slices it slips across. Mixed form, one field, ADI solver,
 * ngrid <= 168 (the fused field kernel), no space charge, full slices (npart a
 * multiple of 4, no one4one counts); other handles are rejected with G4GPU_ERR_ARG.
 * Steps with counts[i] <= 1, chicane steps and partial stages run as before. Calling
 * it again replaces the counts; g4gpu_set_lattice clears them. No reference
 * counterpart (the reference integrates every period, src/Core/Gencore.cpp:102-160). */
int g4gpu_set_field_substeps(g4gpu_handle h, int nsteps, const int *counts);
/* coarse steps istep0 .. istep0+ncoarse-1 of hc with the closure; every check_every
 * steps the fine handle hf integrates the same interval (fine steps fine_start[i],
 * fine_count[i]) from the same state; above tol relative slice-power error the fine
 * result replaces the coarse one and the next check_every-1 intervals run fine. */
int g4gpu_run_learned(g4gpu_handle hc, g4gpu_handle hf, int istep0, int ncoarse, const int *fine_start,
                      const int *fine_count, int check_every, double tol, int *nchecks, int *nfallback,
                      double *max_err);

/* ---- ADI field step without device allocation ------------------------------ */

/* No counterpart in the reference: an addition of this library for callers that
 * cannot allocate device memory. The handle API allocates its buffers with
 * cudaMalloc; a caller whose device memory all belongs to another allocator (a
 * framework's caching allocator that has reserved the device), or that cannot let
 * cudaFree synchronise the device while its own work is in flight, can use this
 * call instead. It allocates nothing: its scratch is a static device array of
 * G4GPU_NOALLOC_SCRATCH_BYTES (32 MiB) in the library's mixed-precision module,
 * which every device that loads that module holds until the process exits.
 *
 * One Crank-Nicolson ADI step (FieldSolverADI::ADI) of nslice field slices in
 * single precision, in place:
 *   field   device, [nslice][ngrid*ngrid] complex float (re, im), 8-byte aligned;
 *           storage slot (is + first) % nslice is advanced with source slice is
 *   source  device, [nslice][ngrid*ngrid] complex float in beam-slice order (the
 *           crsource term of FieldSolverADI::advance), or NULL for none; must not
 *           overlap field
 *   delz, dgrid, xks   step length, grid spacing, wavenumber (FieldSolverADI::init)
 *   device, stream     the CUDA device and a cudaStream_t on it (NULL: the default
 *                      stream); the call returns after the step has finished.
 * Limits: 3 <= ngrid <= G4GPU_NOALLOC_MAX_NGRID (a slice must fit in shared
 * memory); larger grids are rejected with G4GPU_ERR_ARG, and g4gpu_last_error(NULL)
 * gives the message. Any nslice: slices are taken in turns by at most one CTA per
 * SM, each with one scratch slot of ngrid^2 complex floats.
 * The first call on a device looks up the array's device address and sets the
 * kernel's shared-memory limit.
 * Every call on a device shares the one array, which keeps the last call's
 * contents (the call clears its error flag and rewrites its coefficients, and every
 * slot is written before it is read): calls that overlap on the GPU, from two host
 * threads or on two streams, race. */
#define G4GPU_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
#define G4GPU_NOALLOC_MAX_NGRID 168
int g4gpu_adi_advance_noalloc(float *field, const float *source, int nslice, int ngrid, int first,
                              double delz, double dgrid, double xks, int device, void *stream);

/* ---- host-side loading (bit-exact with the reference, run on the CPU) ------ */

/* Quiet loading plus shot noise of nslice consecutive slices for one rank, as
 * LoadBeam::init drives QuietLoading::loadQuiet and ShotNoise::applyShotNoise
 * (src/Loading/LoadBeam.cpp:157-212, src/Loading/QuietLoading.cpp:50-260,
 * src/Loading/ShotNoise.cpp:16-68). slicepar[nslice][17]: gamma, delgam, ex, ey,
 * betax, betay, alphax, alphay, xcen, ycen, pxcen, pycen, bunch, bunchphase, emod,
 * emodphase, current. out: particles [nslice][npart][6]. */
int g4gpu_host_load_beam(int nslice, int islice0, int npart, int nbins, int seed,
                         int shotnoise, double lambda0, double sample, const double *slicepar,
                         double *out);

/* Gauss-Hermite seed field of one slice (src/Util/GaussHermite.cpp:20-85).
 * par: lambda, power, phase, z0, w0, xcen, ycen, xangle, yangle, nx, ny, harm.
 * out: [ngrid*ngrid][2]. */
int g4gpu_host_gauss_hermite(const double *par, double gridmax, int ngrid, double *out);

/* Undulator coupling fc(h) (src/Core/Undulator.cpp:141-167). */
double g4gpu_host_fc(double aw, int helical, int h);

/* HDF5 output without the HDF5 library: the reference's .out.h5 layout (groups of FP64
 * datasets with a string attribute "unit", Output::writeGroup / writeDataset,
 * src/IO/Output.cpp:309-340, HDF5Base::writeBuffer, src/IO/HDF5base.cpp:74-128), written
 * by this project's own encoder of the HDF5 file format (version 0 superblock, version 1
 * object headers, symbol-table groups, contiguous little-endian doubles). Datasets are
 * collected in memory; g4gpu_h5_close writes the file and releases the handle. path
 * "Beam/energy": intermediate groups are created; at most 256 members per group. */
typedef struct g4gpu_h5_s *g4gpu_h5;
int g4gpu_h5_create(const char *path, g4gpu_h5 *out);
int g4gpu_h5_dataset(g4gpu_h5 f, const char *path, int rank, const long long *dims, const double *data,
                     const char *unit);
/* A 1-D dataset of 32-bit integers without attributes (HDF5Base::writeSingleNodeInt). */
int g4gpu_h5_dataset_int(g4gpu_h5 f, const char *path, int n, const int *data);
int g4gpu_h5_close(g4gpu_h5 f);

/* Single-particle longitudinal wakes on ns points spaced ds, for g4gpu_set_wake:
 * resistive wall (conductivity, relaxation c tau, round pipe of radius `radius` or
 * parallel plates of half gap `radius`), geometric (gaps of length gap every lgap) and
 * surface roughness (height hrough, period lrough); a zero conductivity, gap or hrough
 * gives zeros for that wake. Replaces Wake::singleWakeResistive, singleWakeGeometric
 * and singleWakeRoughness (src/Main/Wake.cpp:140-434) with the same numerical recipe. */
int g4gpu_host_single_wakes(int ns, double ds, double radius, double conductivity, double relaxation,
                            int roundpipe, double gap, double lgap, double hrough, double lrough, double *res,
                            double *geo, double *rou);

#ifdef __cplusplus
}
#endif
#endif
