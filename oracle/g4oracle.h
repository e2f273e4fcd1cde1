/* g4oracle — plain-C FP64 restatement of the GENESIS 1.3 v4 undulator step.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load this library, and
 * only as the checker or as the timed CPU baseline. The product (the CUDA path
 * behind include/g4gpu.h) never calls it.
 *
 * Every function restates the reference algorithm at the cited file:line in
 * GENESIS 1.3 v4.6.14 (svenreiche/Genesis-1.3-Version4). Parity is pinned against
 * the reference itself, compiled from its own sources by oracle/ref_build/ into
 * oracle/_ref/libg4ref.so, and against the fixtures in tests/golden/.
 *
 * Array conventions (shared with oracle/ref_build/g4ref_harness.cpp):
 *   particles  [ns][npart][6] doubles: gamma, theta, x, y, px, py
 *   fields     [nfld][ns][ngrid*ngrid] complex doubles (re, im), storage order;
 *              window slice j lives in storage slot (j + first) % ns
 *   lattice    [nsteps][G4_LAT_NCOL] doubles, one row per integration step
 */
#ifndef G4ORACLE_H
#define G4ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  G4_LAT_AW, G4_LAT_AX, G4_LAT_AY, G4_LAT_KU, G4_LAT_KX, G4_LAT_KY, G4_LAT_GRADX,
  G4_LAT_GRADY, G4_LAT_QF, G4_LAT_QX, G4_LAT_QY, G4_LAT_CX, G4_LAT_CY, G4_LAT_DZ,
  G4_LAT_SLIP, G4_LAT_PHASE, G4_LAT_HELICAL, G4_LAT_Z, G4_LAT_NCOL
};

/* stage bits for orc_run_steps */
#define ORC_STAGE_PUSH 1
#define ORC_STAGE_FIELD 2
#define ORC_STAGE_SLIP 4

/* Runs nsteps integration steps in place (Gencore.cpp:102-147 without markers,
 * sorting or diagnostics). solver: 0 = ADI, 1 = FFT (unfiltered), 2 = FFT with the
 * sigmoid source filter (xcut, ycut, sigmoid in filt[0..2]). accuslip[nfld] is the
 * accumulated slippage per field (Field::accuslip), carried in and out.
 * nthreads >= 1 splits every per-slice loop over that many host threads. */
int orc_run_steps(int nsteps, const double *lat, double gammaref, int ns, int npart,
                  double *particles, const double *current, double reflength,
                  double sample, int nfld, const int *harm, int ngrid,
                  const double *gridmax, double *fields, int *first, double *accuslip,
                  int time_run, int periodic, int stages, int solver, const double *filt,
                  int nthreads);

/* Random and quasi-random streams (RandomU.cpp:17-73, Hammerslay.cpp:15-49). */
void orc_ran2(int seed, int n, double *out);
void orc_hammersley(int base_index, int start, int n, double *out);
/* Inverse complementary error function (Inverfc.cpp:16-65). */
void orc_inverfc(int n, const double *in, double *out);
/* Bessel J_n (BesselJ.cpp) and undulator coupling fc(h) (Undulator.cpp:141-167). */
double orc_besselj(int n, double x);
double orc_fc(double aw, int helical, int h);

/* Quiet loading + shot noise for nslice consecutive slices of one rank
 * (LoadBeam.cpp:157-212, QuietLoading.cpp:50-260, ShotNoise.cpp:16-68).
 * slicepar[nslice][17]: gamma, delgam, ex, ey, betax, betay, alphax, alphay,
 * xcen, ycen, pxcen, pycen, bunch, bunchphase, emod, emodphase, current. */
void orc_load_beam(int nslice, int islice0, int npart, int nbins, int seed, int shotnoise,
                   double lambda, double sample, const double *slicepar, double *out);

/* Gauss-Hermite seed field of one slice (GaussHermite.cpp:20-85).
 * par: lambda, power, phase, z0, w0, xcen, ycen, xangle, yangle, nx, ny, harm */
void orc_gauss_hermite(const double *par, double gridmax, int ngrid, double *out);

/* Source term of one field per beam slice at lattice step istep
 * (FieldSolverADI.cpp:13-52): out [ns][ngrid^2][2] (re, im). */
void orc_deposit_source(const double *lat, int istep, int ns, int npart, const double *particles,
                        const double *current, double reflength, int harm, int ngrid,
                        double gridmax, double *out);
/* One ADI step of ns slices with a given source (FieldSolverADI.cpp:9-122): field
 * storage slot (ii + first) % ns takes source slice ii; source may be NULL. */
void orc_adi_advance(int ns, int ngrid, int first, double delz, double dgrid, double xks,
                     double *field, const double *source);

/* Per-slice beam diagnostics (Diagnostic.cpp:373-563) for nharm bunching
 * harmonics. out[ns][ORC_DB_NCOL + 2*nharm]: the columns below, then
 * |b_h| and arg(b_h) for h = 1..nharm. */
enum {
  ORC_DB_ENERGY, ORC_DB_ENERGYSPREAD, ORC_DB_XPOS, ORC_DB_XSIZE, ORC_DB_YPOS, ORC_DB_YSIZE,
  ORC_DB_PXPOS, ORC_DB_PYPOS, ORC_DB_EMITX, ORC_DB_EMITY, ORC_DB_BETAX, ORC_DB_BETAY,
  ORC_DB_ALPHAX, ORC_DB_ALPHAY, ORC_DB_XMIN, ORC_DB_XMAX, ORC_DB_PXMIN, ORC_DB_PXMAX,
  ORC_DB_YMIN, ORC_DB_YMAX, ORC_DB_PYMIN, ORC_DB_PYMAX, ORC_DB_EMIN, ORC_DB_EMAX,
  ORC_DB_NCOL
};
void orc_diag_beam(int ns, int npart, const double *particles, int nharm, double *out);

/* Per-slice field diagnostics (Diagnostic.cpp:718-902, without the FFTW part),
 * indexed by window slice. out[ns][ORC_DF_NCOL]. */
enum {
  ORC_DF_POWER, ORC_DF_XPOS, ORC_DF_XSIZE, ORC_DF_YPOS, ORC_DF_YSIZE, ORC_DF_NF_INT,
  ORC_DF_NF_PHI, ORC_DF_FF_INT, ORC_DF_FF_PHI, ORC_DF_NCOL
};
void orc_diag_field(int ns, int ngrid, double gridmax, double lambda0, int harm,
                    const double *field, int first, double *out);
/* Space charge (&efield, EField.cpp:19-39) for the following orc_run_steps calls:
 * radial grid extent rmax (grown as the reference does), ngrid radial points, nz
 * longitudinal and nphi azimuthal modes of the short-range field, longrange the
 * long-range loss. nz = 0 and longrange = 0 switch it off (the default). */
void orc_set_efield(double rmax, int ngrid, int nz, int nphi, int longrange);

/* One4one windows for the following orc_run_steps calls: particles per slice counts
 * [nslice] (the particle array's npart is then a slice's capacity), and a sort after the
 * push of every sort_every-th step (0: never); nslice 0 clears them. orc_get_counts
 * reads the counts back (-1 without a one4one window). */
void orc_set_counts(int nslice, const int *counts, int sort_every);
void orc_get_counts(int nslice, int *out);
/* Beam::sort for one rank (Beam.cpp:81-94, Sorting.cpp:55-145, 364-421) on particles
 * [ns][cap][6] with counts [ns]; currents [ns] follow the counts. Returns the particles
 * that found no room (0 when cap suffices). */
int orc_sort(int ns, int cap, double *particles, int *counts, double *current, double reflength, double sample);

/* Incoherent synchrotron radiation (&sponrad, Incoherent::init for rank 0,
 * Incoherent.cpp:12-27) for the following orc_run_steps calls; the random stream carries
 * over calls until the next orc_set_incoherent; nbins: beamlet size (one draw per
 * beamlet). do_loss = do_spread = 0 switches it off. */
void orc_set_incoherent(int seed, int do_loss, int do_spread, int nbins);

/* Chicanes (Undulator::chic_*) of the following orc_run_steps calls: tab [nsteps][4] =
 * angle, lb, ld, lt for each row of the lattice passed there (0 angle: none); nsteps 0
 * clears them. */
void orc_set_chicanes(int nsteps, const double *tab);

/* Wakes (&wake, Collective::initWake, Collective.cpp:39-107) for the following
 * orc_run_steps calls: external loss ext[nslice] (eV/m), single-particle wakes res, geo,
 * rou[ns_hr] on the fine grid spaced ds; on = 0 switches them off. */
void orc_set_wake(int on, int ns_hr, int nslice, double ds, const double *ext, const double *res,
                  const double *geo, const double *rou, double ztrans, double radius, int transient);
/* Window ("Global/") values from the raw sums: DiagBeam (Diagnostic.cpp:551-606),
 * out[6] = energy, energyspread, xposition, xsize, yposition, ysize; DiagField
 * (Diagnostic.cpp:902-975), out[11] = energy [J], xposition, xsize, yposition, ysize,
 * intensity-nearfield, intensity-farfield, xpointing, xdivergence, ypointing,
 * ydivergence. */
void orc_diag_global_beam(int ns, int npart, const double *particles, const double *current, double *out);
void orc_diag_global_field(int ns, int ngrid, double gridmax, double lambda0, int harm, double sample,
                           const double *field, double *out);
/* Far-field pointing and divergence (DiagField, Diagnostic.cpp:786-847, "fft"):
 * out[ns][4] = xpointing, xdivergence, ypointing, ydivergence by window slice. */
void orc_diag_field_fft(int ns, int ngrid, double gridmax, double lambda0, int harm, const double *field,
                        int first, double *out);

#ifdef __cplusplus
}
#endif
#endif
