// C entry points into the compiled GENESIS 1.3 v4 reference, used only to produce
// known-answer vectors for the tests (tests/golden/) and to validate the C
// restatement in oracle/g4oracle.c. It builds the reference's own Beam, Field,
// Undulator and Control objects from flat arrays and runs the reference's step
// sequence (Gencore.cpp:102-147): Beam::track, Field::track for every field and
// Control::applySlippage, without diagnostics or markers.
//
// Test infrastructure only; the product never links or loads it.

#include <cstring>
#include <string>
#include <vector>
#include <complex>

#include "Beam.h"
#include "Field.h"
#include "Undulator.h"
#include "Control.h"
#include "QuietLoading.h"
#include "ShotNoise.h"
#include "GaussHermite.h"
#include "Inverfc.h"
#include "RandomU.h"
#include "Hammerslay.h"
#include "BesselJ.h"
#include "Diagnostic.h"

// Electron charge as in GenMain.cpp:68 (ce), used for the electrons per slice.
static const double kCe = 4.8032045e-11;

// Column order of the per-step lattice table (one row per integration step).
enum {
  T_AW, T_AX, T_AY, T_KU, T_KX, T_KY, T_GRADX, T_GRADY, T_QF, T_QX, T_QY,
  T_CX, T_CY, T_DZ, T_SLIP, T_PHASE, T_HELICAL, T_Z, T_NCOL
};

// chicanes of the following g4ref_run_steps calls: [nsteps][4] angle, lb, ld, lt
static std::vector<double> g_chic;

// &sponrad of the following g4ref_run_steps calls (SponRad.cpp:34: Beam::initIncoherent)
// and the beamlet size the beam is set up with (Beam::init's nbins)
static int g_isr_seed = 0, g_isr_loss = 0, g_isr_spread = 0, g_isr_nbins = 1;

// one4one windows of the following g4ref_run_steps calls: particles per slice, and a
// Beam::sort after the push of every sort_every-th step (Gencore.cpp:121-132); the counts
// after the last call
static std::vector<int> g_o4o_counts, g_o4o_out;
static int g_o4o_sort_every = 0;

static void fill_undulator(Undulator *und, int nsteps, const double *tab, double gammaref) {
  auto col = [&](std::vector<double> &v, int c) {
    v.resize(nsteps);
    for (int i = 0; i < nsteps; i++) v[i] = tab[i * T_NCOL + c];
  };
  col(und->aw, T_AW); col(und->ax, T_AX); col(und->ay, T_AY); col(und->ku, T_KU);
  col(und->kx, T_KX); col(und->ky, T_KY); col(und->gradx, T_GRADX); col(und->grady, T_GRADY);
  col(und->qf, T_QF); col(und->qx, T_QX); col(und->qy, T_QY); col(und->cx, T_CX);
  col(und->cy, T_CY); col(und->dz, T_DZ); col(und->slip, T_SLIP); col(und->phaseshift, T_PHASE);
  col(und->z, T_Z);
  und->helical.resize(nsteps);
  for (int i = 0; i < nsteps; i++) und->helical[i] = tab[i * T_NCOL + T_HELICAL] != 0 ? 1 : 0;
  und->chic_angle.assign(nsteps, 0.0);
  und->chic_lb.assign(nsteps, 0.0);
  und->chic_ld.assign(nsteps, 0.0);
  und->chic_lt.assign(nsteps, 0.0);
  if (g_chic.size() == 4 * static_cast<size_t>(nsteps))
    for (int i = 0; i < nsteps; i++) {
      und->chic_angle[i] = g_chic[4 * i];
      und->chic_lb[i] = g_chic[4 * i + 1];
      und->chic_ld[i] = g_chic[4 * i + 2];
      und->chic_lt[i] = g_chic[4 * i + 3];
    }
  und->marker.assign(nsteps + 1, 0);
  und->setGammaRef(gammaref);
  und->updateMarker(0, 0, 0, 1e9);
  und->updateOutput(1);
}

// &efield parameters applied to the Beam of the following g4ref_run_steps calls
// (EField.cpp:38: Beam::initEField); nz = 0 and longrange = 0 leave space charge off.
static double g_sc_rmax = 0;
static int g_sc_ngrid = 0, g_sc_nz = 0, g_sc_nphi = 0, g_sc_longrange = 0;

// &wake of the following g4ref_run_steps calls (Wake.cpp:123: Beam::initWake): the
// external loss per slice and the single-particle wakes on the fine grid of ns_hr
// points spaced ds.
static bool g_wk_on = false;
static unsigned g_wk_ns = 0;
static double g_wk_ds = 0, g_wk_ztrans = 0, g_wk_radius = 0;
static bool g_wk_transient = false;
static std::vector<double> g_wk_ext, g_wk_res, g_wk_geo, g_wk_rou;

// field solver of the following g4ref_run_steps calls (&track fft_fieldsolver,
// source_filter, xcut, ycut, sigmoid as Track::run passes them to Field::initSolver,
// Track.cpp:88-112): 0 ADI, 1 FFT, 2 FFT with the source filter (xc, yc, sig)
static int g_solver = 0;
static double g_filt[3] = {1, 1, 1};

extern "C" {

void g4ref_set_solver(int solver, const double *filt) {
  g_solver = solver;
  for (int k = 0; k < 3; k++) g_filt[k] = filt ? filt[k] : 1.0;
}

// DiagField::getValues (Diagnostic.cpp:718-996) with every filter on (spatial,
// intensity, fft, global) on one field of ns slices in storage order with ring start
// `first`. out_slice [ns][13] by window slice: power, xposition, xsize, yposition,
// ysize, intensity-nearfield, phase-nearfield, intensity-farfield, phase-farfield,
// xpointing, xdivergence, ypointing, ydivergence. out_global [11]: energy, xposition,
// xsize, yposition, ysize, intensity-nearfield, intensity-farfield, xpointing,
// xdivergence, ypointing, ydivergence.
int g4ref_diag_field(int ns, int ngrid, double gridmax, double reflength, double sample, int harm,
                     const double *field, int first, double *out_slice, double *out_global) {
  Field f;
  f.init(ns, ngrid, gridmax, reflength, reflength * sample, 0.0, harm);
  const size_t ncell = static_cast<size_t>(ngrid) * ngrid;
  for (int is = 0; is < ns; is++)
    for (size_t c = 0; c < ncell; c++) {
      const double *v = field + (static_cast<size_t>(is) * ncell + c) * 2;
      f.field[is][c] = std::complex<double>(v[0], v[1]);
    }
  f.first = first;
  FilterDiagnostics filt;
  filt.field.global = true;
  filt.field.spatial = true;
  filt.field.fft = true;
  filt.field.intensity = true;
  DiagField diag;
  std::map<std::string, OutputInfo> tags = diag.getTags(filt);
  std::map<std::string, std::vector<double> > val;
  for (auto &t : tags) val[t.first].assign(t.second.global ? 1 : ns, 0.0);
  diag.getValues(&f, val, 0);
  static const char *slice_names[13] = {"power", "xposition", "xsize", "yposition", "ysize",
                                        "intensity-nearfield", "phase-nearfield", "intensity-farfield",
                                        "phase-farfield", "xpointing", "xdivergence", "ypointing",
                                        "ydivergence"};
  static const char *global_names[11] = {"Global/energy", "Global/xposition", "Global/xsize",
                                         "Global/yposition", "Global/ysize", "Global/intensity-nearfield",
                                         "Global/intensity-farfield", "Global/xpointing",
                                         "Global/xdivergence", "Global/ypointing", "Global/ydivergence"};
  for (int k = 0; k < 13; k++) {
    auto it = val.find(slice_names[k]);
    if (it == val.end()) return 1;
    for (int is = 0; is < ns; is++) out_slice[static_cast<size_t>(is) * 13 + k] = it->second[is];
  }
  for (int k = 0; k < 11; k++) {
    auto it = val.find(global_names[k]);
    if (it == val.end()) return 2;
    out_global[k] = it->second[0];
  }
  diag.cleanup_FFT_resources();
  return 0;
}

void g4ref_set_incoherent(int seed, int do_loss, int do_spread, int nbins) {
  g_isr_seed = seed;
  g_isr_loss = do_loss;
  g_isr_spread = do_spread;
  g_isr_nbins = nbins > 0 ? nbins : 1;
}

void g4ref_set_one4one(int nslice, const int *counts, int sort_every) {
  g_o4o_counts.assign(counts, counts + (nslice > 0 && counts ? nslice : 0));
  g_o4o_sort_every = sort_every;
}

void g4ref_get_counts(int nslice, int *out) {
  for (int i = 0; i < nslice; i++) out[i] = i < (int)g_o4o_out.size() ? g_o4o_out[i] : -1;
}

void g4ref_set_chicanes(int nsteps, const double *tab) {
  g_chic.assign(tab, tab + 4 * static_cast<size_t>(nsteps > 0 ? nsteps : 0));
}

// on = 0 switches the wake off; ext has nslice entries, res / geo / rou ns_hr
void g4ref_set_wake(int on, int ns_hr, int nslice, double ds, const double *ext, const double *res,
                    const double *geo, const double *rou, double ztrans, double radius, int transient) {
  g_wk_on = on != 0;
  if (!g_wk_on) return;
  g_wk_ns = static_cast<unsigned>(ns_hr);
  g_wk_ds = ds;
  g_wk_ext.assign(ext, ext + nslice);
  g_wk_res.assign(res, res + ns_hr);
  g_wk_geo.assign(geo, geo + ns_hr);
  g_wk_rou.assign(rou, rou + ns_hr);
  g_wk_ztrans = ztrans;
  g_wk_radius = radius;
  g_wk_transient = transient != 0;
}

void g4ref_set_efield(double rmax, int ngrid, int nz, int nphi, int longrange) {
  g_sc_rmax = rmax;
  g_sc_ngrid = ngrid;
  g_sc_nz = nz;
  g_sc_nphi = nphi;
  g_sc_longrange = longrange;
}

// Runs `nsteps` reference integration steps in place.
//   particles: [ns][npart][6] (gamma, theta, x, y, px, py)
//   fields:    [nfld][ns][ngrid*ngrid][2] in storage order; first[nfld] is the ring start
//   stages:    bit 1 beam push, bit 2 field solve, bit 4 slippage
// Returns 0 on success.
int g4ref_run_steps(int nsteps, const double *tab, double gammaref, int ns, int npart,
                    double *particles, const double *current, double reflength, double sample,
                    int nfld, const int *harm, int ngrid, const double *gridmax, double *fields,
                    int *first, int time_run, int periodic, int stages) {
  Undulator und;
  fill_undulator(&und, nsteps, tab, gammaref);

  Beam beam;
  const bool o4o = g_o4o_counts.size() == static_cast<size_t>(ns);
  const bool isr = g_isr_loss || g_isr_spread;
  beam.init(ns, isr ? g_isr_nbins : 1, reflength, reflength * sample, 0.0, o4o);
  if (o4o) beam.initSorting(0, 1, false, true);
  if (isr) beam.initIncoherent(g_isr_seed, 0, g_isr_loss != 0, g_isr_spread != 0);
  if (g_sc_nz > 0 || g_sc_longrange)
    beam.initEField(g_sc_rmax, g_sc_ngrid, g_sc_nz, g_sc_nphi, reflength, g_sc_longrange != 0);
  if (g_wk_on) {
    if (g_wk_ext.size() != static_cast<size_t>(ns)) return 2;
    beam.initWake(g_wk_ns, static_cast<unsigned>(ns), g_wk_ds, g_wk_ext.data(), g_wk_res.data(), g_wk_geo.data(),
                  g_wk_rou.data(), g_wk_ztrans, g_wk_radius, g_wk_transient);
  }
  for (int is = 0; is < ns; is++) {
    beam.current[is] = current[is];
    const int n = o4o ? g_o4o_counts[is] : npart;
    beam.beam[is].resize(n);
    for (int ip = 0; ip < n; ip++) {
      const double *p = particles + (static_cast<size_t>(is) * npart + ip) * 6;
      Particle &q = beam.beam[is][ip];
      q.gamma = p[0]; q.theta = p[1]; q.x = p[2]; q.y = p[3]; q.px = p[4]; q.py = p[5];
    }
  }

  std::vector<Field *> fld;
  size_t ncell = static_cast<size_t>(ngrid) * ngrid;
  for (int k = 0; k < nfld; k++) {
    Field *f = new Field;
    f->init(ns, ngrid, gridmax[k], reflength, reflength * sample, 0.0, harm[k]);
    f->initSolver(g_solver != 0, g_solver == 2, g_filt[0], g_filt[1], g_filt[2]);
    for (int is = 0; is < ns; is++)
      for (size_t c = 0; c < ncell; c++) {
        const double *v = fields + ((static_cast<size_t>(k) * ns + is) * ncell + c) * 2;
        f->field[is][c] = std::complex<double>(v[0], v[1]);
      }
    f->first = first[k];
    fld.push_back(f);
  }

  Control control;
  control.init(0, 1, "g4ref", &beam, &fld, &und, time_run != 0, false, periodic != 0);
  int istep = 0;
  while (und.advance(0)) {
    double delz = und.steplength();
    if (stages & 1) beam.track(delz, &fld, &und);
    if (o4o && g_o4o_sort_every > 0 && (istep + 1) % g_o4o_sort_every == 0) {
      int shift = beam.sort();
      if (shift != 0)
        for (auto *f : fld) control.applySlippage(shift, f);
    }
    istep++;
    if (stages & 2)
      for (auto *f : fld) f->track(delz, &beam, &und);
    if (stages & 4)
      for (auto *f : fld) control.applySlippage(und.slippage(), f);
  }

  g_o4o_out.assign(ns, npart);
  for (int is = 0; is < ns; is++) {
    const int n = static_cast<int>(beam.beam[is].size());
    if (n > npart) return 3;  // the window's capacity is too small for the sorted slice
    g_o4o_out[is] = n;
    for (int ip = 0; ip < n; ip++) {
      double *p = particles + (static_cast<size_t>(is) * npart + ip) * 6;
      const Particle &q = beam.beam[is][ip];
      p[0] = q.gamma; p[1] = q.theta; p[2] = q.x; p[3] = q.y; p[4] = q.px; p[5] = q.py;
    }
  }
  for (int k = 0; k < nfld; k++) {
    for (int is = 0; is < ns; is++)
      for (size_t c = 0; c < ncell; c++) {
        double *v = fields + ((static_cast<size_t>(k) * ns + is) * ncell + c) * 2;
        v[0] = fld[k]->field[is][c].real();
        v[1] = fld[k]->field[is][c].imag();
      }
    first[k] = static_cast<int>(fld[k]->first);
    delete fld[k];
  }
  return 0;
}

// Reference random streams, for known-answer vectors.
void g4ref_ran2(int seed, int n, double *out) {
  RandomU r(seed);
  for (int i = 0; i < n; i++) out[i] = r.getElement();
}
void g4ref_hammersley(int base_index, int start, int n, double *out) {
  Hammerslay h(base_index);
  h.set(start);
  for (int i = 0; i < n; i++) out[i] = h.getElement();
}
void g4ref_inverfc(int n, const double *in, double *out) {
  Inverfc e;
  for (int i = 0; i < n; i++) out[i] = e.value(in[i]);
}
double g4ref_besselj(int n, double x) {
  BesselJ b;
  return b.value(n, x);
}
// Coupling factor fc(h) of Undulator.cpp:141-167 for one step.
double g4ref_fc(double aw, int helical, int h) {
  Undulator und;
  double tab[T_NCOL] = {0};
  tab[T_AW] = aw;
  tab[T_HELICAL] = helical;
  tab[T_DZ] = 1;
  fill_undulator(&und, 1, tab, 1000.0);
  und.advance(0);
  return und.fc(h);
}

// One quiet-loaded slice (QuietLoading.cpp:50-260) plus optional shot noise
// (ShotNoise.cpp:29-68), as LoadBeam.cpp:157-200 drives them for a single rank.
// slicepar: gamma, delgam, ex, ey, betax, betay, alphax, alphay, xcen, ycen,
//           pxcen, pycen, bunch, bunchphase, emod, emodphase, current
// Slices islice0 .. islice0+nslice-1 are loaded in order with one shot-noise
// stream seeded from `seed`, exactly as a single rank does.
void g4ref_load_beam(int nslice, int islice0, int npart, int nbins, int seed, int shotnoise,
                     double lambda, double sample, const double *slicepar, double *out) {
  QuietLoading ql;
  int base[6] = {0, 1, 2, 3, 4, 5};
  ql.init(false, base);
  ShotNoise sn;
  sn.init(seed, 0);
  std::vector<Particle> buf(npart);
  for (int j = 0; j < nslice; j++) {
    const double *sp = slicepar + static_cast<size_t>(j) * 17;
    BeamSlice s;
    s.gamma = sp[0]; s.delgam = sp[1]; s.ex = sp[2]; s.ey = sp[3];
    s.betax = sp[4]; s.betay = sp[5]; s.alphax = sp[6]; s.alphay = sp[7];
    s.xcen = sp[8]; s.ycen = sp[9]; s.pxcen = sp[10]; s.pycen = sp[11];
    s.bunch = sp[12]; s.bunchphase = sp[13]; s.emod = sp[14]; s.emodphase = sp[15];
    s.current = sp[16];
    double ne = s.current * lambda * sample / kCe;
    ql.loadQuiet(buf.data(), &s, npart, nbins, 4. * asin(1.), islice0 + j);
    if (shotnoise) sn.applyShotNoise(buf.data(), npart, nbins, ne);
    for (int k = 0; k < npart; k++) {
      double *p = out + (static_cast<size_t>(j) * npart + k) * 6;
      p[0] = buf[k].gamma; p[1] = buf[k].theta; p[2] = buf[k].x;
      p[3] = buf[k].y; p[4] = buf[k].px; p[5] = buf[k].py;
    }
  }
}

// Gauss-Hermite seed field for one slice (GaussHermite.cpp:20-63).
// par: lambda, power, phase, z0, w0, xcen, ycen, xangle, yangle, nx, ny, harm
void g4ref_gauss_hermite(const double *par, double gridmax, int ngrid, double *out) {
  FieldSlice s;
  s.lambda = par[0]; s.power = par[1]; s.phase = par[2]; s.z0 = par[3]; s.w0 = par[4];
  s.xcen = par[5]; s.ycen = par[6]; s.xangle = par[7]; s.yangle = par[8];
  s.nx = static_cast<int>(par[9]); s.ny = static_cast<int>(par[10]); s.harm = static_cast<int>(par[11]);
  std::vector<std::complex<double> > f(static_cast<size_t>(ngrid) * ngrid);
  GaussHermite gh;
  gh.loadGauss(f.data(), &s, gridmax, ngrid);
  for (size_t i = 0; i < f.size(); i++) {
    out[2 * i] = f[i].real();
    out[2 * i + 1] = f[i].imag();
  }
}

}  // extern "C"
