// GencoreGPU::run — Gencore::run (src/Core/Gencore.cpp:9-195) with the integration step
// (Beam::track, Field::track, Control::applySlippage) on the GB300 engine. Everything
// around the step stays the reference's own code on the host objects: the marker
// actions (Control::applyMarker: dumps, sorting), the diagnostics (Diagnostic::calc)
// and the output file. The host Beam / Field are refreshed from the device before each
// of them, so their results are those of the reference on the engine's state.
//
// A time window split over MPI ranks keeps the reference's partition (one block of
// slices per rank); the slippage between the blocks is exchanged per slice shift as
// Control::applySlippage does (Control.cpp:183-275), staged through host memory with
// MPI_Sendrecv (the engine takes no part in the transfer: g4gpu_shift_out / _in).
#include "GencoreGPU.h"

#include <algorithm>
#include <cstring>
#include <iostream>

extern bool MPISingle;

// the engine's host particle record is the reference's Particle
static_assert(sizeof(Particle) == 6 * sizeof(double), "Particle is {gamma, theta, x, y, px, py}");

void GencoreGPU::setEField(double rmax, int ngrid, int nz, int nphi, bool longrange) {
  efield_ = nz > 0 || longrange;
  ef_rmax_ = rmax;
  ef_ngrid_ = ngrid;
  ef_nz_ = nz;
  ef_nphi_ = nphi;
  ef_lr_ = longrange;
}

void GencoreGPU::setIncoherent(int seed, bool loss, bool spread, int nbins) {
  isr_ = loss || spread;
  isr_seed_ = seed;
  isr_loss_ = loss;
  isr_spread_ = spread;
  isr_nbins_ = nbins > 0 ? nbins : 1;
}

void GencoreGPU::setWake(unsigned int ns, double ds, const double *ext, int nslice, const double *res,
                         const double *geo, const double *rou, double ztrans, double radius, bool transient) {
  wake_ = ext != nullptr;
  wk_ns_ = ns;
  wk_ds_ = ds;
  wk_ext_.assign(ext, ext + (ext ? nslice : 0));
  wk_res_.assign(res, res + ns);
  wk_geo_.assign(geo, geo + ns);
  wk_rou_.assign(rou, rou + ns);
  wk_ztrans_ = ztrans;
  wk_radius_ = radius;
  wk_transient_ = transient;
}

namespace {

// The per-step vectors of the Undulator (include/Undulator.h:58-62) as the engine's
// lattice table, one row per integration step.
std::vector<double> lattice_table(Undulator *und) {
  const size_t n = und->aw.size();
  std::vector<double> t(n * G4GPU_LAT_NCOL);
  for (size_t i = 0; i < n; i++) {
    double *r = &t[i * G4GPU_LAT_NCOL];
    r[G4GPU_LAT_AW] = und->aw[i];
    r[G4GPU_LAT_AX] = und->ax[i];
    r[G4GPU_LAT_AY] = und->ay[i];
    r[G4GPU_LAT_KU] = und->ku[i];
    r[G4GPU_LAT_KX] = und->kx[i];
    r[G4GPU_LAT_KY] = und->ky[i];
    r[G4GPU_LAT_GRADX] = und->gradx[i];
    r[G4GPU_LAT_GRADY] = und->grady[i];
    r[G4GPU_LAT_QF] = und->qf[i];
    r[G4GPU_LAT_QX] = und->qx[i];
    r[G4GPU_LAT_QY] = und->qy[i];
    r[G4GPU_LAT_CX] = und->cx[i];
    r[G4GPU_LAT_CY] = und->cy[i];
    r[G4GPU_LAT_DZ] = und->dz[i];
    r[G4GPU_LAT_SLIP] = und->slip[i];
    r[G4GPU_LAT_PHASE] = und->phaseshift[i];
    r[G4GPU_LAT_HELICAL] = und->helical[i];
    r[G4GPU_LAT_Z] = und->z[i];
  }
  return t;
}

// The chicanes of the steps (Undulator::chic_*, set by Lattice::generateLattice), or
// an empty table when the lattice has none.
std::vector<double> chicane_table(Undulator *und) {
  const size_t n = und->aw.size();
  std::vector<double> t;
  bool any = false;
  for (size_t i = 0; i < n && i < und->chic_angle.size(); i++) any = any || und->chic_angle[i] != 0;
  if (!any) return t;
  t.resize(4 * n);
  for (size_t i = 0; i < n; i++) {
    t[4 * i] = und->chic_angle[i];
    t[4 * i + 1] = und->chic_lb[i];
    t[4 * i + 2] = und->chic_ld[i];
    t[4 * i + 3] = und->chic_lt[i];
  }
  return t;
}

// Particle records are {gamma, theta, x, y, px, py} (include/Particle.h:6-13), the
// engine's host layout: the slices are packed into one array of capacity npart each.
void pack_beam(Beam *beam, int npart, std::vector<double> &parts, std::vector<int> &counts) {
  const int ns = (int)beam->beam.size();
  parts.assign(6 * (size_t)ns * npart, 0.0);
  counts.resize(ns);
  for (int is = 0; is < ns; is++) {
    counts[is] = (int)beam->beam[is].size();
    std::memcpy(&parts[6 * (size_t)is * npart], beam->beam[is].data(), sizeof(Particle) * counts[is]);
  }
}

void unpack_beam(Beam *beam, int npart, const std::vector<double> &parts, const std::vector<int> &counts) {
  for (size_t is = 0; is < beam->beam.size(); is++) {
    beam->beam[is].resize(counts[is]);
    std::memcpy(beam->beam[is].data(), &parts[6 * is * npart], sizeof(Particle) * counts[is]);
  }
}

}  // namespace

bool GencoreGPU::run(Beam *beam, std::vector<Field *> *field, Setup *setup, Undulator *und, bool isTime,
                     bool isScan, bool periodic, FilterDiagnostics &filter, bool *stepped) {
  if (stepped) *stepped = false;
  int size = 1, rank = 0;
  if (!MPISingle) {
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
  }
  const int ns = (int)beam->beam.size();
  const int nfld = (int)field->size();
  if (ns < 1 || nfld < 1 || nfld > G4GPU_MAX_FIELDS) {
    error_ = "no slices or an unsupported number of fields";
    return false;
  }
  // the beam's slices: uniform, or one4one with a capacity of the largest slice
  int npart = 0;
  bool uniform = true;
  for (auto &s : beam->beam) {
    if ((int)s.size() != (int)beam->beam[0].size()) uniform = false;
    npart = std::max(npart, (int)s.size());
  }
  const int ngrid = field->at(0)->ngrid;
  for (auto *f : *field)
    if (f->ngrid != ngrid) {
      error_ = "the engine holds fields of one grid size";
      return false;
    }

  g4gpu_config cfg;
  g4gpu_config_defaults(&cfg);
  cfg.nslice = ns;
  cfg.npart = npart;
  cfg.ngrid = ngrid;
  cfg.nfield = nfld;
  for (int k = 0; k < nfld; k++) {
    cfg.harm[k] = field->at(k)->getHarm();
    cfg.gridmax[k] = field->at(k)->gridmax;
  }
  cfg.lambda0 = beam->reflength;
  cfg.sample = beam->slicelength / beam->reflength;
  cfg.gammaref = und->getGammaRef();
  cfg.precision = precision_;
  cfg.time_run = isTime;
  cfg.periodic = periodic;
  cfg.device = device_;
  g4gpu_handle h = nullptr;
  if (g4gpu_create(&cfg, &h)) {
    error_ = g4gpu_last_error(nullptr);
    return false;  // nothing ran: the caller runs Gencore::run
  }
  struct Release {
    g4gpu_handle h;
    ~Release() { g4gpu_destroy(h); }
  } release{h};
  auto fail = [&]() {
    error_ = g4gpu_last_error(h);
    return false;
  };

  std::vector<double> tab = lattice_table(und);
  if (g4gpu_set_lattice(h, (int)und->aw.size(), tab.data())) return fail();
  std::vector<double> chic = chicane_table(und);
  if (!chic.empty() && g4gpu_set_chicanes(h, (int)und->aw.size(), chic.data())) return fail();
  std::vector<double> parts;
  std::vector<int> counts;
  pack_beam(beam, npart, parts, counts);
  if (uniform ? g4gpu_load_beam(h, parts.data(), beam->current.data())
              : g4gpu_load_beam_counts(h, parts.data(), beam->current.data(), counts.data()))
    return fail();
  const size_t ncell = (size_t)ngrid * ngrid;
  std::vector<double> fbuf(2 * (size_t)ns * ncell);
  for (int k = 0; k < nfld; k++) {
    Field *f = field->at(k);
    for (int is = 0; is < ns; is++) std::memcpy(&fbuf[2 * is * ncell], f->field[is].data(), 16 * ncell);
    if (g4gpu_load_field(h, k, fbuf.data(), f->first, f->accuslip)) return fail();
  }
  if (efield_ && g4gpu_set_efield(h, ef_rmax_, ef_ngrid_, ef_nz_, ef_nphi_, ef_lr_)) return fail();
  if (isr_ && g4gpu_set_incoherent(h, isr_seed_, isr_loss_, isr_spread_, isr_nbins_)) return fail();
  if (wake_ && g4gpu_set_wake(h, (int)wk_ns_, wk_ds_, wk_ext_.data(), wk_res_.data(), wk_geo_.data(),
                              wk_rou_.data(), wk_ztrans_, wk_radius_, wk_transient_))
    return fail();

  // the host objects from the device state, before the reference's code reads them
  auto to_host = [&]() -> bool {
    if (g4gpu_get_beam(h, parts.data()) || g4gpu_get_counts(h, counts.data())) return false;
    unpack_beam(beam, npart, parts, counts);
    for (int k = 0; k < nfld; k++) {
      Field *f = field->at(k);
      int first;
      double acc;
      if (g4gpu_get_field(h, k, fbuf.data(), &first, &acc)) return false;
      // std::complex<double> is laid out as double[2]
      for (int is = 0; is < ns; is++)
        std::memcpy(static_cast<void *>(f->field[is].data()), &fbuf[2 * is * ncell], 16 * ncell);
      f->first = first;
      f->accuslip = acc;
    }
    return true;
  };

  std::string rn, fnbase;
  setup->getRootName(&rn);
  setup->RootName_to_FileName(&fnbase, &rn);
  Control *control = new Control;
  struct Del {
    Control *c;
    ~Del() { delete c; }
  } del{control};
  control->init(rank, size, fnbase, beam, field, und, isTime, isScan, periodic);
  Diagnostic diag;
  diag.init(rank, size, und->outlength(), ns, nfld, isTime, isScan, filter);
  diag.calc(beam, field, und->getz());

  // slippage across ranks: per shift the leaving slice goes to the next rank and the
  // entering one comes from the previous (Control.cpp:183-275), through host buffers
  // (a CUDA-aware MPI could take device buffers instead)
  const size_t sbytes = g4gpu_slice_bytes(h);
  std::vector<unsigned char> hsend(size > 1 ? sbytes : 0), hrecv(size > 1 ? sbytes : 0);
  auto exchange = [&](int k, double slippage) -> bool {
    int nshift = 0, dir = 1;
    if (g4gpu_slip_count(h, k, slippage, &nshift, &dir)) return false;
    for (int i = 0; i < nshift; i++) {
      int next = (rank + 1) % size, prev = (rank + size - 1) % size;
      if (dir < 0) std::swap(next, prev);
      const bool head = rank == (dir > 0 ? size - 1 : 0), tail = rank == (dir > 0 ? 0 : size - 1);
      const bool snd = periodic || !head, rcv = periodic || !tail;
      if (g4gpu_shift_out(h, k, dir, snd ? hsend.data() : nullptr) || g4gpu_synchronize(h)) return false;
      MPI_Sendrecv(hsend.data(), snd ? (int)sbytes : 0, MPI_CHAR, snd ? next : MPI_PROC_NULL, 1, hrecv.data(),
                   rcv ? (int)sbytes : 0, MPI_CHAR, rcv ? prev : MPI_PROC_NULL, 1, MPI_COMM_WORLD,
                   MPI_STATUS_IGNORE);
      if (g4gpu_shift_in(h, k, rcv ? hrecv.data() : nullptr) || g4gpu_synchronize(h)) return false;
    }
    return true;
  };
  auto sort_and_shift = [&]() -> bool {
    int shift = 0;
    if (g4gpu_sort(h, &shift)) return false;
    for (int k = 0; k < nfld && shift != 0; k++)
      if (g4gpu_apply_slippage(h, k, shift)) return false;
    return true;
  };

  while (und->advance(rank)) {
    const int istep = und->getStep();
    // step 1: marker actions on the host objects (dumps; the sort request)
    bool sort = false;
    if (und->getMarker() != 0) {
      if (!to_host()) return fail();
      bool error_IO = false;
      sort = control->applyMarker(beam, field, und, error_IO);
      if (error_IO) return false;
    }
    if (stepped) *stepped = true;
    // step 2: Beam::track
    if (g4gpu_run(h, istep, 1, G4GPU_STAGE_PUSH)) return fail();
    // step 3: Beam::sort (one4one windows)
    if (sort && !sort_and_shift()) return fail();
    // step 4: Field::track of every field
    if (g4gpu_run(h, istep, 1, G4GPU_STAGE_FIELD)) return fail();
    // step 5: Control::applySlippage of every field
    if (size == 1) {
      if (g4gpu_run(h, istep, 1, G4GPU_STAGE_SLIP)) return fail();
    } else if (isTime) {
      for (int k = 0; k < nfld; k++)
        if (!exchange(k, und->slippage())) return fail();
    }
    // step 6: diagnostics of an output step, on the host objects
    if (und->outstep()) {
      if (!to_host()) return fail();
      diag.calc(beam, field, und->getz());
    }
  }
  if (g4gpu_synchronize(h) || !to_host()) return fail();

  // the last marker action and the output file, as Gencore.cpp:162-190
  bool error_IO = false;
  const bool sort = control->applyMarker(beam, field, und, error_IO);
  if (error_IO) return false;
  if (sort) {
    const int shift = beam->sort();
    if (shift != 0)
      for (auto *f : *field) control->applySlippage(shift, f);
  }
  if (rank == 0) std::cout << "Writing output file..." << std::endl;
  if (!diag.writeToOutputFile(beam, field, setup, und)) return false;
  if (rank == 0) std::cout << std::endl << "Core Simulation done." << std::endl;
  return true;
}
