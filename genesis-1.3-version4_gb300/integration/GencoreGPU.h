// GencoreGPU — the reference's integration loop (Gencore::run, src/Core/Gencore.cpp:9-195)
// with the integration step on the GB300 engine (include/g4gpu.h). Compiled inside the
// reference's source tree (its headers: Beam.h, Field.h, Undulator.h, Control.h,
// Diagnostic.h, Setup.h); Track::run (src/Main/Track.cpp:170-171) calls
// GencoreGPU::run in place of Gencore::run when a GPU is wanted, and falls back to
// Gencore::run when it returns false before any step ran (no device, a feature the
// engine does not cover).
//
// The namelists that give the step more physics than the beam and field objects carry
// (&efield, &sponrad, &wake) keep their parameters in private members of the
// reference's classes; the caller that parsed them passes them here (set* below)
// before run, as EField.cpp, SponRad.cpp and Wake.cpp pass them to Beam::init*.
#ifndef GENCORE_GPU_H
#define GENCORE_GPU_H

#include <string>
#include <vector>

#include "Gencore.h"
#include "g4gpu.h"

class GencoreGPU {
 public:
  // G4GPU_PLAIN (the reference's FP64 arithmetic) or G4GPU_MIXED; CUDA device
  explicit GencoreGPU(int precision = G4GPU_PLAIN, int device = 0) : precision_(precision), device_(device) {}
  // &efield as Beam::initEField receives it (EField.cpp:38)
  void setEField(double rmax, int ngrid, int nz, int nphi, bool longrange);
  // &sponrad as Beam::initIncoherent receives it (SponRad.cpp:34), with the beamlet size
  void setIncoherent(int seed, bool loss, bool spread, int nbins);
  // &wake as Beam::initWake receives it (Wake.cpp:123): ns fine points spaced ds, the
  // external loss per slice and the three single-particle wakes
  void setWake(unsigned int ns, double ds, const double *ext, int nslice, const double *res, const double *geo,
               const double *rou, double ztrans, double radius, bool transient);
  // Gencore::run's signature and result. *stepped (may be null) tells the caller
  // whether any step ran on the GPU: false with a false result means "use Gencore::run".
  bool run(Beam *beam, std::vector<Field *> *field, Setup *setup, Undulator *und, bool isTime, bool isScan,
           bool periodic, FilterDiagnostics &filter, bool *stepped = nullptr);
  // the engine's message of the last failure
  const std::string &error() const { return error_; }

 private:
  int precision_, device_;
  bool efield_ = false, isr_ = false, wake_ = false;
  double ef_rmax_ = 0;
  int ef_ngrid_ = 0, ef_nz_ = 0, ef_nphi_ = 0;
  bool ef_lr_ = false;
  int isr_seed_ = 0, isr_nbins_ = 1;
  bool isr_loss_ = false, isr_spread_ = false;
  unsigned int wk_ns_ = 0;
  double wk_ds_ = 0, wk_ztrans_ = 0, wk_radius_ = 0;
  bool wk_transient_ = false;
  std::vector<double> wk_ext_, wk_res_, wk_geo_, wk_rou_;
  std::string error_;
};

#endif
