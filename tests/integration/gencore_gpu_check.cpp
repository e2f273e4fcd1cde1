// Builds a small time-dependent deck with the reference's own objects (Undulator,
// Beam, Field, Setup) and runs it twice: through the reference's Gencore::run on the
// CPU, and through GencoreGPU::run (genesis-1.3-version4_gb300/integration) on the
// engine. Prints one line:
//   FALLBACK <message>   GencoreGPU::run found no usable device and ran no step (the
//                        caller then keeps Gencore::run), exit 0
//   MATCH <field> <particles>  both ran; the largest relative differences of the
//                        final field and particles, exit 0 if below 1e-9
//   MISMATCH ...         exit 1
// Test infrastructure: compiled against the reference's headers and objects by
// oracle/ref_build/Makefile, run by tests/test_integration_build.py.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdint>
#include <vector>

#include "GencoreGPU.h"

extern bool MPISingle;

namespace {

const int kNs = 4, kNpart = 64, kNgrid = 21, kSteps = 12;
const double kLambda = 1e-10, kGamma = 11357.8, kGridmax = 6e-5;

void make_undulator(Undulator *und) {
  const double ku = 2 * M_PI / 0.015, aw = 1.7;
  const int n = kSteps;
  auto fill = [&](std::vector<double> &v, double x) { v.assign(n, x); };
  fill(und->aw, aw);
  fill(und->ax, 0);
  fill(und->ay, 0);
  fill(und->ku, ku);
  fill(und->kx, 0);
  fill(und->ky, ku * ku);
  fill(und->gradx, 0);
  fill(und->grady, 0);
  fill(und->qf, 0);
  fill(und->qx, 0);
  fill(und->qy, 0);
  fill(und->cx, 0);
  fill(und->cy, 0);
  fill(und->dz, 0.015);
  fill(und->slip, 0.015 / (2 * kGamma * kGamma * kLambda / (1 + aw * aw)));
  fill(und->phaseshift, 0);
  und->z.resize(n);
  for (int i = 0; i < n; i++) und->z[i] = 0.015 * i;
  und->helical.assign(n, 0);
  und->chic_angle.assign(n, 0);
  und->chic_lb.assign(n, 0);
  und->chic_ld.assign(n, 0);
  und->chic_lt.assign(n, 0);
  und->marker.assign(n + 1, 0);
  und->setGammaRef(kGamma);
  und->updateMarker(0, 0, 0, 1e9);
  und->updateOutput(1);
}

// a deterministic beam: Gaussian-ish offsets from a 64-bit linear congruential stream
void make_beam(Beam *beam) {
  beam->init(kNs, 4, kLambda, kLambda, 0.0, false);
  uint64_t s = 12345;
  auto u = [&]() {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int is = 0; is < kNs; is++) {
    beam->current[is] = 3000.0;
    beam->beam[is].resize(kNpart);
    for (int ip = 0; ip < kNpart; ip++) {
      Particle &p = beam->beam[is][ip];
      p.gamma = kGamma + 2.0 * (u() - 0.5);
      p.theta = 2 * M_PI * u();
      p.x = 2e-5 * (u() - 0.5);
      p.y = 2e-5 * (u() - 0.5);
      p.px = 0.02 * (u() - 0.5);
      p.py = 0.02 * (u() - 0.5);
    }
  }
}

Field *make_field() {
  Field *f = new Field;
  f->init(kNs, kNgrid, kGridmax, kLambda, kLambda, 0.0, 1);
  f->initSolver(false, false, 1, 1, 1);
  const double dg = 2 * kGridmax / (kNgrid - 1);
  for (int is = 0; is < kNs; is++)
    for (int iy = 0; iy < kNgrid; iy++)
      for (int ix = 0; ix < kNgrid; ix++) {
        const double x = -kGridmax + ix * dg, y = -kGridmax + iy * dg;
        f->field[is][iy * kNgrid + ix] = std::complex<double>(1e6 * exp(-(x * x + y * y) / 4e-10), 1e5 * is);
      }
  return f;
}

}  // namespace

int main() {
  MPISingle = true;
  FilterDiagnostics filter;
  Setup setup;
  Undulator ua, ub;
  make_undulator(&ua);
  make_undulator(&ub);
  Beam ba, bb;
  make_beam(&ba);
  make_beam(&bb);
  std::vector<Field *> fa{make_field()}, fb{make_field()};

  GencoreGPU gpu(G4GPU_PLAIN, 0);
  bool stepped = false;
  const bool ok = gpu.run(&bb, &fb, &setup, &ub, true, false, false, filter, &stepped);
  if (!ok && !stepped) {
    std::printf("FALLBACK %s\n", gpu.error().c_str());
    return 0;
  }
  if (!ok) {
    std::printf("MISMATCH GencoreGPU::run failed after stepping: %s\n", gpu.error().c_str());
    return 1;
  }
  Gencore core;
  if (!core.run(&ba, &fa, &setup, &ua, true, false, false, filter)) {
    std::printf("MISMATCH Gencore::run failed\n");
    return 1;
  }
  double ef = 0, fmax = 0, ep = 0;
  for (int is = 0; is < kNs; is++) {
    const int ia = (is + fa[0]->first) % kNs, ib = (is + fb[0]->first) % kNs;
    for (int c = 0; c < kNgrid * kNgrid; c++) {
      ef = std::fmax(ef, std::abs(fa[0]->field[ia][c] - fb[0]->field[ib][c]));
      fmax = std::fmax(fmax, std::abs(fa[0]->field[ia][c]));
    }
    for (int ip = 0; ip < kNpart; ip++) {
      const double *a = &ba.beam[is][ip].gamma, *b = &bb.beam[is][ip].gamma;
      for (int k = 0; k < 6; k++) ep = std::fmax(ep, std::fabs(a[k] - b[k]) / std::fmax(std::fabs(a[k]), 1e-30));
    }
  }
  ef /= fmax;
  const bool match = ef < 1e-9 && ep < 1e-9;
  std::printf("%s %.3e %.3e\n", match ? "MATCH" : "MISMATCH", ef, ep);
  return match ? 0 : 1;
}
