// Diagnostic plugins for the tests of the engine's plugin runner, built against
// include/g4gpu_dpi_abi.h (the layout of the reference's plugin interface).
//   field plugin: per slice the sum of |u|^2 over the grid, the window slice index it
//                 was given and iz; with -DG4_TEST_MULTI it asks for all slices at once
//   -DG4_TEST_BEAM: beam plugin, per slice <gamma> and the slice index
#include <vector>

#include "g4gpu_dpi_abi.h"

namespace {
std::vector<const char *> kNames = {"sum_abs2", "slice", "iz"};
std::vector<const char *> kBeamNames = {"mean_gamma", "slice"};

double sum_abs2(const std::vector<std::complex<double>> &s) {
  double r = 0;
  for (const auto &v : s) r += std::norm(v);
  return r;
}
}  // namespace

#ifndef G4_TEST_BEAM
class TestField : public g4dpi::FieldPlugin {
 public:
  bool get_infos(g4dpi::FieldInfos *pi) override {
    pi->obj_names = &kNames;
    pi->info_txt = "test field plugin";
#ifdef G4_TEST_MULTI
    pi->do_multi = true;
#endif
    return pi->version == g4dpi::kDataVersion;
  }
  void doit(g4dpi::FieldData *pd) override {
    if (pd->version != g4dpi::kDataVersion) return;
    if (pd->do_multi) {
      for (int is = 0; is < pd->ns; is++) {
        auto &o = pd->multi_dataout->at(is);
        o.at(0) = sum_abs2(*pd->multi_datain->at(is));
        o.at(1) = is;
        o.at(2) = pd->iz;
      }
    } else {
      pd->dataout->at(0) = sum_abs2(*pd->datain);
      pd->dataout->at(1) = pd->is;
      pd->dataout->at(2) = pd->iz;
    }
  }
};
extern "C" g4dpi::FieldPlugin *factory(void) { return new TestField; }
extern "C" void destroy(g4dpi::FieldPlugin *p) { delete p; }
#else
class TestBeam : public g4dpi::BeamPlugin {
 public:
  bool get_infos(g4dpi::BeamInfos *pi) override {
    pi->obj_names = &kBeamNames;
    pi->info_txt = "test beam plugin";
    return pi->version == g4dpi::kDataVersion;
  }
  void doit(g4dpi::BeamData *pd) override {
    double g = 0;
    for (const auto &p : *pd->datain) g += p.gamma;
    pd->dataout->at(0) = pd->datain->empty() ? 0. : g / pd->datain->size();
    pd->dataout->at(1) = pd->is;
  }
};
extern "C" g4dpi::BeamPlugin *factory_beamdiag(void) { return new TestBeam; }
extern "C" void destroy_beamdiag(g4dpi::BeamPlugin *p) { delete p; }
#endif
