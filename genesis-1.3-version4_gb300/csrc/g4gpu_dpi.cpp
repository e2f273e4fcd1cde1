// Diagnostic plugins (DPI) fed from the engine: the runner that GENESIS 1.3 v4's
// DiagFieldHook / DiagBeamHook provide (src/Core/DiagnosticHook.cpp,
// DiagnosticHookBeam.cpp, DiagnosticHookLI.cpp), for plugins built against the
// reference's plugin headers. A plugin is a shared library exporting
// `factory` / `destroy` (field diagnostics) or `factory_beamdiag` /
// `destroy_beamdiag` (beam diagnostics); its object reports its output names through
// get_infos and computes them per slice (or, field plugins that ask for it, for all
// slices at once) through doit.
//
// The data structures and plugin base classes (g4gpu_dpi_abi.h) repeat the
// reference's layout member for member and its virtual functions in order.
#include <dlfcn.h>

#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "g4gpu.h"
#include "g4gpu_dpi_abi.h"

struct g4gpu_dpi_s {
  void *lib = nullptr;
  int kind = -1;  // G4GPU_DPI_FIELD or G4GPU_DPI_BEAM
  g4dpi::FieldPlugin *field = nullptr;
  g4dpi::BeamPlugin *beam = nullptr;
  void (*destroy_field)(g4dpi::FieldPlugin *) = nullptr;
  void (*destroy_beam)(g4dpi::BeamPlugin *) = nullptr;
  std::vector<std::string> names;  // copies: the plugin's list may change later
  std::string info;
  bool multi = false;
  int verbose = 0;
  int runid = 0;
};

namespace {

void copy_out(const std::string &s, char *buf, int n) {
  if (!buf || n <= 0) return;
  std::strncpy(buf, s.c_str(), (size_t)n - 1);
  buf[n - 1] = 0;
}

// DiagBeamHook::getValues: slice by slice, counts (may be null: npart each) the particles
// of every slice of the [nslice][npart][6] array
void beam_slices(g4gpu_dpi p, int iz, int nslice, int npart, const double *particles, const int *counts,
                 double *out) {
  const size_t nobj = p->names.size();
  g4dpi::BeamData hd{};
  hd.version = g4dpi::kDataVersion;
  hd.verbose = p->verbose;
  hd.mpi_rank = 0;
  hd.mpi_size = 1;
  hd.runid = p->runid;
  hd.iz = iz;
  hd.ns = nslice;
  std::vector<g4dpi::Particle> slice;
  for (int is = 0; is < nslice; is++) {
    const int n = counts ? counts[is] : npart;
    slice.resize((size_t)n);
    std::memcpy(slice.data(), particles + (size_t)is * npart * 6, sizeof(g4dpi::Particle) * (size_t)n);
    std::vector<double> res(nobj, -1.);
    hd.is = is;
    hd.datain = &slice;
    hd.dataout = &res;
    p->beam->doit(&hd);
    for (size_t k = 0; k < nobj; k++) out[k * nslice + is] = res[k];
  }
}

}  // namespace

extern "C" {

int g4gpu_dpi_open(const char *libfile, const char *parameter, int verbose, g4gpu_dpi *out, char *err,
                   int errlen) {
  if (!libfile || !out) {
    copy_out("null argument", err, errlen);
    return G4GPU_ERR_ARG;
  }
  *out = nullptr;
  // DiagnosticHookLI.cpp: RTLD_NOW, so that missing symbols show at once
  void *lib = dlopen(libfile, RTLD_NOW);
  if (!lib) {
    const char *e = dlerror();
    copy_out(std::string("cannot load the plugin: ") + (e ? e : "?"), err, errlen);
    return G4GPU_ERR_ARG;
  }
  void *ff = dlsym(lib, "factory"), *fd = dlsym(lib, "destroy");
  void *bf = dlsym(lib, "factory_beamdiag"), *bd = dlsym(lib, "destroy_beamdiag");
  // exactly one kind of plugin, with both its factory and its destroyer
  const bool is_field = ff && fd, is_beam = bf && bd;
  if (is_field == is_beam) {
    dlclose(lib);
    copy_out("the library must export either factory/destroy or factory_beamdiag/destroy_beamdiag", err,
             errlen);
    return G4GPU_ERR_ARG;
  }
  auto *p = new g4gpu_dpi_s;
  p->lib = lib;
  p->verbose = verbose;
  bool ok;
  const std::vector<const char *> *names = nullptr;
  if (is_field) {
    p->kind = G4GPU_DPI_FIELD;
    p->field = reinterpret_cast<g4dpi::FieldPlugin *(*)()>(ff)();
    p->destroy_field = reinterpret_cast<void (*)(g4dpi::FieldPlugin *)>(fd);
    g4dpi::FieldInfos in{};
    in.version = g4dpi::kDataVersion;
    in.parameter = parameter ? parameter : "";
    in.mpi_rank = 0;
    in.mpi_size = 1;
    ok = p->field && p->field->get_infos(&in);
    names = in.obj_names;
    p->info = in.info_txt ? in.info_txt : "";
    p->multi = in.do_multi;
  } else {
    p->kind = G4GPU_DPI_BEAM;
    p->beam = reinterpret_cast<g4dpi::BeamPlugin *(*)()>(bf)();
    p->destroy_beam = reinterpret_cast<void (*)(g4dpi::BeamPlugin *)>(bd);
    g4dpi::BeamInfos in{};
    in.version = g4dpi::kDataVersion;
    in.parameter = parameter ? parameter : "";
    in.mpi_rank = 0;
    in.mpi_size = 1;
    ok = p->beam && p->beam->get_infos(&in);
    names = in.obj_names;
    p->info = in.info_txt ? in.info_txt : "";
    // DiagnosticHookBeam.cpp: beam plugins are fed slice by slice
    p->multi = false;
  }
  if (!ok) {
    g4gpu_dpi_close(p);
    copy_out("the plugin's get_infos failed", err, errlen);
    return G4GPU_ERR_STATE;
  }
  if (names)
    for (const char *s : *names) p->names.push_back(s ? s : "");
  *out = p;
  return G4GPU_OK;
}

int g4gpu_dpi_kind(g4gpu_dpi p) { return p ? p->kind : -1; }
int g4gpu_dpi_nobj(g4gpu_dpi p) { return p ? (int)p->names.size() : -1; }
int g4gpu_dpi_multi(g4gpu_dpi p) { return p ? (int)p->multi : -1; }

int g4gpu_dpi_obj_name(g4gpu_dpi p, int i, char *buf, int n) {
  if (!p || i < 0 || i >= (int)p->names.size()) return G4GPU_ERR_ARG;
  copy_out(p->names[i], buf, n);
  return G4GPU_OK;
}

int g4gpu_dpi_info(g4gpu_dpi p, char *buf, int n) {
  if (!p) return G4GPU_ERR_ARG;
  copy_out(p->info, buf, n);
  return G4GPU_OK;
}

int g4gpu_dpi_field(g4gpu_dpi p, int iz, int harm, int ngrid, double dgrid, double xlambda, int nslice,
                    const double *field, int first, double *out) {
  if (!p || p->kind != G4GPU_DPI_FIELD || !field || !out || nslice <= 0 || ngrid <= 0) return G4GPU_ERR_ARG;
  if (first < 0 || first >= nslice) return G4GPU_ERR_ARG;
  const size_t ncell = (size_t)ngrid * ngrid, nobj = p->names.size();
  // the slices as the plugin receives them: vectors of complex<double> in storage order
  std::vector<std::vector<std::complex<double>>> slices(nslice);
  for (int is0 = 0; is0 < nslice; is0++) {
    const std::complex<double> *s = reinterpret_cast<const std::complex<double> *>(field) + (size_t)is0 * ncell;
    slices[is0].assign(s, s + ncell);
  }
  g4dpi::FieldData hd{};
  hd.version = g4dpi::kDataVersion;
  hd.verbose = p->verbose;
  hd.mpi_rank = 0;
  hd.mpi_size = 1;
  hd.runid = p->runid;
  hd.iz = iz;
  hd.ns = nslice;
  hd.harm = harm;
  hd.ngrid = ngrid;
  hd.dgrid = dgrid;
  hd.xlambda = xlambda;
  if (p->multi) {
    // DiagFieldHook::getValues_multiworker: all slices at once, by window slice
    std::vector<const std::vector<std::complex<double>> *> in(nslice, nullptr);
    std::vector<std::vector<double>> res(nslice, std::vector<double>(nobj, -1.));
    for (int is0 = 0; is0 < nslice; is0++) in[(nslice + is0 - first) % nslice] = &slices[is0];
    hd.is = -1;
    hd.do_multi = true;
    hd.multi_datain = &in;
    hd.multi_dataout = &res;
    p->field->doit(&hd);
    for (int is = 0; is < nslice; is++)
      for (size_t k = 0; k < nobj; k++) out[k * nslice + is] = k < res[is].size() ? res[is][k] : -1.;
  } else {
    // DiagFieldHook::getValues_worker: slice by slice in storage order, stored by
    // window slice
    for (int is0 = 0; is0 < nslice; is0++) {
      std::vector<double> res(nobj, -1.);
      const int is = (nslice + is0 - first) % nslice;
      hd.is = is;
      hd.do_multi = false;
      hd.datain = &slices[is0];
      hd.dataout = &res;
      p->field->doit(&hd);
      for (size_t k = 0; k < nobj; k++) out[k * nslice + is] = res[k];
    }
  }
  return G4GPU_OK;
}

int g4gpu_dpi_beam(g4gpu_dpi p, int iz, int nslice, int npart, const double *particles, double *out) {
  if (!p || p->kind != G4GPU_DPI_BEAM || !particles || !out || nslice <= 0 || npart < 0) return G4GPU_ERR_ARG;
  beam_slices(p, iz, nslice, npart, particles, nullptr, out);
  return G4GPU_OK;
}

int g4gpu_dpi_field_from(g4gpu_dpi p, g4gpu_handle h, int ifld, int iz, double *out) {
  if (!p || !h || !out) return G4GPU_ERR_ARG;
  g4gpu_config c;
  int rc = g4gpu_get_config(h, &c);
  if (rc) return rc;
  if (ifld < 0 || ifld >= c.nfield) return G4GPU_ERR_ARG;
  std::vector<double> f(2 * (size_t)c.nslice * c.ngrid * c.ngrid);
  int first = 0;
  double acc = 0;
  if ((rc = g4gpu_get_field(h, ifld, f.data(), &first, &acc))) return rc;
  const double xlambda = c.lambda0 / (double)c.harm[ifld];
  const double dgrid = 2 * c.gridmax[ifld] / (double)(c.ngrid - 1);
  return g4gpu_dpi_field(p, iz, c.harm[ifld], c.ngrid, dgrid, xlambda, c.nslice, f.data(), first, out);
}

int g4gpu_dpi_beam_from(g4gpu_dpi p, g4gpu_handle h, int iz, double *out) {
  if (!p || !h || !out) return G4GPU_ERR_ARG;
  g4gpu_config c;
  int rc = g4gpu_get_config(h, &c);
  if (rc) return rc;
  if (p->kind != G4GPU_DPI_BEAM) return G4GPU_ERR_ARG;
  std::vector<double> part(6 * (size_t)c.nslice * c.npart);
  std::vector<int> counts(c.nslice);
  if ((rc = g4gpu_get_beam(h, part.data()))) return rc;
  if ((rc = g4gpu_get_counts(h, counts.data()))) return rc;
  beam_slices(p, iz, c.nslice, c.npart, part.data(), counts.data(), out);
  return G4GPU_OK;
}

void g4gpu_dpi_close(g4gpu_dpi p) {
  if (!p) return;
  if (p->field && p->destroy_field) p->destroy_field(p->field);
  if (p->beam && p->destroy_beam) p->destroy_beam(p->beam);
  if (p->lib) dlclose(p->lib);
  delete p;
}

}  // extern "C"
