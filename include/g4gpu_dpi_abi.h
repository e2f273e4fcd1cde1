/* Binary interface of diagnostic plugins (DPI) as GENESIS 1.3 v4 defines it
 * (include/DiagnosticHookS.h, DiagnosticPlugin.h, DiagnosticHook_V.h,
 * Particle.h of the reference): the data exchanged with a plugin and the plugin base
 * classes, repeated member for member and with the virtual functions in the same
 * order, so that plugins built against either declaration load in the other's
 * runner. A field plugin exports
 *   extern "C" g4dpi::FieldPlugin *factory(void);  extern "C" void destroy(g4dpi::FieldPlugin *);
 * a beam plugin
 *   extern "C" g4dpi::BeamPlugin *factory_beamdiag(void);  extern "C" void destroy_beamdiag(g4dpi::BeamPlugin *);
 * C++ only. */
#ifndef G4GPU_DPI_ABI_H
#define G4GPU_DPI_ABI_H

#include <complex>
#include <string>
#include <vector>

namespace g4dpi {

struct Particle {
  double gamma, theta, x, y, px, py;
};

constexpr int kDataVersion = 2023092701;

class CommonInfos {
 public:
  int version;
  const char *info_txt;
  const std::vector<const char *> *obj_names;
  std::string parameter;
  bool do_multi{false};
  int mpi_rank, mpi_size;
};
class BeamInfos : public CommonInfos {};
class FieldInfos : public CommonInfos {};

class BeamData {
 public:
  int version;
  int mpi_rank, mpi_size;
  int runid;
  int iz;
  int is, ns;
  bool do_multi{false};
  const std::vector<Particle> *datain{nullptr};
  std::vector<double> *dataout{nullptr};
  std::vector<const std::vector<Particle> *> *multi_datain{nullptr};
  std::vector<std::vector<double>> *multi_dataout{nullptr};
  int verbose;
};

class FieldData {
 public:
  int version;
  int mpi_rank, mpi_size;
  int runid;
  int iz;
  int is, ns;
  int harm;
  int ngrid;
  double dgrid;
  double xlambda;
  bool do_multi{false};
  const std::vector<std::complex<double>> *datain{nullptr};
  std::vector<double> *dataout{nullptr};
  std::vector<const std::vector<std::complex<double>> *> *multi_datain{nullptr};
  std::vector<std::vector<double>> *multi_dataout{nullptr};
  int verbose;
};

class BeamPlugin {
 public:
  virtual ~BeamPlugin() {}
  virtual bool get_infos(BeamInfos *) = 0;
  virtual void doit(BeamData *) = 0;
};
class FieldPlugin {
 public:
  virtual ~FieldPlugin() {}
  virtual bool get_infos(FieldInfos *) = 0;
  virtual void doit(FieldData *) = 0;
};

}  // namespace g4dpi

#endif /* G4GPU_DPI_ABI_H */
