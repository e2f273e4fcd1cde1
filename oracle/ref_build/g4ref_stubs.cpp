// Link-time stand-ins for the GENESIS 1.3 v4 reference's HDF5 I/O classes, written
// for this project so that the reference's own physics sources (everything under
// src/ except src/IO/, the diagnostic-plugin loader and the unused FieldSolver.cpp)
// link into a single-rank CPU checker without libhdf5.
//
// Instead of HDF5 they write a small raw binary so that the checker's results can
// be read from Python:
//   <root>.out.h5.raw  diagnostics buffers written by Output::writeGroup
//   <root>.fld.h5.raw  field dump written by WriteFieldHDF5::write
//   <root>.par.h5.raw  particle dump written by WriteBeamHDF5::write
// Every record is: u32 len, group name; u32 len, dataset name; u8 single flag;
// u64 count; count little-endian doubles. The file starts with "G4RAW1\0\0".
//
// This is test infrastructure only; it contains no reference code.

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <map>
#include <complex>

#include "HDF5base.h"
#include "Output.h"
#include "readBeamHDF5.h"
#include "readFieldHDF5.h"
#include "readMapHDF5.h"
#include "writeBeamHDF5.h"
#include "writeFieldHDF5.h"
#include "writeWakeHDF5.h"
#include "SDDSBeam.h"
#include "Beam.h"
#include "Field.h"

namespace {

struct RawFile {
  FILE *f = nullptr;
  bool open(const std::string &fn) {
    f = std::fopen(fn.c_str(), "wb");
    if (!f) return false;
    std::fwrite("G4RAW1\0\0", 1, 8, f);
    return true;
  }
  void str(const std::string &s) {
    uint32_t n = static_cast<uint32_t>(s.size());
    std::fwrite(&n, 4, 1, f);
    std::fwrite(s.data(), 1, n, f);
  }
  void rec(const std::string &group, const std::string &name, bool single, const double *d, uint64_t n) {
    str(group);
    str(name);
    uint8_t s = single ? 1 : 0;
    std::fwrite(&s, 1, 1, f);
    std::fwrite(&n, 8, 1, f);
    if (n) std::fwrite(d, 8, n, f);
  }
  void close() {
    if (f) std::fclose(f);
    f = nullptr;
  }
};

RawFile g_out;

}  // namespace

HDF5Base::HDF5Base() : isOpen(false), nwork(0), work(nullptr), s0(0), ds(0) {}
HDF5Base::~HDF5Base() {}
bool HDF5Base::simpleReadDouble1D(const string &, vector<double> *) { return false; }
bool HDF5Base::browseFile(const string &, vector<string> *) { return false; }

Output::Output() : noOutput(false), fid(0) {}
Output::~Output() { g_out.close(); }
bool Output::open(string file, int, int) { return g_out.open(file + ".raw"); }
void Output::close() { g_out.close(); }
void Output::writeMeta(Undulator *) {}
void Output::writeGroup(std::string group, std::map<std::string, std::vector<double> > &val,
                        std::map<std::string, std::string> &, std::map<std::string, bool> &single) {
  for (auto &kv : val) {
    bool s = single.count(kv.first) ? single[kv.first] : false;
    g_out.rec(group, kv.first, s, kv.second.data(), kv.second.size());
  }
}

ReadBeamHDF5::ReadBeamHDF5() {}
ReadBeamHDF5::~ReadBeamHDF5() {}
bool ReadBeamHDF5::readGlobal(int, int, string, Setup *, Time *, bool) { return false; }
bool ReadBeamHDF5::readSlice(double, vector<Particle> *, double *, bool) { return false; }
void ReadBeamHDF5::close() {}

ReadFieldHDF5::ReadFieldHDF5() {}
ReadFieldHDF5::~ReadFieldHDF5() {}
bool ReadFieldHDF5::readGlobal(int, int, const string &, Setup *, Time *, int, bool) { return false; }
bool ReadFieldHDF5::readSlice(double, vector<complex<double> > *) { return false; }
void ReadFieldHDF5::close() {}

ReadMapHDF5::ReadMapHDF5() {}
ReadMapHDF5::~ReadMapHDF5() {}
bool ReadMapHDF5::readDataset(const std::string &, std::vector<double> &, bool) { return false; }
bool ReadMapHDF5::open(unsigned long, const string &) { return false; }
void ReadMapHDF5::close() const {}

WriteBeamHDF5::WriteBeamHDF5() {}
WriteBeamHDF5::~WriteBeamHDF5() {}
bool WriteBeamHDF5::write(string root, Beam *beam, int) {
  RawFile f;
  if (!f.open(root + ".par.h5.raw")) return false;
  for (size_t is = 0; is < beam->beam.size(); is++) {
    const auto &s = beam->beam[is];
    std::vector<double> buf(s.size() * 6);
    for (size_t i = 0; i < s.size(); i++) {
      buf[6 * i + 0] = s[i].gamma;
      buf[6 * i + 1] = s[i].theta;
      buf[6 * i + 2] = s[i].x;
      buf[6 * i + 3] = s[i].y;
      buf[6 * i + 4] = s[i].px;
      buf[6 * i + 5] = s[i].py;
    }
    char name[32];
    std::snprintf(name, sizeof(name), "slice%06zu", is + 1);
    f.rec(name, "particles", false, buf.data(), buf.size());
    double cur = beam->current[is];
    f.rec(name, "current", true, &cur, 1);
  }
  f.close();
  return true;
}

WriteFieldHDF5::WriteFieldHDF5() {}
WriteFieldHDF5::~WriteFieldHDF5() {}
bool WriteFieldHDF5::write(string root, vector<Field *> *field) {
  for (size_t k = 0; k < field->size(); k++) {
    Field *fld = field->at(k);
    std::string fn = root;
    if (fld->getHarm() != 1) fn += ".h" + std::to_string(fld->getHarm());
    RawFile f;
    if (!f.open(fn + ".fld.h5.raw")) return false;
    size_t ns = fld->field.size();
    // slices are written in time-window order: the storage slot of window slice j
    // is (j + first) % ns
    for (size_t j = 0; j < ns; j++) {
      const auto &sl = fld->field[(j + fld->first) % ns];
      std::vector<double> buf(sl.size() * 2);
      for (size_t i = 0; i < sl.size(); i++) {
        buf[2 * i] = sl[i].real();
        buf[2 * i + 1] = sl[i].imag();
      }
      char name[32];
      std::snprintf(name, sizeof(name), "slice%06zu", j + 1);
      f.rec(name, "field", false, buf.data(), buf.size());
    }
    f.close();
  }
  return true;
}

WriteWakeHDF5::WriteWakeHDF5() {}
WriteWakeHDF5::~WriteWakeHDF5() {}
bool WriteWakeHDF5::write(string, double *, double *, double *, double *, unsigned long) { return true; }

SDDSBeam::SDDSBeam() {}
SDDSBeam::~SDDSBeam() {}
bool SDDSBeam::init(int, int, map<string, string> *, Beam *, Setup *, Time *, Lattice *) { return false; }
