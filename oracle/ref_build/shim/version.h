/* Version stamp for the CPU checker build of the GENESIS 1.3 v4 reference
 * (4.6.14); written for this project in place of the CMake-generated header. */
#ifndef G4REF_VERSION_SHIM_H
#define G4REF_VERSION_SHIM_H
#include <string>
class VersionInfo {
  int vmajor = 4, vminor = 6, vrev = 14;
  bool vbeta = false;
 public:
  VersionInfo() {}
  ~VersionInfo() {}
  int Major(void) { return vmajor; }
  int Minor(void) { return vminor; }
  int Rev(void) { return vrev; }
  bool isBeta(void) { return vbeta; }
  const char *Build(void) { return "g4 checker build"; }
};
#endif
