/* Type-only stand-in for the HDF5 C API, used only to compile the GENESIS 1.3 v4
 * reference headers into a CPU checker (oracle/_ref). The reference's HDF5 I/O
 * sources are not compiled; g4ref_stubs.cpp provides do-nothing definitions of
 * the I/O classes plus a raw-binary writer for the diagnostics buffers.
 *
 * This file is test infrastructure written for this project. */
#ifndef G4REF_HDF5_SHIM_H
#define G4REF_HDF5_SHIM_H

typedef long long hid_t;
typedef unsigned long long hsize_t;
typedef int herr_t;
typedef struct { int type; } H5L_info_t;
#define H5P_DEFAULT 0
static inline int H5Lexists(hid_t, const char *, hid_t) { return 0; }

#endif
