// A writer of HDF5 files for the reference's output layout (.out.h5: groups of FP64
// datasets, each with a string attribute "unit"; Output::writeGroup / writeDataset,
// src/IO/Output.cpp:309-340, HDF5Base::writeBuffer, src/IO/HDF5base.cpp:74-128), for
// machines without the HDF5 library.
//
// The file follows the HDF5 file format specification (version 0 superblock, version 1
// object headers, groups as symbol tables: a version 1 B-tree of group nodes over symbol
// table nodes and a local heap of link names), the layout the HDF5 library itself writes
// by default:
//   superblock (96 B) | per object, children first: dataset raw data (contiguous
//   little-endian doubles), dataset object headers (dataspace v1, datatype v1 IEEE
//   double, layout v3 contiguous, attribute v1 "unit": fixed-length ASCII string of the
//   unit's length, null-terminated padding, scalar dataspace); per group: local heap
//   (names at 8-byte offsets, "" at 0), symbol table nodes of 2K = 8 entries sorted by
//   name, B-tree nodes of up to 2K = 32 children (leaves over the symbol table nodes,
//   then as many internal levels as the group needs), the group's object header (one
//   symbol-table message).
// Group leaf node K = 4, internal node K = 16 (the library's defaults). The local heap's
// free list is empty, written as the library's end marker 1. Integer datasets are 32-bit
// signed little-endian without attributes (HDF5Base::writeSingleNodeInt). Everything is
// 8-byte aligned; the whole file is assembled in memory and written at g4gpu_h5_close.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "g4gpu.h"

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kLeafK = 4, kInternalK = 16;
constexpr size_t kEntry = 40;                                     // symbol table entry
constexpr size_t kSnodSize = 8 + 2 * kLeafK * kEntry;             // SNOD: 8 entries
constexpr size_t kTreeSize = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;  // 32 children

struct Obj {
  bool group = true;
  std::map<std::string, std::unique_ptr<Obj>> members;  // sorted by name (strcmp order)
  std::vector<uint64_t> dims;
  std::vector<double> data;
  std::vector<int32_t> idata;  // integer datasets
  bool is_int = false;
  bool has_unit = true;
  std::string unit;
};

struct Buf {
  std::vector<uint8_t> b;
  size_t tell() const { return b.size(); }
  void align8() {
    while (b.size() % 8) b.push_back(0);
  }
  void u8(unsigned v) { b.push_back((uint8_t)v); }
  void u16(unsigned v) {
    u8(v & 0xff);
    u8((v >> 8) & 0xff);
  }
  void u32(uint32_t v) {
    for (int i = 0; i < 4; i++) u8((v >> (8 * i)) & 0xff);
  }
  void u64(uint64_t v) {
    for (int i = 0; i < 8; i++) u8((v >> (8 * i)) & 0xff);
  }
  void bytes(const void *p, size_t n) {
    const uint8_t *q = (const uint8_t *)p;
    b.insert(b.end(), q, q + n);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void put64(size_t at, uint64_t v) {
    for (int i = 0; i < 8; i++) b[at + i] = (uint8_t)((v >> (8 * i)) & 0xff);
  }
};

size_t pad8(size_t n) { return (n + 7) & ~(size_t)7; }

// one header message of a version 1 object header: type, size, flags, data padded to 8
void message(Buf &m, unsigned type, const Buf &data) {
  m.u16(type);
  m.u16((unsigned)pad8(data.tell()));
  m.u8(0);
  m.zeros(3);
  m.bytes(data.b.data(), data.tell());
  m.zeros(pad8(data.tell()) - data.tell());
}

// version 1 object header with `count` messages in `m`; returns its address
uint64_t object_header(Buf &f, const Buf &m, unsigned count) {
  f.align8();
  const uint64_t at = f.tell();
  f.u8(1);  // version
  f.u8(0);
  f.u16(count);
  f.u32(1);  // reference count
  f.u32((uint32_t)m.tell());
  f.u32(0);  // pads the 12-byte prefix to 16
  f.bytes(m.b.data(), m.tell());
  return at;
}

// dataspace message, version 1: rank and dimensions (rank 0: scalar)
Buf dataspace(const std::vector<uint64_t> &dims) {
  Buf d;
  d.u8(1);
  d.u8((unsigned)dims.size());
  d.u8(0);  // no maximum dimensions
  d.u8(0);
  d.u32(0);
  for (uint64_t n : dims) d.u64(n);
  return d;
}

// datatype message, version 1: IEEE 754 double, little endian
Buf datatype_double() {
  Buf d;
  d.u8((1 << 4) | 1);  // version 1, floating point
  d.u8(0x20);          // little endian, no padding, implied leading mantissa bit
  d.u8(63);            // sign bit
  d.u8(0);
  d.u32(8);
  d.u16(0);   // bit offset
  d.u16(64);  // precision
  d.u8(52);   // exponent location
  d.u8(11);   // exponent size
  d.u8(0);    // mantissa location
  d.u8(52);   // mantissa size
  d.u32(1023);
  return d;
}

// datatype message, version 1: fixed-length ASCII string of n bytes, null-terminated
Buf datatype_string(uint32_t n) {
  Buf d;
  d.u8((1 << 4) | 3);
  d.u8(0);  // null terminated, ASCII
  d.u8(0);
  d.u8(0);
  d.u32(n);
  return d;
}

// datatype message, version 1: 32-bit signed integer, little endian
Buf datatype_int32() {
  Buf d;
  d.u8((1 << 4) | 0);  // version 1, fixed point
  d.u8(0x08);          // little endian, no padding, signed
  d.u8(0);
  d.u8(0);
  d.u32(4);
  d.u16(0);   // bit offset
  d.u16(32);  // precision
  return d;
}

uint64_t write_dataset(Buf &f, const Obj &o) {
  f.align8();
  const uint64_t raw = f.tell();
  size_t n = o.is_int ? o.idata.size() : o.data.size();
  if (o.is_int) {
    for (int32_t v : o.idata) f.u32((uint32_t)v);
  } else {
    for (double v : o.data) {
      uint64_t u;
      std::memcpy(&u, &v, 8);
      f.u64(u);
    }
  }
  Buf m;
  message(m, 0x0001, dataspace(o.dims));
  message(m, 0x0003, o.is_int ? datatype_int32() : datatype_double());
  Buf lay;  // layout, version 3, contiguous
  lay.u8(3);
  lay.u8(1);
  lay.u64(n == 0 ? kUndef : raw);
  lay.u64(n * (o.is_int ? 4 : 8));
  message(m, 0x0008, lay);
  if (!o.has_unit) return object_header(f, m, 3);
  // attribute "unit", version 1
  const std::string unit = o.unit.empty() ? std::string(" ") : o.unit;
  const Buf dt = datatype_string((uint32_t)unit.size()), ds = dataspace({});
  const std::string name = "unit";
  Buf at;
  at.u8(1);
  at.u8(0);
  at.u16((unsigned)name.size() + 1);
  at.u16((unsigned)dt.tell());
  at.u16((unsigned)ds.tell());
  at.bytes(name.c_str(), name.size() + 1);
  at.zeros(pad8(name.size() + 1) - (name.size() + 1));
  at.bytes(dt.b.data(), dt.tell());
  at.zeros(pad8(dt.tell()) - dt.tell());
  at.bytes(ds.b.data(), ds.tell());
  at.zeros(pad8(ds.tell()) - ds.tell());
  at.bytes(unit.data(), unit.size());
  message(m, 0x000C, at);
  return object_header(f, m, 4);
}

struct GroupAddr {
  uint64_t header, btree, heap;
};

GroupAddr write_group(Buf &f, const Obj &g, std::string &err) {
  // children first
  std::vector<std::pair<std::string, GroupAddr>> kids;
  for (auto &kv : g.members) {
    GroupAddr a{};
    if (kv.second->group) {
      a = write_group(f, *kv.second, err);
      if (!err.empty()) return {};
    } else {
      a.header = write_dataset(f, *kv.second);
    }
    kids.push_back({kv.first, a});
  }
  const size_t n = kids.size();
  const size_t nsnod = n ? (n + 2 * kLeafK - 1) / (2 * kLeafK) : 0;
  // local heap: "" at offset 0, then the names
  Buf seg;
  seg.zeros(8);
  std::vector<uint64_t> off(n);
  for (size_t i = 0; i < n; i++) {
    off[i] = seg.tell();
    seg.bytes(kids[i].first.c_str(), kids[i].first.size() + 1);
    seg.align8();
  }
  f.align8();
  const uint64_t heap = f.tell();
  f.bytes("HEAP", 4);
  f.u8(0);
  f.zeros(3);
  f.u64(seg.tell());
  f.u64(1);  // free list: none (the library's end marker)
  f.u64(heap + 32);
  f.bytes(seg.b.data(), seg.tell());
  // symbol table nodes of up to 8 sorted entries; each child of a B-tree node carries
  // the heap offset of the last (largest) name below it as its right key
  std::vector<std::pair<uint64_t, uint64_t>> level;  // (address, offset of its last name)
  for (size_t s = 0; s < nsnod; s++) {
    f.align8();
    const uint64_t at = f.tell();
    const size_t i0 = s * 2 * kLeafK, i1 = std::min(n, i0 + 2 * kLeafK);
    f.bytes("SNOD", 4);
    f.u8(1);
    f.u8(0);
    f.u16((unsigned)(i1 - i0));
    for (size_t i = i0; i < i1; i++) {
      f.u64(off[i]);
      f.u64(kids[i].second.header);
      const bool grp = g.members.at(kids[i].first)->group;
      f.u32(grp ? 1 : 0);  // cache type: groups carry their B-tree and heap
      f.u32(0);
      f.u64(grp ? kids[i].second.btree : 0);
      f.u64(grp ? kids[i].second.heap : 0);
    }
    f.zeros(kSnodSize - 8 - (i1 - i0) * kEntry);
    level.push_back({at, off[i1 - 1]});
  }
  // B-tree nodes, leaves first (level 0 over the symbol table nodes), up the levels until
  // one node remains: key 0 (""), child, key, child, ..., key
  uint64_t tree = 0;
  int depth = 0;
  do {
    std::vector<std::pair<uint64_t, uint64_t>> up;
    const size_t nnode = std::max<size_t>(1, (level.size() + 2 * kInternalK - 1) / (2 * kInternalK));
    for (size_t b = 0; b < nnode; b++) {
      const size_t c0 = b * 2 * kInternalK, c1 = std::min(level.size(), c0 + 2 * kInternalK);
      f.align8();
      const uint64_t at = f.tell();
      f.bytes("TREE", 4);
      f.u8(0);  // group node
      f.u8((unsigned)depth);
      f.u16((unsigned)(c1 - c0));
      f.u64(kUndef);  // siblings: readers of symbol tables follow the children only
      f.u64(kUndef);
      f.u64(0);
      for (size_t c = c0; c < c1; c++) {
        f.u64(level[c].first);
        f.u64(level[c].second);
      }
      f.zeros(kTreeSize - (f.tell() - at));
      up.push_back({at, c1 > c0 ? level[c1 - 1].second : 0});
    }
    level.swap(up);
    tree = level[0].first;
    depth++;
  } while (level.size() > 1);
  // the group's object header: one symbol table message
  Buf st;
  st.u64(tree);
  st.u64(heap);
  Buf m;
  message(m, 0x0011, st);
  const uint64_t hdr = object_header(f, m, 1);
  return {hdr, tree, heap};
}

}  // namespace

struct g4gpu_h5_s {
  std::string path, err;
  Obj root;
};

extern "C" {

int g4gpu_h5_create(const char *path, g4gpu_h5 *out) {
  if (!path || !out) return G4GPU_ERR_ARG;
  auto *f = new g4gpu_h5_s;
  f->path = path;
  *out = f;
  return G4GPU_OK;
}

int g4gpu_h5_dataset(g4gpu_h5 f, const char *path, int rank, const long long *dims, const double *data,
                     const char *unit) {
  if (!f || !path || rank < 1 || rank > 8 || !dims || !data) return G4GPU_ERR_ARG;
  size_t n = 1;
  for (int i = 0; i < rank; i++) {
    if (dims[i] < 0) return G4GPU_ERR_ARG;
    n *= (size_t)dims[i];
  }
  // path a/b/c: groups a, b (created as needed), dataset c
  std::string p(path);
  Obj *g = &f->root;
  size_t pos;
  while ((pos = p.find('/')) != std::string::npos) {
    const std::string part = p.substr(0, pos);
    p = p.substr(pos + 1);
    if (part.empty()) continue;
    auto it = g->members.find(part);
    if (it == g->members.end()) it = g->members.emplace(part, std::make_unique<Obj>()).first;
    if (!it->second->group) return G4GPU_ERR_ARG;  // a dataset of that name
    g = it->second.get();
  }
  if (p.empty() || g->members.count(p)) return G4GPU_ERR_ARG;
  auto o = std::make_unique<Obj>();
  o->group = false;
  o->dims.assign(dims, dims + rank);
  o->data.assign(data, data + n);
  o->unit = unit ? unit : "";
  g->members.emplace(p, std::move(o));
  return G4GPU_OK;
}

int g4gpu_h5_dataset_int(g4gpu_h5 f, const char *path, int n, const int *data) {
  if (!f || !path || n < 0 || (n > 0 && !data)) return G4GPU_ERR_ARG;
  const long long dims[1] = {n};
  // placed like a double dataset, then retyped
  std::vector<double> tmp((size_t)n, 0.0);
  int rc = g4gpu_h5_dataset(f, path, 1, dims, tmp.data(), nullptr);
  if (rc) return rc;
  std::string p(path);
  Obj *g = &f->root;
  size_t pos;
  while ((pos = p.find('/')) != std::string::npos) {
    const std::string part = p.substr(0, pos);
    p = p.substr(pos + 1);
    if (!part.empty()) g = g->members.at(part).get();
  }
  Obj &o = *g->members.at(p);
  o.is_int = true;
  o.has_unit = false;
  o.data.clear();
  o.idata.assign(data, data + n);
  return G4GPU_OK;
}

int g4gpu_h5_close(g4gpu_h5 f) {
  if (!f) return G4GPU_ERR_ARG;
  Buf b;
  b.zeros(96);  // the superblock, filled in below
  std::string err;
  GroupAddr root = write_group(b, f->root, err);
  int rc = G4GPU_OK;
  if (!err.empty()) {
    rc = G4GPU_ERR_ARG;
  } else {
    b.align8();
    Buf sb;
    sb.bytes("\x89HDF\r\n\x1a\n", 8);
    sb.u8(0);  // superblock version
    sb.u8(0);  // free-space storage version
    sb.u8(0);  // root group symbol table entry version
    sb.u8(0);
    sb.u8(0);  // shared header message format version
    sb.u8(8);  // size of offsets
    sb.u8(8);  // size of lengths
    sb.u8(0);
    sb.u16(kLeafK);
    sb.u16(kInternalK);
    sb.u32(0);  // file consistency flags
    sb.u64(0);  // base address
    sb.u64(kUndef);
    sb.u64(b.tell());  // end of file
    sb.u64(kUndef);
    // root group symbol table entry
    sb.u64(0);
    sb.u64(root.header);
    sb.u32(1);
    sb.u32(0);
    sb.u64(root.btree);
    sb.u64(root.heap);
    std::memcpy(b.b.data(), sb.b.data(), 96);
    FILE *fp = std::fopen(f->path.c_str(), "wb");
    if (!fp) {
      rc = G4GPU_ERR_ARG;
    } else {
      if (std::fwrite(b.b.data(), 1, b.tell(), fp) != b.tell()) rc = G4GPU_ERR_ARG;
      if (std::fclose(fp) != 0) rc = G4GPU_ERR_ARG;
    }
  }
  delete f;
  return rc;
}

}  // extern "C"
