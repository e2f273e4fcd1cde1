"""A reader of HDF5 files written from the file format specification (Hierarchical Data
Format Version 5 File Format Specification: superblock version 0 and 1, version 1 object
headers, symbol-table groups with version 1 B-trees, local heaps and symbol table nodes,
contiguous datasets of little-endian floating point, attributes of fixed-length strings).

Test infrastructure: it checks the files of the engine's HDF5 writer where no HDF5
library exists. It decodes only what that layout uses and raises on anything else.
"""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(ValueError):
    pass


class H5File:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        b = self.b
        if b[:8] != b"\x89HDF\r\n\x1a\n":
            raise H5Error("no HDF5 signature")
        ver = b[8]
        if ver not in (0, 1):
            raise H5Error(f"superblock version {ver}")
        self.so, self.sl = b[13], b[14]
        if self.so != 8 or self.sl != 8:
            raise H5Error("offset / length sizes other than 8")
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", b, 16)
        p = 24 + (4 if ver == 1 else 0)
        base, _free, eof, _drv = struct.unpack_from("<QQQQ", b, p)
        if base != 0:
            raise H5Error("base address")
        if eof != len(b):
            raise H5Error(f"end of file address {eof} != file size {len(b)}")
        p += 32
        _name_off, self.root_header = struct.unpack_from("<QQ", b, p)

    # -- object headers ---------------------------------------------------------------
    def messages(self, addr):
        b = self.b
        ver, _r, nmsg, _refc, size = struct.unpack_from("<BBHII", b, addr)
        if ver != 1:
            raise H5Error(f"object header version {ver}")
        p, end = addr + 16, addr + 16 + size
        out = []
        while p < end and len(out) < nmsg:
            mtype, msize, _flags = struct.unpack_from("<HHB", b, p)
            if msize % 8:
                raise H5Error("message size not a multiple of 8")
            out.append((mtype, b[p + 8:p + 8 + msize]))
            p += 8 + msize
        if len(out) != nmsg or p != end:
            raise H5Error("object header: message count or size mismatch")
        return out

    @staticmethod
    def dataspace(m):
        ver, rank, flags = m[0], m[1], m[2]
        if ver != 1:
            raise H5Error(f"dataspace version {ver}")
        return tuple(struct.unpack_from("<" + "Q" * rank, m, 8)) if rank else ()

    @staticmethod
    def datatype(m):
        cls, ver = m[0] & 0x0F, m[0] >> 4
        size = struct.unpack_from("<I", m, 4)[0]
        if cls == 1:  # floating point
            if m[1] & 1 or size != 8:
                raise H5Error("only little-endian 8-byte floats")
            off, prec, eloc, esize, mloc, msize, bias = struct.unpack_from("<HHBBBBI", m, 8)
            if (off, prec, eloc, esize, mloc, msize, bias) != (0, 64, 52, 11, 0, 52, 1023) or m[2] != 63:
                raise H5Error("not an IEEE double")
            return ("f8", size)
        if cls == 3:
            return ("str", size)
        if cls == 0:  # fixed point
            if m[1] & 1 or size != 4 or not (m[1] & 8):
                raise H5Error("only little-endian signed 4-byte integers")
            return ("i4", size)
        raise H5Error(f"datatype class {cls}")

    def attribute(self, m):
        ver, _r, nsize, tsize, ssize = struct.unpack_from("<BBHHH", m, 0)
        if ver != 1:
            raise H5Error(f"attribute version {ver}")
        pad = lambda n: (n + 7) & ~7
        p = 8
        name = m[p:p + nsize].split(b"\x00")[0].decode()
        p += pad(nsize)
        dtype = self.datatype(m[p:p + tsize])
        p += pad(tsize)
        dims = self.dataspace(m[p:p + ssize])
        p += pad(ssize)
        n = int(np.prod(dims)) if dims else 1
        raw = m[p:p + n * dtype[1]]
        if dtype[0] == "str":
            return name, raw.split(b"\x00")[0].decode()
        return name, np.frombuffer(raw, "<f8").reshape(dims)

    # -- groups -------------------------------------------------------------------------
    def heap(self, addr):
        b = self.b
        if b[addr:addr + 4] != b"HEAP" or b[addr + 4] != 0:
            raise H5Error("local heap")
        size, free, data = struct.unpack_from("<QQQ", b, addr + 8)
        if free != 1 and free >= size:  # 1: the HDF5 library's empty free list
            raise H5Error("local heap free list")
        return b[data:data + size]

    def btree_children(self, addr):
        b = self.b
        if b[addr:addr + 4] != b"TREE" or b[addr + 4] != 0:
            raise H5Error("group B-tree node")
        level, used = b[addr + 5], struct.unpack_from("<H", b, addr + 6)[0]
        size = 24 + (2 * self.internal_k + 1) * 8 + 2 * self.internal_k * 8
        if addr + size > len(b):
            raise H5Error("B-tree node beyond the end of the file")
        kids = [struct.unpack_from("<Q", b, addr + 24 + 8 + 16 * i)[0] for i in range(used)]
        if level == 0:
            return kids
        return [s for k in kids for s in self.btree_children(k)]

    def find(self, header, name):
        """The member `name` of a group found as the HDF5 library finds it: down the
        B-tree by its keys (child i holds the names in (key i, key i+1]), then a search
        of the symbol table node. Returns the member's object header address."""
        st = [m for t, m in self.messages(header) if t == 0x0011][0]
        tree, heap = struct.unpack_from("<QQ", st, 0)
        names = self.heap(heap)
        key = lambda off: names[off:names.index(b"\x00", off)].decode()
        b, node = self.b, tree
        while True:
            level, used = b[node + 5], struct.unpack_from("<H", b, node + 6)[0]
            keys = [key(struct.unpack_from("<Q", b, node + 24 + 16 * i)[0]) for i in range(used + 1)]
            kids = [struct.unpack_from("<Q", b, node + 32 + 16 * i)[0] for i in range(used)]
            for i in range(used):
                if keys[i] != keys[i + 1] and not keys[i] < keys[i + 1]:
                    raise H5Error("B-tree keys out of order")
            i = next((i for i in range(used) if keys[i] < name <= keys[i + 1]), None)
            if i is None:
                raise KeyError(name)
            if level == 0:
                snod = kids[i]
                n = struct.unpack_from("<H", b, snod + 6)[0]
                for j in range(n):
                    noff, oh = struct.unpack_from("<QQ", b, snod + 8 + 40 * j)
                    if key(noff) == name:
                        return oh
                raise KeyError(name)
            node = kids[i]

    def group(self, header):
        msgs = self.messages(header)
        st = [m for t, m in msgs if t == 0x0011]
        if not st:
            raise H5Error("a group without a symbol table message")
        tree, heap = struct.unpack_from("<QQ", st[0], 0)
        names = self.heap(heap)
        if names[:1] != b"\x00":
            raise H5Error("local heap offset 0 is not the empty name")
        out = {}
        prev = None
        snod_size = 8 + 2 * self.leaf_k * 40
        for snod in self.btree_children(tree):
            b = self.b
            if b[snod:snod + 4] != b"SNOD" or b[snod + 4] != 1 or snod + snod_size > len(b):
                raise H5Error("symbol table node")
            n = struct.unpack_from("<H", b, snod + 6)[0]
            for i in range(n):
                e = snod + 8 + 40 * i
                noff, oh, cache = struct.unpack_from("<QQI", b, e)
                name = names[noff:names.index(b"\x00", noff)].decode()
                if prev is not None and name <= prev:
                    raise H5Error("symbol table entries out of order")
                prev = name
                out[name] = self.obj(oh)
        return out

    def obj(self, header):
        msgs = self.messages(header)
        types = {t for t, _ in msgs}
        if 0x0011 in types:
            return self.group(header)
        dims = dtype = layout = None
        attrs = {}
        for t, m in msgs:
            if t == 0x0001:
                dims = self.dataspace(m)
            elif t == 0x0003:
                dtype = self.datatype(m)
            elif t == 0x0008:
                if m[0] != 3 or m[1] != 1:
                    raise H5Error("only version 3 contiguous layouts")
                layout = struct.unpack_from("<QQ", m, 2)
            elif t == 0x000C:
                k, v = self.attribute(m)
                attrs[k] = v
        if dims is None or dtype is None or layout is None:
            raise H5Error("a dataset without dataspace, datatype or layout")
        addr, size = layout
        n = int(np.prod(dims))
        item = 4 if dtype[0] == "i4" else 8
        if size != item * n:
            raise H5Error("layout size does not match the dataspace")
        fmt = "<i4" if dtype[0] == "i4" else "<f8"
        data = np.frombuffer(self.b, fmt, count=n, offset=addr).reshape(dims) if n else np.zeros(dims)
        return data, attrs

    def tree(self):
        return self.obj(self.root_header)


def read(path):
    """{name: subtree or (array, {attribute: value})}"""
    return H5File(path).tree()


def get(path, name):
    """One object by its path ("Beam/energy"), found through the groups' B-tree keys."""
    f = H5File(path)
    h = f.root_header
    for part in name.strip("/").split("/"):
        h = f.find(h, part)
    return f.obj(h)
