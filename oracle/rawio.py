"""Reader for the raw binary files written by the reference checker build
(oracle/ref_build/g4ref_stubs.cpp): a magic "G4RAW1\\0\\0" followed by records of
(group, dataset, single flag, float64 data).

Test infrastructure: imported only by tests/ and the fixture generator.
"""
import struct

import numpy as np


def read_raw(path):
    """Returns {group: {dataset: np.ndarray(float64)}}."""
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != b"G4RAW1\x00\x00":
        raise ValueError(f"{path}: not a raw checker file")
    pos = 8

    def rstr():
        nonlocal pos
        (n,) = struct.unpack_from("<I", buf, pos)
        pos += 4
        s = buf[pos:pos + n].decode()
        pos += n
        return s

    while pos < len(buf):
        g = rstr()
        d = rstr()
        pos += 1  # single flag
        (n,) = struct.unpack_from("<Q", buf, pos)
        pos += 8
        a = np.frombuffer(buf, dtype="<f8", count=n, offset=pos).copy()
        pos += 8 * n
        out.setdefault(g, {})[d] = a
    return out
