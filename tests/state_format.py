"""Reader of the reference's state-file layout, for tests.

Restates the field order of FLUID_3D_MIC::readGz (FLUID_3D_MIC.cpp:1115-1246):
10 int32, 7 doubles, 17 fields (each: 3 int32 dims, center, lengths, doubles),
the obstacle bytes, center, lengths, an int32 IOP count, then prevorticity,
midMaccormack and postIOP, and, once a moving-box step has built it, the
obstacle matrix (SPARSE_MATRIX::writeGz, SPARSE_MATRIX.cpp:537-561: int32
rows, cols, entry count, then per entry int32 row, int32 col, double value).
Handles concatenated gzip members like zlib.
"""
import gzip
import struct

import numpy as np

FIELD_ORDER = ["density", "densityOld", "heat", "heatOld", "pressure", "divergence",
               "velocity", "velocityOld", "force", "vorticity", "preprojection",
               "prediffusion", "preadvection", "cachedQuadratic", "postadvection",
               "cachedPressure", "cachedDivergence"]
VECTOR = {"velocity", "velocityOld", "force", "vorticity", "preprojection", "prediffusion",
          "preadvection", "cachedQuadratic", "postadvection", "prevorticity",
          "midMaccormack", "postIOP"}


class _Cursor:
    def __init__(self, b):
        self.b, self.o = b, 0

    def take(self, fmt, n=1):
        size = struct.calcsize(fmt) * n
        v = struct.unpack_from("<" + fmt * n, self.b, self.o)
        self.o += size
        return v

    def raw(self, nbytes):
        v = self.b[self.o:self.o + nbytes]
        self.o += nbytes
        return v


def read_state(path):
    with gzip.open(path, "rb") as f:
        c = _Cursor(f.read())
    ints = c.take("i", 10)
    dbls = c.take("d", 7)
    out = {"header_ints": ints, "header_doubles": dbls}

    def field(name):
        dims = c.take("i", 3)
        center = c.take("d", 3)
        lengths = c.take("d", 3)
        n = dims[0] * dims[1] * dims[2] * (3 if name in VECTOR else 1)
        data = np.frombuffer(c.raw(8 * n), dtype="<f8").copy()
        out[name] = data
        out[name + "_meta"] = (dims, center, lengths)

    for n in FIELD_ORDER:
        field(n)
    total = ints[7]
    out["obstacles"] = np.frombuffer(c.raw(total), dtype=np.uint8).copy()
    out["center"] = c.take("d", 3)
    out["lengths"] = c.take("d", 3)
    out["iop_count"] = c.take("i")[0]
    for n in ("prevorticity", "midMaccormack", "postIOP"):
        field(n)
    if len(c.b) - c.o >= 12:
        rows, cols, total = c.take("i", 3)
        e = np.frombuffer(c.raw(16 * total), dtype=SPARSE_ENTRY)
        out["iop_dims"] = (rows, cols)
        out["iop_ij"] = np.stack([e["row"], e["col"]], axis=1).astype(np.int32)
        out["iop_val"] = e["val"].copy()
    out["trailing_bytes"] = len(c.b) - c.o
    return out


SPARSE_ENTRY = np.dtype([("row", "<i4"), ("col", "<i4"), ("val", "<f8")])


def read_sparse_matrices(path):
    """Consecutive SPARSE_MATRIX::write records (SPARSE_MATRIX.cpp:508-532),
    e.g. appendStreams' neumann.iop.matrices: a list of (dims, ij, values)."""
    b = open(path, "rb").read()
    c = _Cursor(b)
    mats = []
    while c.o < len(b):
        rows, cols, total = c.take("i", 3)
        e = np.frombuffer(c.raw(16 * total), dtype=SPARSE_ENTRY)
        mats.append(((rows, cols), np.stack([e["row"], e["col"]], axis=1).astype(np.int32),
                     e["val"].copy()))
    return mats
