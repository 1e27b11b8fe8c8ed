"""The ``.dgt`` table bundle: named float64 arrays in one flat file.

It replaces the reference's HDF5 files (``<name>_tables.h5`` and
``<name>_initial_conditions.h5``, dengo/chemical_network.py:310-328), whose
library is not available here.  Layout, all little-endian::

    8 bytes   magic  b"DGTBL001"
    uint32    number of datasets
    per dataset:
      uint32  name length L;  L bytes of ASCII name (no leading '/')
      uint64  element count n;  n float64 values

The C reader lives in ``csrc/dg_tablefile.h``.
"""

import struct

import numpy as np

MAGIC = b"DGTBL001"


def write_table_file(path, datasets):
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<I", len(datasets)))
        for name, arr in datasets.items():
            a = np.ascontiguousarray(arr, dtype="<f8").ravel()
            b = name.strip("/").encode("ascii")
            f.write(struct.pack("<I", len(b)))
            f.write(b)
            f.write(struct.pack("<Q", a.size))
            f.write(a.tobytes())


def read_table_file(path):
    out = {}
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError("%s is not a .dgt table bundle" % path)
        (count,) = struct.unpack("<I", f.read(4))
        for _ in range(count):
            (ln,) = struct.unpack("<I", f.read(4))
            name = f.read(ln).decode("ascii")
            (n,) = struct.unpack("<Q", f.read(8))
            out[name] = np.frombuffer(f.read(8 * n), dtype="<f8").copy()
    return out
