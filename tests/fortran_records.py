"""Reader for Fortran sequential-unformatted files (4-byte record markers, little endian)."""
import struct

import numpy as np


def records(path):
    data = open(path, "rb").read()
    out, o = [], 0
    while o < len(data):
        n = struct.unpack("<i", data[o:o + 4])[0]
        out.append(data[o + 4:o + 4 + n])
        o += 8 + n
    return out


class Cursor:
    def __init__(self, buf):
        self.buf, self.o = buf, 0

    def take(self, dtype, count):
        dt = np.dtype(dtype)
        v = np.frombuffer(self.buf[self.o:self.o + dt.itemsize * count], dtype=dt).copy()
        self.o += dt.itemsize * count
        return v
