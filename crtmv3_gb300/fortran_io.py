"""Fortran sequential-unformatted record files, as CRTM writes its coefficient tables.

A record is ``<int32 n> <n bytes> <int32 n>``.  CRTM's binary coefficient files
begin with a record holding the magic number 123456789, which also tells the
reader the byte order (``src/Utility/Binary_File_Utility.f90:56,154-260``).
This module writes and reads such files with numpy; it is the repository's own
writer (the reference's is Fortran), used to produce the synthetic coefficient
files that both the oracle and the GPU library read.
"""
from __future__ import annotations

import struct
from typing import BinaryIO, List, Sequence

import numpy as np

MAGIC_NUMBER = 123456789


class RecordWriter:
    """Write Fortran sequential records (little endian unless told otherwise)."""

    def __init__(self, f: BinaryIO, byteorder: str = "<"):
        self.f = f
        self.bo = byteorder
        self.record(np.array([MAGIC_NUMBER], dtype=np.int32))

    def record(self, *items) -> None:
        """Write one record made of the concatenation of ``items``.

        Each item is a numpy array (written in Fortran order, i.e. the first
        index fastest: pass arrays already shaped in Fortran index order and
        they are raveled with ``order='F'``) or ``bytes``.
        """
        parts: List[bytes] = []
        for it in items:
            if isinstance(it, (bytes, bytearray)):
                parts.append(bytes(it))
            else:
                a = np.asarray(it)
                dt = a.dtype.newbyteorder(self.bo)
                parts.append(np.ravel(a, order="F").astype(dt).tobytes())
        payload = b"".join(parts)
        n = struct.pack(self.bo + "i", len(payload))
        self.f.write(n)
        self.f.write(payload)
        self.f.write(n)


class RecordReader:
    """Read Fortran sequential records; the byte order is taken from the magic record."""

    def __init__(self, f: BinaryIO):
        self.f = f
        head = f.read(4)
        if len(head) != 4:
            raise IOError("empty coefficient file")
        for bo in ("<", ">"):
            n = struct.unpack(bo + "i", head)[0]
            if n == 4:
                body = f.read(4)
                if struct.unpack(bo + "i", body)[0] != MAGIC_NUMBER:
                    raise IOError("bad magic number in coefficient file")
                f.read(4)
                self.bo = bo
                return
        raise IOError("unrecognised record marker in coefficient file")

    def record(self) -> bytes:
        head = self.f.read(4)
        if len(head) != 4:
            raise IOError("unexpected end of coefficient file")
        n = struct.unpack(self.bo + "i", head)[0]
        data = self.f.read(n)
        tail = struct.unpack(self.bo + "i", self.f.read(4))[0]
        if tail != n or len(data) != n:
            raise IOError("corrupt record markers in coefficient file")
        return data

    def split(self, data: bytes, spec: Sequence) -> list:
        """Split one record payload by ``spec``: a list of (dtype, shape) or ('S', nchar)."""
        out = []
        off = 0
        for dt, shape in spec:
            if dt == "S":
                out.append(data[off:off + shape].decode("ascii", "replace").rstrip())
                off += shape
                continue
            dtype = np.dtype(dt).newbyteorder(self.bo)
            count = int(np.prod(shape)) if shape else 1
            a = np.frombuffer(data, dtype=dtype, count=count, offset=off).astype(np.dtype(dt))
            off += count * dtype.itemsize
            out.append(a.reshape(shape, order="F") if shape else a[0])
        if off != len(data):
            raise IOError("record length does not match its layout")
        return out
