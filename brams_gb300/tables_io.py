"""Reader/writer for the RRTMG_LW table container (``*.gblw`` files).

The solver's constant data (reference atmosphere, Planck integrals, cloud
optics, g-point reduction maps, k-distribution tables) lives in one flat
binary container so that the CUDA library, the CPU oracle and the Python
tests all read the same bytes.  Layout (little endian):

    magic   8 bytes  b"GBLWTBL1"
    count   u32
    entries count x {
        name   48 bytes, NUL padded ASCII
        dtype  u32     0 = float64, 1 = int32
        ndim   u32     0..4
        dims   4 x u32 Fortran extents, first index fastest (unused = 1)
        nbytes u64
        data   nbytes  column-major (Fortran) element order
    }

Arrays keep the Fortran index order of the reference modules
(e.g. ``totplnk(181,16)`` is stored with the 181 axis fastest), so the
1-based Fortran subscripts in the reference map to flat offsets directly.
"""
from __future__ import annotations

import struct
from collections import OrderedDict

import numpy as np

MAGIC = b"GBLWTBL1"
_DT = {0: np.float64, 1: np.int32}


def write_tables(path: str, tables: "OrderedDict[str, np.ndarray]") -> None:
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<I", len(tables)))
        for name, arr in tables.items():
            arr = np.asarray(arr)
            if arr.dtype.kind == "f":
                code, arr = 0, arr.astype(np.float64)
            elif arr.dtype.kind in "iu":
                code, arr = 1, arr.astype(np.int32)
            else:
                raise TypeError(f"{name}: unsupported dtype {arr.dtype}")
            if arr.ndim > 4:
                raise ValueError(f"{name}: ndim {arr.ndim} > 4")
            dims = list(arr.shape) + [1] * (4 - arr.ndim)
            raw = np.asfortranarray(arr).tobytes(order="F")
            nb = name.encode("ascii")
            if len(nb) >= 48:
                raise ValueError(f"name too long: {name}")
            f.write(nb + b"\0" * (48 - len(nb)))
            f.write(struct.pack("<II4IQ", code, arr.ndim, *dims, len(raw)))
            f.write(raw)


def read_tables(path: str) -> "OrderedDict[str, np.ndarray]":
    out: "OrderedDict[str, np.ndarray]" = OrderedDict()
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError(f"{path}: bad magic")
        (count,) = struct.unpack("<I", f.read(4))
        for _ in range(count):
            name = f.read(48).rstrip(b"\0").decode("ascii")
            code, ndim, d0, d1, d2, d3, nbytes = struct.unpack("<II4IQ", f.read(32))
            dims = (d0, d1, d2, d3)[:ndim]
            data = np.frombuffer(f.read(nbytes), dtype=_DT[code])
            out[name] = data.reshape(dims, order="F") if ndim else data.reshape(())
    return out
