"""Output files: the reference's text layouts and a binary layout.

Text (the reference's ``wfile`` / ``wfile3d``, outputfunc.cpp:35-50, 97-123): every value printed as
``"%e "``, a newline after the last column of a row and one more after the row, so that rows are separated
by a blank line.  ``wfile`` writes a 2-D array (seismograms: one row per receiver, one column per step);
``wfile3d`` writes the xz slice at y = ny // 2 of a [nz][ny][nx] volume.

Binary (``.bin``): the 8 bytes ``BEHFOUT1``, int32 ndim, int32 dtype (1 = float32, 2 = int32), int64
dims[ndim], then the values, all little-endian, row-major.

The command-line driver ``behf_run`` writes both layouts with the same functions' conventions.
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"BEHFOUT1"


def write_wfile(path, data) -> None:
    """2-D float array -> the reference's text layout (values rounded to float32 first, as the reference's
    ``float**`` buffers are)."""
    a = np.asarray(data, np.float32)
    if a.ndim != 2:
        raise ValueError("wfile writes a 2-D array")
    with open(path, "w") as f:
        for row in a:
            f.write("".join("%e " % v for v in row.tolist()))
            f.write("\n\n")


def write_wfile3d(path, volume) -> None:
    """[nz][ny][nx] volume -> its y-mid xz slice in the reference's text layout."""
    v = np.asarray(volume, np.float32)
    if v.ndim != 3:
        raise ValueError("wfile3d writes a slice of a 3-D array")
    write_wfile(path, v[:, v.shape[1] // 2, :])


def read_wfile(path) -> np.ndarray:
    """Text layout -> float32 [rows][cols] (blank lines separate rows; a row may not be empty)."""
    rows = []
    with open(path) as f:
        for line in f:
            t = line.split()
            if t:
                rows.append(np.array(t, dtype=np.float64))
    if not rows:
        return np.zeros((0, 0), np.float32)
    if len({len(r) for r in rows}) != 1:
        raise ValueError(f"{path}: ragged rows")
    return np.asarray(rows).astype(np.float32)


_DTYPES = {1: "<f4", 2: "<i4"}


def write_binary(path, data) -> None:
    """float arrays as float32, integer arrays as int32."""
    a = np.asarray(data)
    code = 2 if np.issubdtype(a.dtype, np.integer) else 1
    a = np.ascontiguousarray(a, _DTYPES[code])
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<ii", a.ndim, code))
        f.write(struct.pack("<%dq" % a.ndim, *a.shape))
        f.write(a.tobytes())


def read_binary(path) -> np.ndarray:
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:8] != MAGIC:
        raise ValueError(f"{path}: not a BEHFOUT1 file")
    ndim, dtype = struct.unpack_from("<ii", raw, 8)
    if dtype not in _DTYPES or not 0 < ndim <= 8:
        raise ValueError(f"{path}: unsupported header (ndim {ndim}, dtype {dtype})")
    dims = struct.unpack_from("<%dq" % ndim, raw, 16)
    off = 16 + 8 * ndim
    n = int(np.prod(dims))
    if len(raw) != off + 4 * n:
        raise ValueError(f"{path}: size does not match the header")
    out = np.frombuffer(raw, _DTYPES[dtype], n, off).reshape(dims)
    return out.astype(np.float32 if dtype == 1 else np.int32)


def read(path) -> np.ndarray:
    """Either layout, by extension (.bin = binary)."""
    return read_binary(path) if str(path).endswith(".bin") else read_wfile(path)
