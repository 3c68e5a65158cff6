"""var.dat snapshots in the reference layout (src/io_dist.f90:108-199 output_snap,
:657-787 input_snap / read_snap).

A snapshot is a gfortran sequential unformatted file:
  record 1: f(mx,my,mz,nvar)                     (REAL, Fortran order, ghosts included)
  record 2: t, x(mx), y(my), z(mz), dx, dy, dz   (REAL; t is REAL too in the double build)
  optional persistent block: [id_block_PERSISTENT=2000] then [id][value] records
  (src/record_types.h:13, src/io_dist.f90:495-616).
Every record is framed by 4-byte length markers.  Records longer than
2**31-9 bytes are split into subrecords: the leading marker is negative when
more subrecords follow, the trailing marker is negative for a continuation
subrecord (readers take its absolute value), as gfortran writes them and as
python/pencil/read/fortran_file.py:95-130 reads them.
"""
from __future__ import annotations

import os
import struct

import numpy as np

MAX_SUBRECORD = 2 ** 31 - 9
ID_BLOCK_PERSISTENT = 2000


def _write_record(fh, payload: memoryview, max_sub: int = MAX_SUBRECORD) -> None:
    n = len(payload)
    if n == 0:
        fh.write(struct.pack("<i", 0)); fh.write(struct.pack("<i", 0))
        return
    off, first = 0, True
    while off < n:
        ln = min(max_sub, n - off)
        last = off + ln >= n
        fh.write(struct.pack("<i", ln if last else -ln))
        fh.write(payload[off:off + ln])
        fh.write(struct.pack("<i", ln if first else -ln))
        off += ln
        first = False


def _read_record(fh) -> bytes:
    chunks = []
    while True:
        head = fh.read(4)
        if len(head) < 4:
            raise EOFError("end of file")
        h = struct.unpack("<i", head)[0]
        ln = abs(h)
        data = fh.read(ln)
        tail = fh.read(4)
        if len(data) < ln or len(tail) < 4 or abs(struct.unpack("<i", tail)[0]) != ln:
            raise ValueError("corrupt record markers")
        chunks.append(data)
        if h >= 0:
            return b"".join(chunks)


def write_var(path: str, f: np.ndarray, t: float, x, y, z, dx: float, dy: float, dz: float,
              precision: int = 8, persistent: dict | None = None, max_subrecord: int = MAX_SUBRECORD) -> None:
    """Write a snapshot; f is (mx,my,mz,nvar).  persistent: {id: array-like} records."""
    dt = np.float64 if precision == 8 else np.float32
    fa = np.asfortranarray(f, dtype=dt)
    with open(path, "wb") as fh:
        _write_record(fh, memoryview(fa.reshape(-1, order="F")).cast("B"), max_subrecord)
        grid = np.concatenate([[t], np.asarray(x), np.asarray(y), np.asarray(z), [dx, dy, dz]]).astype(dt)
        _write_record(fh, memoryview(grid).cast("B"))
        if persistent:
            _write_record(fh, memoryview(np.array([ID_BLOCK_PERSISTENT], np.int32)).cast("B"))
            for rid, val in persistent.items():
                _write_record(fh, memoryview(np.array([rid], np.int32)).cast("B"))
                _write_record(fh, memoryview(np.ascontiguousarray(val)).cast("B"))


def read_var(path: str, mx: int, my: int, mz: int, nvar: int, precision: int = 8) -> dict:
    """Read a snapshot written by the reference or by write_var."""
    dt = np.float64 if precision == 8 else np.float32
    with open(path, "rb") as fh:
        rec = _read_record(fh)
        n = mx * my * mz * nvar
        if len(rec) != n * np.dtype(dt).itemsize:
            raise ValueError(f"f record holds {len(rec)} bytes, expected {n * np.dtype(dt).itemsize}")
        f = np.frombuffer(rec, dtype=dt).reshape((mx, my, mz, nvar), order="F").copy(order="F")
        g = np.frombuffer(_read_record(fh), dtype=dt)
        if g.size < 1 + mx + my + mz + 3:
            raise ValueError("grid record too short")
        out = dict(f=f, t=float(g[0]), x=g[1:1 + mx].copy(), y=g[1 + mx:1 + mx + my].copy(),
                   z=g[1 + mx + my:1 + mx + my + mz].copy())
        out["dx"], out["dy"], out["dz"] = (float(v) for v in g[1 + mx + my + mz:4 + mx + my + mz])
        pers = {}
        try:
            head = _read_record(fh)
            if np.frombuffer(head, np.int32)[0] == ID_BLOCK_PERSISTENT:
                while True:
                    rid = int(np.frombuffer(_read_record(fh), np.int32)[0])
                    pers[rid] = _read_record(fh)
        except EOFError:
            pass
        out["persistent"] = pers
    return out


def read_dim(path: str) -> tuple[int, int, int, int]:
    """mx, my, mz, mvar from a reference dim.dat."""
    with open(path) as fh:
        v = fh.readline().split()
    return int(v[0]), int(v[1]), int(v[2]), int(v[3])


def write_box_snapshot(path: str, p, f: np.ndarray, t: float) -> None:
    """Snapshot of a box with the grid of grid.f90:123-151 (x_i = x0 + (i-3+1/2) dx on a
    periodic axis, x0 + (i-3) dx with dx = L/(n-1) otherwise)."""
    x, y, z = (p.axis(i) for i in range(3))
    write_var(path, f, t, x, y, z, p.spacing(0), p.spacing(1), p.spacing(2), precision=8)


def file_size(path: str) -> int:
    return os.path.getsize(path)
