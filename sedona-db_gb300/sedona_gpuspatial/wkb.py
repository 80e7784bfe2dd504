"""Arrow binary WKB columns as plain numpy buffers.

A column is ``WkbColumn(offsets, data, validity)``: ``offsets`` is int32 (Arrow
``binary``) or int64 (Arrow ``large_binary``) with n+1 entries, ``data`` the
concatenated little-endian WKB bytes, ``validity`` an optional LSB bitmap.
This is the layout the reference hands to its refiner through the Arrow C
data interface (c/sedona-libgpuspatial/src/libgpuspatial.rs:380-486).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

WKB_POINT = 1
WKB_LINESTRING = 2
WKB_POLYGON = 3
WKB_MULTIPOLYGON = 6


@dataclass
class WkbColumn:
    offsets: np.ndarray
    data: np.ndarray
    validity: Optional[np.ndarray] = None

    def __len__(self) -> int:
        return len(self.offsets) - 1

    @property
    def nbytes(self) -> int:
        n = self.offsets.nbytes + self.data.nbytes
        if self.validity is not None:
            n += self.validity.nbytes
        return n

    def value(self, i: int) -> bytes:
        return self.data[int(self.offsets[i]):int(self.offsets[i + 1])].tobytes()

    def is_valid(self, i: int) -> bool:
        if self.validity is None:
            return True
        return bool((self.validity[i >> 3] >> (i & 7)) & 1)

    def slice(self, start: int, stop: int) -> "WkbColumn":
        """Rows [start, stop) as a new column with offsets rebased to 0."""
        off = self.offsets[start:stop + 1]
        base = int(off[0])
        data = self.data[base:int(off[-1])]
        validity = None
        if self.validity is not None:
            bits = np.unpackbits(self.validity, bitorder="little")[start:stop]
            validity = np.packbits(bits, bitorder="little")
        return WkbColumn((off - base).astype(self.offsets.dtype), data, validity)

    def offsets64(self) -> np.ndarray:
        return self.offsets.astype(np.int64)

    def take(self, rows: np.ndarray) -> "WkbColumn":
        """The given rows (ascending or not) as a new column."""
        rows = np.asarray(rows, dtype=np.int64)
        off = self.offsets.astype(np.int64)
        starts, lens = off[rows], off[rows + 1] - off[rows]
        new_off = np.zeros(len(rows) + 1, dtype=np.int64)
        np.cumsum(lens, out=new_off[1:])
        total = int(new_off[-1])
        src = np.repeat(starts - new_off[:-1], lens) + np.arange(total, dtype=np.int64)
        data = self.data[src] if total else np.zeros(0, np.uint8)
        validity = None
        if self.validity is not None:
            bits = np.unpackbits(self.validity, bitorder="little")[rows]
            validity = np.packbits(bits, bitorder="little")
        dt = np.int64 if total >= 2**31 else self.offsets.dtype
        return WkbColumn(new_off.astype(dt), data, validity)


def _offsets_dtype(total: int, large: Optional[bool]) -> np.dtype:
    if large is None:
        large = total >= 2**31
    return np.dtype(np.int64 if large else np.int32)


_POINT_REC = np.dtype([("bo", "u1"), ("t", "<u4"), ("x", "<f8"), ("y", "<f8")])
assert _POINT_REC.itemsize == 21


def points_column(x: np.ndarray, y: np.ndarray, large: Optional[bool] = None) -> WkbColumn:
    """Little-endian WKB POINT per row (21 bytes each)."""
    n = len(x)
    rec = np.empty(n, dtype=_POINT_REC)
    rec["bo"] = 1
    rec["t"] = WKB_POINT
    rec["x"] = x
    rec["y"] = y
    data = rec.view(np.uint8).reshape(-1) if n else np.zeros(0, np.uint8)
    dt = _offsets_dtype(21 * n, large)
    offsets = (np.arange(n + 1, dtype=np.int64) * 21).astype(dt)
    return WkbColumn(offsets, data)


def polygons_column(npts: np.ndarray, xy: np.ndarray, large: Optional[bool] = None) -> WkbColumn:
    """Single-ring polygons.  ``npts[i]`` points per ring (ring already
    closed by the caller), ``xy`` the (sum(npts), 2) float64 vertices."""
    npts = np.asarray(npts, dtype=np.int64)
    n = len(npts)
    sizes = 13 + 16 * npts
    offsets = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(sizes, out=offsets[1:])
    total = int(offsets[-1])
    data = np.empty(total, dtype=np.uint8)
    if n:
        hdr = np.empty(n, dtype=[("bo", "u1"), ("t", "<u4"), ("nr", "<u4"), ("np", "<u4")])
        hdr["bo"] = 1
        hdr["t"] = WKB_POLYGON
        hdr["nr"] = 1
        hdr["np"] = npts
        # mark 13 header bytes per row without a (n, 13) index array
        marks = np.zeros(total + 1, dtype=np.int8)
        np.add.at(marks, offsets[:-1], 1)
        np.add.at(marks, offsets[:-1] + 13, -1)
        is_hdr = np.cumsum(marks[:-1]).astype(bool)
        data[is_hdr] = hdr.view(np.uint8)
        data[~is_hdr] = np.ascontiguousarray(xy, dtype="<f8").view(np.uint8).reshape(-1)
    return WkbColumn(offsets.astype(_offsets_dtype(total, large)), data)


# ---------------------------------------------------------------------------
# small hand-built geometries for tests

def wkb_point(x: float, y: float, big_endian: bool = False) -> bytes:
    if big_endian:
        return struct.pack(">BIdd", 0, WKB_POINT, x, y)
    return struct.pack("<BIdd", 1, WKB_POINT, x, y)


def _ring_bytes(ring: Sequence[Sequence[float]], e: str) -> bytes:
    out = [struct.pack(e + "I", len(ring))]
    for x, y in ring:
        out.append(struct.pack(e + "dd", x, y))
    return b"".join(out)


def wkb_polygon(rings: Sequence[Sequence[Sequence[float]]], big_endian: bool = False) -> bytes:
    e = ">" if big_endian else "<"
    out = [struct.pack(e + "BII", 0 if big_endian else 1, WKB_POLYGON, len(rings))]
    out += [_ring_bytes(r, e) for r in rings]
    return b"".join(out)


def wkb_multipolygon(polys: Sequence[Sequence[Sequence[Sequence[float]]]],
                     big_endian: bool = False) -> bytes:
    e = ">" if big_endian else "<"
    out = [struct.pack(e + "BII", 0 if big_endian else 1, WKB_MULTIPOLYGON, len(polys))]
    out += [wkb_polygon(p, big_endian) for p in polys]
    return b"".join(out)


def column_from_values(values: Sequence[Optional[bytes]], large: bool = False) -> WkbColumn:
    """Column from a list of WKB byte strings; None rows are null."""
    n = len(values)
    sizes = np.array([len(v) if v is not None else 0 for v in values], dtype=np.int64)
    offsets = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(sizes, out=offsets[1:])
    data = np.frombuffer(b"".join(v for v in values if v is not None), dtype=np.uint8).copy()
    validity = None
    if any(v is None for v in values):
        bits = np.array([v is not None for v in values], dtype=np.uint8)
        validity = np.packbits(bits, bitorder="little")
    return WkbColumn(offsets.astype(np.int64 if large else np.int32), data, validity)
