"""GeoParquet WKB columns read onto the device (SpjParquet*, include/spj_gb300.h).

The reference reads GeoParquet with arrow-rs on the CPU
(rust/sedona-geoparquet/src/file_opener.rs, format.rs) and parses the WKB
again on the CPU before the join.  ``GeoParquetFile.read_wkb`` instead
copies the column chunks to HBM once and decompresses and decodes their pages
there; the result is a device column (``SpjDeviceWkb``) that the join, the
learned index and the KNN join take as is.

``write_wkb`` writes a GeoParquet file from a host ``WkbColumn`` (PLAIN
pages, SNAPPY or stored, data page v1 or v2), for inputs on machines without
a Parquet library.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np

from .capi import GpuSpatialError, SpjDeviceWkb, SpjParquetWriteOptions, lib
from .wkb import WkbColumn


def _open_error() -> str:
    return lib().SpjParquetLastError(None).decode(errors="replace")


class GeoParquetFile:
    """An open GeoParquet file: metadata on the host, WKB columns read to
    the device."""

    def __init__(self, path: str):
        self.h = C.c_void_p()
        if lib().SpjParquetOpen(path.encode(), C.byref(self.h)) != 0:
            self.h = None
            raise GpuSpatialError(f"open {path}: {_open_error()}")
        self.path = path

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = lib().SpjParquetLastError(self.h).decode(errors="replace")
            raise GpuSpatialError(f"{what}: {msg}")

    def info(self) -> dict:
        rows, rgs, cols = C.c_int64(), C.c_int32(), C.c_int32()
        self._check(lib().SpjParquetInfo(self.h, C.byref(rows), C.byref(rgs), C.byref(cols)),
                    "info")
        return {"num_rows": rows.value, "num_row_groups": rgs.value, "num_columns": cols.value}

    def column_names(self) -> List[str]:
        out = []
        for i in range(self.info()["num_columns"]):
            buf = C.create_string_buffer(4096)
            self._check(lib().SpjParquetColumnName(self.h, i, buf, len(buf)), "column name")
            out.append(buf.value.decode())
        return out

    def primary_column(self) -> Optional[str]:
        buf = C.create_string_buffer(4096)
        if lib().SpjParquetColumnName(self.h, -1, buf, len(buf)) != 0:
            return None
        return buf.value.decode()

    def row_group_rows(self, rg: int) -> int:
        n = C.c_int64()
        self._check(lib().SpjParquetRowGroupRows(self.h, rg, C.byref(n)), "row group rows")
        return n.value

    def read_wkb(self, column: Optional[str] = None, rg_begin: int = 0, rg_end: int = -1,
                 device: int = 0) -> SpjDeviceWkb:
        """The column's rows in [rg_begin, rg_end) as a device large_binary
        column, valid until the next read or until this file is closed."""
        out = SpjDeviceWkb()
        self._check(lib().SpjParquetReadWkb(self.h, column.encode() if column else None,
                                            rg_begin, rg_end, device, C.byref(out)), "read_wkb")
        return out

    def stats(self) -> dict:
        ms = C.c_double()
        v = [C.c_uint64() for _ in range(3)]
        self._check(lib().SpjParquetGetStats(self.h, C.byref(ms), *[C.byref(x) for x in v]),
                    "stats")
        return {"ms_device": ms.value, "file_bytes": v[0].value, "page_bytes": v[1].value,
                "value_bytes": v[2].value}

    def phases(self) -> dict:
        v = [C.c_double() for _ in range(4)]
        self._check(lib().SpjParquetGetPhases(self.h, *[C.byref(x) for x in v]), "phases")
        return dict(zip(("h2d", "decompress", "decode", "values"), (x.value for x in v)))

    def close(self):
        if getattr(self, "h", None):
            lib().SpjParquetRelease(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()


def write_wkb(path: str, col: WkbColumn, column: str = "geometry", compression: str = "snappy",
              page_version: int = 1, row_group_rows: int = 0, page_bytes: int = 0):
    """Writes ``col`` as a GeoParquet file with one WKB column."""
    codecs = {"none": 0, "uncompressed": 0, "snappy": 1}
    if compression not in codecs:
        raise GpuSpatialError(f"compression must be one of {sorted(codecs)}")
    opt = SpjParquetWriteOptions(codecs[compression], page_version, row_group_rows, page_bytes)
    off = np.ascontiguousarray(col.offsets)
    data = np.ascontiguousarray(col.data) if len(col.data) else np.zeros(1, np.uint8)
    val = np.ascontiguousarray(col.validity) if col.validity is not None else None
    rc = lib().SpjParquetWriteWkb(path.encode(), column.encode(), len(col), off.ctypes.data,
                                  int(off.dtype == np.int64), data.ctypes.data,
                                  val.ctypes.data if val is not None else None, 0, C.byref(opt))
    if rc != 0:
        raise GpuSpatialError(f"write {path}: {_open_error()}")


def device_to_host(d: SpjDeviceWkb) -> WkbColumn:
    """Copies a device column back (int64 offsets, data, validity or None)."""
    import torch

    class _Dev:
        def __init__(self, ptr, n, typestr):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                             "data": (ptr, False), "version": 3,
                                             "strides": None}

    n = int(d.length)
    torch.cuda.synchronize()
    off = torch.as_tensor(_Dev(d.offsets, n + 1, "<i8"), device="cuda").cpu().numpy()
    nbytes = int(d.data_length)
    data = (torch.as_tensor(_Dev(d.data, nbytes, "|u1"), device="cuda").cpu().numpy()
            if nbytes else np.zeros(0, np.uint8))
    validity = None
    if d.validity:
        validity = torch.as_tensor(_Dev(d.validity, (n + 7) // 8, "|u1"),
                                   device="cuda").cpu().numpy()
    return WkbColumn(off.astype(np.int64), data, validity)
