"""ctypes front end of the CPU oracle (libspj_oracle.so).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / reference legs — the checker, never the product.
``build()`` compiles the restatement with the Makefile beside this file; on a
machine where the reference tree is mounted it also compiles the reference's
own tg library into oracle/_ref/ (``ref_available()``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libspj_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libtgref.so")
# the reference tree (apache/sedona-db sources), where it is mounted: set by
# the caller (the build entry point or gen_golden.py); unset, only the
# restatement is built
REFERENCE_TREE = os.environ.get("SPJ_REFERENCE_TREE", "")

PRED = {"equals": 0, "disjoint": 1, "touches": 2, "contains": 3, "covers": 4,
        "intersects": 5, "within": 6, "coveredby": 7, "dwithin": 100}

_lib = None
_ref = None


def build(with_ref: Optional[bool] = None) -> None:
    targets = ["all"]
    if with_ref is None:
        with_ref = bool(REFERENCE_TREE) and os.path.isdir(
            os.path.join(REFERENCE_TREE, "c", "sedona-tg", "src", "tg"))
    if with_ref and not REFERENCE_TREE:
        raise RuntimeError("set SPJ_REFERENCE_TREE to the reference source tree to build oracle/_ref")
    if with_ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE, f"REFERENCE={REFERENCE_TREE}"] + targets,
                   check=True)


def _u8p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint8)) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        L = C.CDLL(LIB_PATH)
        L.spjo_parse.restype = C.c_void_p
        L.spjo_parse.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_uint8),
                                 C.POINTER(C.c_uint8), C.c_int64, C.c_char_p, C.c_int]
        L.spjo_free_geoms.argtypes = [C.c_void_p]
        L.spjo_count.restype = C.c_int64
        L.spjo_count.argtypes = [C.c_void_p]
        L.spjo_kind.argtypes = [C.c_void_p, C.c_int64]
        L.spjo_num_vertices.restype = C.c_int64
        L.spjo_num_vertices.argtypes = [C.c_void_p]
        L.spjo_boxes.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float)]
        L.spjo_point.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
        L.spjo_predicate.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int]
        L.spjo_raycast.argtypes = [C.c_double] * 6
        L.spjo_segment_intersects.argtypes = [C.c_double] * 8
        L.spjo_collinear.argtypes = [C.c_double] * 6
        L.spjo_rect_join.restype = C.c_int64
        L.spjo_rect_join.argtypes = [C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float),
                                     C.c_int64, C.c_int, C.POINTER(C.POINTER(C.c_uint32)),
                                     C.POINTER(C.POINTER(C.c_uint32))]
        L.spjo_join.restype = C.c_int64
        L.spjo_join.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int,
                                C.POINTER(C.POINTER(C.c_uint32)),
                                C.POINTER(C.POINTER(C.c_uint32)), C.c_char_p, C.c_int]
        L.spjo_join_dists.restype = C.c_int64
        L.spjo_join_dists.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_int,
                                      C.POINTER(C.POINTER(C.c_uint32)),
                                      C.POINTER(C.POINTER(C.c_uint32)), C.c_char_p, C.c_int]
        L.spjo_geo_distance.restype = C.c_double
        L.spjo_geo_distance.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]
        L.spjo_knn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                               C.POINTER(C.c_uint32), C.POINTER(C.c_double), C.c_char_p,
                               C.c_int]
        L.spjo_digest.restype = C.c_uint64
        L.spjo_digest.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_int64]
        L.spjo_free.argtypes = [C.c_void_p]
        L.spjo_parquet_read.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_int64),
                                        C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                        C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
        _lib = L
    return _lib


class Geoms:
    """A parsed WKB column held by the oracle."""

    def __init__(self, col):
        L = lib()
        self._keep = col
        off = np.ascontiguousarray(col.offsets, dtype=np.int64)
        self._off = off
        err = C.create_string_buffer(512)
        data = col.data if len(col.data) else np.zeros(1, np.uint8)
        self._data = data
        self.ptr = L.spjo_parse(off.ctypes.data_as(C.POINTER(C.c_int64)), _u8p(data),
                                _u8p(col.validity), len(col), err, 512)
        if not self.ptr:
            raise ValueError(err.value.decode())
        self.n = len(col)

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().spjo_free_geoms(self.ptr)
            self.ptr = None

    def kind(self, i: int) -> int:
        return lib().spjo_kind(self.ptr, i)

    def num_vertices(self) -> int:
        return lib().spjo_num_vertices(self.ptr)

    def boxes(self, mode: int = 1) -> np.ndarray:
        out = np.empty((self.n, 4), dtype=np.float32)
        lib().spjo_boxes(self.ptr, mode, out.ctypes.data_as(C.POINTER(C.c_float)))
        return out


def _take_pairs(n, pb, pp) -> Tuple[np.ndarray, np.ndarray]:
    L = lib()
    if n < 0:
        raise RuntimeError("oracle join failed")
    b = np.ctypeslib.as_array(pb, shape=(max(n, 1),))[:n].copy()
    p = np.ctypeslib.as_array(pp, shape=(max(n, 1),))[:n].copy()
    L.spjo_free(C.cast(pb, C.c_void_p))
    L.spjo_free(C.cast(pp, C.c_void_p))
    return b, p


def rect_join(build_rects: np.ndarray, probe_rects: np.ndarray, nthreads: int = 1):
    """Candidate pairs of two f32 rect arrays (closed intervals), sorted by (probe, build)."""
    L = lib()
    br = np.ascontiguousarray(build_rects, dtype=np.float32)
    pr = np.ascontiguousarray(probe_rects, dtype=np.float32)
    pb, pp = C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)()
    n = L.spjo_rect_join(br.ctypes.data_as(C.POINTER(C.c_float)), len(br),
                         pr.ctypes.data_as(C.POINTER(C.c_float)), len(pr), nthreads,
                         C.byref(pb), C.byref(pp))
    return _take_pairs(n, pb, pp)


def join(build: Geoms, probe: Geoms, predicate: str, distance: float = 0.0,
         nthreads: int = 1):
    """Refined pairs (build_idx, probe_idx) sorted by (probe, build)."""
    L = lib()
    pb, pp = C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)()
    err = C.create_string_buffer(512)
    n = L.spjo_join(build.ptr, probe.ptr, PRED[predicate], distance, nthreads, C.byref(pb),
                    C.byref(pp), err, 512)
    if n < 0:
        raise RuntimeError(err.value.decode())
    return _take_pairs(n, pb, pp)


def join_dists(build: Geoms, probe: Geoms, dists: np.ndarray, nthreads: int = 1):
    """ST_DWithin pairs with one distance per probe row, sorted by (probe, build)."""
    L = lib()
    d = np.ascontiguousarray(dists, dtype=np.float64)
    assert len(d) == probe.n
    pb, pp = C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)()
    err = C.create_string_buffer(512)
    n = L.spjo_join_dists(build.ptr, probe.ptr, d.ctypes.data_as(C.POINTER(C.c_double)),
                          nthreads, C.byref(pb), C.byref(pp), err, 512)
    if n < 0:
        raise RuntimeError(err.value.decode())
    return _take_pairs(n, pb, pp)


def geo_distance(build: Geoms, bi: int, probe: Geoms, pi: int) -> float:
    return lib().spjo_geo_distance(build.ptr, bi, probe.ptr, pi)


def knn(build: Geoms, probe: Geoms, k: int, nthreads: int = 1):
    """(build_idx[n_probe, k], dist[n_probe, k]); unused slots are 0xFFFFFFFF / inf."""
    L = lib()
    ob = np.empty((probe.n, k), dtype=np.uint32)
    od = np.empty((probe.n, k), dtype=np.float64)
    err = C.create_string_buffer(512)
    r = L.spjo_knn(build.ptr, probe.ptr, k, nthreads, ob.ctypes.data_as(C.POINTER(C.c_uint32)),
                   od.ctypes.data_as(C.POINTER(C.c_double)), err, 512)
    if r:
        raise RuntimeError(err.value.decode())
    return ob, od


def predicate(build: Geoms, bi: int, probe: Geoms, pi: int, pred: str) -> int:
    return lib().spjo_predicate(build.ptr, bi, probe.ptr, pi, PRED[pred])


def raycast(ax, ay, bx, by, px, py) -> int:
    return lib().spjo_raycast(ax, ay, bx, by, px, py)


def segment_intersects(ax, ay, bx, by, cx, cy, dx, dy) -> int:
    return lib().spjo_segment_intersects(ax, ay, bx, by, cx, cy, dx, dy)


def collinear(x1, y1, x2, y2, x3, y3) -> int:
    return lib().spjo_collinear(x1, y1, x2, y2, x3, y3)


def digest(build_idx: np.ndarray, probe_idx: np.ndarray) -> int:
    b = np.ascontiguousarray(build_idx, dtype=np.uint32)
    p = np.ascontiguousarray(probe_idx, dtype=np.uint32)
    return int(lib().spjo_digest(b.ctypes.data_as(C.POINTER(C.c_uint32)),
                                 p.ctypes.data_as(C.POINTER(C.c_uint32)), len(b)))


# ---------------------------------------------------------------------------
# the reference's own tg, compiled from the reference tree (this container only)

def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.tgref_pred.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, C.c_int, C.c_int]
        R.tgref_raycast.argtypes = [C.c_double] * 6
        R.tgref_segment_intersects.argtypes = [C.c_double] * 8
        _ref = R
    return _ref


def ref_predicate(build_wkb: bytes, probe_wkb: bytes, pred: str, index: int = 3) -> int:
    return ref().tgref_pred(build_wkb, len(build_wkb), probe_wkb, len(probe_wkb), PRED[pred],
                            index)


def parquet_read(path: str, column: Optional[str] = None):
    """A GeoParquet BYTE_ARRAY column read on the CPU (spj_parquet.c):
    (int64 offsets with nulls empty, uint8 data, bool valid)."""
    L = lib()
    n = C.c_int64()
    po, pd, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    err = C.create_string_buffer(512)
    rc = L.spjo_parquet_read(path.encode(), column.encode() if column else None, C.byref(n),
                             C.byref(po), C.byref(pd), C.byref(pv), err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())
    try:
        rows = n.value
        off = np.ctypeslib.as_array(C.cast(po, C.POINTER(C.c_int64)), shape=(rows + 1,)).copy()
        nbytes = int(off[-1])
        data = (np.ctypeslib.as_array(C.cast(pd, C.POINTER(C.c_uint8)), shape=(nbytes,)).copy()
                if nbytes else np.zeros(0, np.uint8))
        valid = (np.ctypeslib.as_array(C.cast(pv, C.POINTER(C.c_uint8)), shape=(rows,)).copy()
                 .astype(bool) if rows else np.zeros(0, bool))
    finally:
        L.spjo_free(po)
        L.spjo_free(pd)
        L.spjo_free(pv)
    return off, data, valid
