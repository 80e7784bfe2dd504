"""ctypes bindings of the C ABI (include/gpuspatial_c.h, include/spj_gb300.h).

The classes mirror the reference's safe Rust wrapper over the same ABI
(c/sedona-libgpuspatial/src/libgpuspatial.rs and src/lib.rs): a
process-global runtime, ``FloatIndex2D`` (push_build / finish_building /
probe returning (build, probe) candidate index arrays) and ``Refiner``
(init_build_schema / push_build / finish_building / refine), with errors
surfaced as ``GpuSpatialError`` carrying the library's last-error message.
There is no CPU fallback: if the CUDA library is missing the import fails.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from typing import Callable, Optional, Tuple

import numpy as np

from .wkb import WkbColumn

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libspj_gb300.so")


class GpuSpatialError(RuntimeError):
    pass


# ---------------------------------------------------------------------------
# ABI structs

class GpuSpatialRuntimeConfig(C.Structure):
    _fields_ = [("ptx_root", C.c_char_p), ("device_id", C.c_int),
                ("use_cuda_memory_pool", C.c_bool), ("cuda_memory_pool_init_precent", C.c_int)]


class GpuSpatialRuntime(C.Structure):
    pass


GpuSpatialRuntime._fields_ = [
    ("init", C.CFUNCTYPE(C.c_int, C.POINTER(GpuSpatialRuntime), C.POINTER(GpuSpatialRuntimeConfig))),
    ("release", C.CFUNCTYPE(None, C.POINTER(GpuSpatialRuntime))),
    ("get_last_error", C.CFUNCTYPE(C.c_char_p, C.POINTER(GpuSpatialRuntime))),
    ("private_data", C.c_void_p)]


class GpuSpatialIndexConfig(C.Structure):
    _fields_ = [("runtime", C.POINTER(GpuSpatialRuntime)), ("concurrency", C.c_uint32)]


class SedonaSpatialIndexContext(C.Structure):
    _fields_ = [("private_data", C.c_void_p)]


PROBE_CB = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint32,
                       C.c_void_p)


class SedonaFloatIndex2D(C.Structure):
    pass


_IDX = C.POINTER(SedonaFloatIndex2D)
_CTX = C.POINTER(SedonaSpatialIndexContext)
SedonaFloatIndex2D._fields_ = [
    ("clear", C.CFUNCTYPE(C.c_int, _IDX)),
    ("create_context", C.CFUNCTYPE(None, _CTX)),
    ("destroy_context", C.CFUNCTYPE(None, _CTX)),
    ("push_build", C.CFUNCTYPE(C.c_int, _IDX, C.POINTER(C.c_float), C.c_uint32)),
    ("finish_building", C.CFUNCTYPE(C.c_int, _IDX)),
    ("probe", C.CFUNCTYPE(C.c_int, _IDX, _CTX, C.POINTER(C.c_float), C.c_uint32, PROBE_CB,
                          C.c_void_p)),
    ("get_last_error", C.CFUNCTYPE(C.c_char_p, _IDX)),
    ("context_get_last_error", C.CFUNCTYPE(C.c_char_p, _CTX)),
    ("release", C.CFUNCTYPE(None, _IDX)),
    ("private_data", C.c_void_p)]


class GpuSpatialRefinerConfig(C.Structure):
    _fields_ = [("runtime", C.POINTER(GpuSpatialRuntime)), ("concurrency", C.c_uint32),
                ("compress_bvh", C.c_bool), ("pipeline_batches", C.c_uint32)]


class ArrowSchema(C.Structure):
    pass


ArrowSchema._fields_ = [
    ("format", C.c_char_p), ("name", C.c_char_p), ("metadata", C.c_char_p), ("flags", C.c_int64),
    ("n_children", C.c_int64), ("children", C.c_void_p), ("dictionary", C.c_void_p),
    ("release", C.c_void_p), ("private_data", C.c_void_p)]


class ArrowArray(C.Structure):
    _fields_ = [
        ("length", C.c_int64), ("null_count", C.c_int64), ("offset", C.c_int64),
        ("n_buffers", C.c_int64), ("n_children", C.c_int64),
        ("buffers", C.POINTER(C.c_void_p)), ("children", C.c_void_p), ("dictionary", C.c_void_p),
        ("release", C.c_void_p), ("private_data", C.c_void_p)]


class SedonaSpatialRefiner(C.Structure):
    pass


_REF = C.POINTER(SedonaSpatialRefiner)
SedonaSpatialRefiner._fields_ = [
    ("clear", C.CFUNCTYPE(C.c_int, _REF)),
    ("init_build_schema", C.CFUNCTYPE(C.c_int, _REF, C.POINTER(ArrowSchema))),
    ("push_build", C.CFUNCTYPE(C.c_int, _REF, C.POINTER(ArrowArray))),
    ("finish_building", C.CFUNCTYPE(C.c_int, _REF)),
    ("refine", C.CFUNCTYPE(C.c_int, _REF, C.POINTER(ArrowSchema), C.POINTER(ArrowArray), C.c_int,
                           C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint32,
                           C.POINTER(C.c_uint32))),
    ("get_last_error", C.CFUNCTYPE(C.c_char_p, _REF)),
    ("release", C.CFUNCTYPE(None, _REF)),
    ("private_data", C.c_void_p)]


class SpjJoinConfig(C.Structure):
    _fields_ = [("runtime", C.POINTER(GpuSpatialRuntime)), ("leaf_size", C.c_uint32),
                ("refine_form", C.c_int32), ("profile", C.c_int32), ("probe_order", C.c_int32)]


class SpjDeviceWkb(C.Structure):
    _fields_ = [("length", C.c_int64), ("offsets", C.c_void_p), ("offsets_are_64bit", C.c_int32),
                ("data", C.c_void_p), ("data_length", C.c_uint64), ("validity", C.c_void_p),
                ("validity_offset", C.c_int64)]


class SpjJoinStats(C.Structure):
    _fields_ = [("ms_decode", C.c_double), ("ms_filter", C.c_double), ("ms_refine", C.c_double),
                ("ms_compact", C.c_double), ("calls", C.c_uint64), ("probe_rows", C.c_uint64),
                ("candidates", C.c_uint64), ("results", C.c_uint64),
                ("escalations", C.c_uint64), ("pairs_evaluated", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("probe_bytes", C.c_uint64),
                ("build_rows", C.c_uint64), ("build_vertices", C.c_uint64),
                ("build_device_bytes", C.c_uint64)]


class SpjKnnConfig(C.Structure):
    _fields_ = [("runtime", C.POINTER(GpuSpatialRuntime)), ("leaf_size", C.c_uint32),
                ("refine_form", C.c_int32)]


JOIN_CB = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint64,
                      C.c_void_p)

class SpjHostWkb(C.Structure):
    _fields_ = [("length", C.c_int64), ("offsets", C.c_void_p), ("offsets_are_64bit", C.c_int32),
                ("data", C.c_void_p), ("validity", C.c_void_p), ("validity_offset", C.c_int64)]


class SpjPartitionOptions(C.Structure):
    _fields_ = [("num_partitions", C.c_uint32), ("sample_rows", C.c_uint32),
                ("build_budget_bytes", C.c_uint64), ("seed", C.c_uint64),
                ("host_gather", C.c_int32), ("record_layout", C.c_int32)]


class SpjPartitionStats(C.Structure):
    _fields_ = [("partitions", C.c_uint32), ("passes", C.c_uint32),
                ("build_rows_max", C.c_uint64), ("probe_rows_multi", C.c_uint64),
                ("probe_rows_none", C.c_uint64), ("probe_rows_probed", C.c_uint64),
                ("pairs", C.c_uint64), ("ms_boxes", C.c_double), ("ms_partition", C.c_double),
                ("ms_passes", C.c_double), ("direct_host_reads", C.c_int32)]


class SpjParquetWriteOptions(C.Structure):
    _fields_ = [("compression", C.c_int32), ("page_version", C.c_int32),
                ("row_group_rows", C.c_int64), ("page_bytes", C.c_int64)]


# exported symbols, declared in include/*.h
EXPORTS = [
    "GpuSpatialRuntimeCreate", "GpuSpatialIndexFloat2DCreate", "GpuSpatialRefinerCreate",
    "SpjJoinCreate", "SpjJoinRelease", "SpjJoinLastError", "SpjJoinSetOption",
    "SpjJoinPushBuildArrow",
    "SpjJoinFinishBuild", "SpjJoinBuildDevice", "SpjJoinProbeArrow", "SpjJoinProbeDevice",
    "SpjJoinProbeHost", "SpjJoinStream", "SpjJoinGetStats", "SpjJoinResetStats",
    "SpjKnnCreate", "SpjKnnRelease", "SpjKnnLastError", "SpjKnnBuild", "SpjKnnQuery",
    "SpjKnnQueryTies", "SpjKnnQueryArrow", "SpjJoinSetProbeDistances",
    "SpjKnnStream", "SpjKnnGetStats", "SpjHostRegister", "SpjHostUnregister", "SpjVersion",
    "SpjIndexProbeNoAlloc", "SpjAllocationCount",
    "SpjMaterializeLastError", "SpjGatherFixed", "SpjGatherValidity", "SpjGatherBinary",
    "SpjVisitedMark", "SpjVisitedCollect",
    "SpjJoinPartitioned", "SpjJoinPartitionLayout",
    "SpjParquetOpen", "SpjParquetRelease", "SpjParquetLastError", "SpjParquetInfo",
    "SpjParquetColumnName", "SpjParquetRowGroupRows", "SpjParquetReadWkb", "SpjParquetGetStats", "SpjParquetGetPhases",
    "SpjParquetWriteWkb",
    "SpjStreamCreate", "SpjStreamRelease", "SpjStreamLastError", "SpjStreamSetBatches",
    "SpjStreamRun", "SpjStreamSetParams", "SpjStreamAutotune", "SpjStreamGetStats",
    "SpjStreamCudaStream",
    "SpjLearnedCreate", "SpjLearnedRelease", "SpjLearnedLastError", "SpjLearnedBuildDevice",
    "SpjLearnedSetTrained", "SpjLearnedQueryDevice", "SpjLearnedLossAndGrad", "SpjLearnedExport",
    "SpjLearnedGetStats", "SpjLearnedStream", "SpjLearnedSetWindow", "SpjLearnedAutotuneWindow",
]


class SpjLearnedConfig(C.Structure):
    _fields_ = [("runtime", C.POINTER(GpuSpatialRuntime)), ("leaves", C.c_uint32),
                ("window", C.c_uint32)]


class SpjLearnedStats(C.Structure):
    _fields_ = [("points", C.c_uint64), ("lookups", C.c_uint64), ("window_misses", C.c_uint64),
                ("lbvh_fallbacks", C.c_uint64), ("search_steps", C.c_uint64),
                ("leaves", C.c_uint32), ("max_err", C.c_uint32),
                ("leaves_over_window", C.c_uint32), ("trained", C.c_uint32),
                ("root_shift", C.c_double), ("root_entries", C.c_double),
                ("mean_err", C.c_double),
                ("grad_norm_after", C.c_double), ("ms_build", C.c_double),
                ("ranges", C.c_uint64), ("ms_order", C.c_double), ("ms_ranges", C.c_double),
                ("ms_eval", C.c_double), ("window", C.c_uint32), ("window_box", C.c_uint32),
                ("kernel_launches", C.c_uint64)]

_lib = None
_lib_lock = threading.Lock()


def lib() -> C.CDLL:
    """Loads lib/libspj_gb300.so (raises if it was not built)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise GpuSpatialError(
                    f"CUDA library not built: {LIB_PATH} (run __graft_entry__.build())")
            L = C.CDLL(LIB_PATH)
            L.GpuSpatialRuntimeCreate.argtypes = [C.POINTER(GpuSpatialRuntime)]
            L.GpuSpatialRuntimeCreate.restype = None
            L.GpuSpatialIndexFloat2DCreate.argtypes = [_IDX, C.POINTER(GpuSpatialIndexConfig)]
            L.GpuSpatialRefinerCreate.argtypes = [_REF, C.POINTER(GpuSpatialRefinerConfig)]
            L.SpjJoinCreate.argtypes = [C.POINTER(SpjJoinConfig), C.POINTER(C.c_void_p)]
            L.SpjJoinSetOption.argtypes = [C.c_void_p, C.c_char_p, C.c_int64]
            L.SpjJoinRelease.argtypes = [C.c_void_p]
            L.SpjJoinRelease.restype = None
            L.SpjJoinLastError.argtypes = [C.c_void_p]
            L.SpjJoinLastError.restype = C.c_char_p
            L.SpjJoinPushBuildArrow.argtypes = [C.c_void_p, C.POINTER(ArrowSchema),
                                                C.POINTER(ArrowArray)]
            L.SpjJoinFinishBuild.argtypes = [C.c_void_p]
            L.SpjJoinBuildDevice.argtypes = [C.c_void_p, C.POINTER(SpjDeviceWkb)]
            L.SpjJoinProbeArrow.argtypes = [C.c_void_p, C.POINTER(ArrowSchema),
                                            C.POINTER(ArrowArray), C.c_int32, C.c_double,
                                            C.c_uint32, JOIN_CB, C.c_void_p]
            L.SpjJoinProbeDevice.argtypes = [C.c_void_p, C.POINTER(SpjDeviceWkb), C.c_int32,
                                             C.c_double, C.c_uint32,
                                             C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                             C.POINTER(C.c_uint64)]
            L.SpjJoinProbeHost.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int32,
                                           C.c_void_p, C.c_void_p, C.c_int32, C.c_double,
                                           C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint64,
                                           C.POINTER(C.c_uint64)]
            L.SpjJoinStream.argtypes = [C.c_void_p]
            L.SpjJoinStream.restype = C.c_void_p
            L.SpjJoinGetStats.argtypes = [C.c_void_p, C.POINTER(SpjJoinStats)]
            L.SpjJoinResetStats.argtypes = [C.c_void_p]
            L.SpjKnnCreate.argtypes = [C.POINTER(SpjKnnConfig), C.POINTER(C.c_void_p)]
            L.SpjKnnRelease.argtypes = [C.c_void_p]
            L.SpjKnnRelease.restype = None
            L.SpjKnnLastError.argtypes = [C.c_void_p]
            L.SpjKnnLastError.restype = C.c_char_p
            L.SpjKnnBuild.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
            L.SpjKnnGetStats.argtypes = [C.c_void_p] + [C.POINTER(C.c_uint64)] * 3
            L.SpjKnnQuery.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32,
                                      C.c_void_p, C.c_void_p, C.c_int32]
            L.SpjKnnStream.argtypes = [C.c_void_p]
            L.SpjKnnStream.restype = C.c_void_p
            L.SpjJoinSetProbeDistances.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64,
                                                   C.c_int32]
            L.SpjKnnQueryTies.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32,
                                          C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
            L.SpjKnnQueryArrow.argtypes = [C.c_void_p, C.POINTER(ArrowSchema),
                                           C.POINTER(ArrowArray), C.c_uint32, C.c_int32,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                           C.POINTER(C.c_uint64)]
            L.SpjMaterializeLastError.argtypes = []
            L.SpjMaterializeLastError.restype = C.c_char_p
            L.SpjGatherFixed.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_void_p,
                                         C.c_uint64, C.c_void_p, C.c_void_p]
            L.SpjGatherValidity.argtypes = [C.c_void_p, C.c_int64, C.c_uint64, C.c_void_p,
                                            C.c_uint64, C.c_void_p, C.POINTER(C.c_uint64),
                                            C.c_void_p]
            L.SpjGatherBinary.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_uint64,
                                          C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                          C.c_uint64, C.POINTER(C.c_uint64), C.c_void_p]
            L.SpjVisitedMark.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                         C.c_void_p]
            L.SpjVisitedCollect.argtypes = [C.c_void_p, C.c_uint64, C.c_int32, C.c_void_p,
                                            C.c_uint64, C.POINTER(C.c_uint64), C.c_void_p]
            L.SpjJoinPartitioned.argtypes = [C.c_void_p, C.POINTER(SpjHostWkb),
                                             C.POINTER(SpjHostWkb), C.c_int32, C.c_double,
                                             C.POINTER(SpjPartitionOptions), JOIN_CB,
                                             C.c_void_p, C.POINTER(SpjPartitionStats)]
            L.SpjJoinPartitionLayout.argtypes = [C.c_void_p] + [C.c_void_p] * 7
            L.SpjParquetOpen.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
            L.SpjParquetRelease.argtypes = [C.c_void_p]
            L.SpjParquetRelease.restype = None
            L.SpjParquetLastError.argtypes = [C.c_void_p]
            L.SpjParquetLastError.restype = C.c_char_p
            L.SpjParquetInfo.argtypes = [C.c_void_p, C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
            L.SpjParquetColumnName.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_uint64]
            L.SpjParquetRowGroupRows.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]
            L.SpjParquetReadWkb.argtypes = [C.c_void_p, C.c_char_p, C.c_int32, C.c_int32,
                                            C.c_int32, C.POINTER(SpjDeviceWkb)]
            L.SpjParquetGetStats.argtypes = [C.c_void_p, C.POINTER(C.c_double)] + \
                [C.POINTER(C.c_uint64)] * 3
            L.SpjParquetGetPhases.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 4
            L.SpjParquetWriteWkb.argtypes = [C.c_char_p, C.c_char_p, C.c_int64, C.c_void_p,
                                             C.c_int32, C.c_void_p, C.c_void_p, C.c_int64,
                                             C.POINTER(SpjParquetWriteOptions)]
            L.SpjAllocationCount.argtypes = []
            L.SpjAllocationCount.restype = C.c_uint64
            L.SpjHostRegister.argtypes = [C.c_void_p, C.c_uint64]
            L.SpjHostUnregister.argtypes = [C.c_void_p]
            L.SpjVersion.restype = C.c_char_p
            L.SpjStreamCreate.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
            L.SpjStreamRelease.argtypes = [C.c_void_p]
            L.SpjStreamRelease.restype = None
            L.SpjStreamLastError.argtypes = [C.c_void_p]
            L.SpjStreamLastError.restype = C.c_char_p
            L.SpjStreamSetBatches.argtypes = [C.c_void_p, C.POINTER(SpjDeviceWkb), C.c_int32]
            L.SpjStreamRun.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p),
                                       C.POINTER(C.c_void_p), C.POINTER(C.c_uint64)]
            L.SpjStreamSetParams.argtypes = [C.c_void_p, C.c_int32, C.c_uint32, C.c_uint32]
            L.SpjStreamAutotune.argtypes = [C.c_void_p, C.c_int32, C.c_char_p,
                                            C.POINTER(C.c_int32), C.POINTER(C.c_uint32),
                                            C.POINTER(C.c_uint32)]
            L.SpjStreamGetStats.argtypes = [C.c_void_p, C.POINTER(C.c_double),
                                            C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
            L.SpjStreamCudaStream.argtypes = [C.c_void_p]
            L.SpjStreamCudaStream.restype = C.c_void_p
            L.SpjLearnedCreate.argtypes = [C.POINTER(SpjLearnedConfig), C.POINTER(C.c_void_p)]
            L.SpjLearnedRelease.argtypes = [C.c_void_p]
            L.SpjLearnedRelease.restype = None
            L.SpjLearnedLastError.argtypes = [C.c_void_p]
            L.SpjLearnedLastError.restype = C.c_char_p
            L.SpjLearnedBuildDevice.argtypes = [C.c_void_p, C.POINTER(SpjDeviceWkb)]
            L.SpjLearnedSetTrained.argtypes = [C.c_void_p, C.c_int32]
            L.SpjLearnedQueryDevice.argtypes = [C.c_void_p, C.POINTER(SpjDeviceWkb), C.c_int32,
                                                C.c_uint32, C.POINTER(C.c_void_p),
                                                C.POINTER(C.c_void_p), C.POINTER(C.c_uint64)]
            L.SpjLearnedLossAndGrad.argtypes = [C.c_void_p] + [C.c_void_p] * 5
            L.SpjLearnedExport.argtypes = [C.c_void_p] + [C.c_void_p] * 6
            L.SpjLearnedGetStats.argtypes = [C.c_void_p, C.POINTER(SpjLearnedStats)]
            L.SpjLearnedStream.argtypes = [C.c_void_p]
            L.SpjLearnedStream.restype = C.c_void_p
            L.SpjLearnedSetWindow.argtypes = [C.c_void_p, C.c_uint32]
            L.SpjLearnedAutotuneWindow.argtypes = [C.c_void_p, C.POINTER(SpjDeviceWkb),
                                                   C.c_uint32, C.c_int32,
                                                   C.POINTER(C.c_uint32)]
            _lib = L
    return _lib


# ---------------------------------------------------------------------------
# Arrow C data interface for binary WKB columns built from numpy buffers

class ArrowBinary:
    """Keeps an ArrowSchema / ArrowArray pair (binary or large_binary) alive."""

    def __init__(self, col: WkbColumn, offset: int = 0, length: Optional[int] = None):
        large = col.offsets.dtype == np.int64
        self._fmt = b"Z" if large else b"z"
        self.schema = ArrowSchema(format=self._fmt, name=b"geometry", metadata=None, flags=2,
                                  n_children=0)
        self._off = np.ascontiguousarray(col.offsets)
        self._data = np.ascontiguousarray(col.data) if len(col.data) else np.zeros(8, np.uint8)
        self._valid = col.validity
        self._bufs = (C.c_void_p * 3)(
            self._valid.ctypes.data if self._valid is not None else None,
            self._off.ctypes.data, self._data.ctypes.data)
        n = (len(col) - offset) if length is None else length
        nulls = 0
        if self._valid is not None:
            bits = np.unpackbits(self._valid, bitorder="little")[offset:offset + n]
            nulls = int(n - bits.sum())
        self.array = ArrowArray(length=n, null_count=nulls, offset=offset, n_buffers=3,
                                n_children=0, buffers=self._bufs)


# ---------------------------------------------------------------------------

class Runtime:
    """The process-global runtime (c/sedona-libgpuspatial/src/lib.rs:41-90)."""

    _instance = None
    _lock = threading.Lock()

    def __init__(self, device_id: int = 0, use_pool: bool = True, pool_percent: int = 0):
        L = lib()
        self.rt = GpuSpatialRuntime()
        L.GpuSpatialRuntimeCreate(C.byref(self.rt))
        cfg = GpuSpatialRuntimeConfig(b"", device_id, use_pool, pool_percent)
        if self.rt.init(C.byref(self.rt), C.byref(cfg)) != 0:
            msg = self.rt.get_last_error(C.byref(self.rt)).decode()
            raise GpuSpatialError(f"runtime init failed: {msg}")
        self.device_id = device_id

    @classmethod
    def get(cls, device_id: int = 0) -> "Runtime":
        with cls._lock:
            if cls._instance is None:
                cls._instance = Runtime(device_id)
            return cls._instance


def _check(rc: int, what: str, msg_fn: Callable[[], bytes]):
    if rc != 0:
        raise GpuSpatialError(f"{what}: {msg_fn().decode(errors='replace')}")


class FloatIndex2D:
    """SedonaFloatIndex2D (c/sedona-libgpuspatial/src/libgpuspatial.rs:126-308)."""

    def __init__(self, runtime: Optional[Runtime] = None, concurrency: int = 1):
        self.runtime = runtime or Runtime.get()
        self.idx = SedonaFloatIndex2D()
        cfg = GpuSpatialIndexConfig(C.pointer(self.runtime.rt), concurrency)
        if lib().GpuSpatialIndexFloat2DCreate(C.byref(self.idx), C.byref(cfg)) != 0:
            raise GpuSpatialError("Index Create failed")

    def _err(self):
        return self.idx.get_last_error(C.byref(self.idx))

    def clear(self):
        _check(self.idx.clear(C.byref(self.idx)), "clear", self._err)

    def push_build(self, rects: np.ndarray):
        r = np.ascontiguousarray(rects, dtype=np.float32).reshape(-1, 4)
        self._keep = r
        _check(self.idx.push_build(C.byref(self.idx), r.ctypes.data_as(C.POINTER(C.c_float)),
                                   len(r)), "push_build", self._err)

    def finish_building(self):
        _check(self.idx.finish_building(C.byref(self.idx)), "finish_building", self._err)

    def probe(self, rects: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
        r = np.ascontiguousarray(rects, dtype=np.float32).reshape(-1, 4)
        ctx = SedonaSpatialIndexContext()
        self.idx.create_context(C.byref(ctx))
        out = {}

        def cb(b, p, n, _ud):
            try:
                out["b"] = np.ctypeslib.as_array(b, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
                out["p"] = np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
                return 0
            except Exception as e:  # panic-safe callback (libgpuspatial.rs:532-572)
                out["err"] = e
                return -1

        ccb = PROBE_CB(cb)
        try:
            rc = self.idx.probe(C.byref(self.idx), C.byref(ctx),
                                r.ctypes.data_as(C.POINTER(C.c_float)), len(r), ccb, None)
            if rc != 0:
                if "err" in out:
                    raise GpuSpatialError(f"probe callback failed: {out['err']}")
                msg = self.idx.context_get_last_error(C.byref(ctx)).decode()
                raise GpuSpatialError(f"probe: {msg}")
        finally:
            self.idx.destroy_context(C.byref(ctx))
        return out["b"], out["p"]

    def __del__(self):
        if getattr(self, "idx", None) is not None and self.idx.private_data:
            self.idx.release(C.byref(self.idx))


PREDICATES = {"equals": 0, "disjoint": 1, "touches": 2, "contains": 3, "covers": 4,
              "intersects": 5, "within": 6, "coveredby": 7, "dwithin": 100}


class Refiner:
    """SedonaSpatialRefiner (c/sedona-libgpuspatial/src/libgpuspatial.rs:310-486)."""

    def __init__(self, runtime: Optional[Runtime] = None, concurrency: int = 1,
                 compress_bvh: bool = False, pipeline_batches: int = 1):
        self.runtime = runtime or Runtime.get()
        self.ref = SedonaSpatialRefiner()
        cfg = GpuSpatialRefinerConfig(C.pointer(self.runtime.rt), concurrency, compress_bvh,
                                      pipeline_batches)
        if lib().GpuSpatialRefinerCreate(C.byref(self.ref), C.byref(cfg)) != 0:
            raise GpuSpatialError("Refiner Create failed")
        self._keep = []

    def _err(self):
        return self.ref.get_last_error(C.byref(self.ref))

    def clear(self):
        _check(self.ref.clear(C.byref(self.ref)), "clear", self._err)

    def init_build_schema(self, large: bool = False):
        self._schema = ArrowSchema(format=b"Z" if large else b"z", name=b"geometry")
        _check(self.ref.init_build_schema(C.byref(self.ref), C.byref(self._schema)),
               "init_build_schema", self._err)

    def push_build(self, col: WkbColumn):
        a = ArrowBinary(col)
        self._keep.append(a)
        _check(self.ref.push_build(C.byref(self.ref), C.byref(a.array)), "push_build", self._err)

    def finish_building(self):
        _check(self.ref.finish_building(C.byref(self.ref)), "finish_building", self._err)

    def refine(self, probe: WkbColumn, predicate: str, build_idx: np.ndarray,
               probe_idx: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
        a = ArrowBinary(probe)
        b = np.ascontiguousarray(build_idx, dtype=np.uint32).copy()
        p = np.ascontiguousarray(probe_idx, dtype=np.uint32).copy()
        new_n = C.c_uint32(0)
        rc = self.ref.refine(C.byref(self.ref), C.byref(a.schema), C.byref(a.array),
                             PREDICATES[predicate], b.ctypes.data_as(C.POINTER(C.c_uint32)),
                             p.ctypes.data_as(C.POINTER(C.c_uint32)), len(b), C.byref(new_n))
        _check(rc, "refine", self._err)
        return b[:new_n.value], p[:new_n.value]

    def __del__(self):
        if getattr(self, "ref", None) is not None and self.ref.private_data:
            self.ref.release(C.byref(self.ref))


class SpatialJoin:
    """The fused build/probe join (SpjJoin*, include/spj_gb300.h)."""

    def __init__(self, runtime: Optional[Runtime] = None, leaf_size: int = 0,
                 refine_form: int = 1, profile: bool = False, probe_order: int = 0):
        self.runtime = runtime or Runtime.get()
        self.h = C.c_void_p()
        cfg = SpjJoinConfig(C.pointer(self.runtime.rt), leaf_size, refine_form, int(profile),
                            probe_order)
        if lib().SpjJoinCreate(C.byref(cfg), C.byref(self.h)) != 0:
            raise GpuSpatialError("SpjJoinCreate failed")
        self._keep = []

    def _err(self):
        return lib().SpjJoinLastError(self.h)

    def set_option(self, key: str, value: int):
        _check(lib().SpjJoinSetOption(self.h, key.encode(), int(value)), "set_option", self._err)

    def build(self, col: WkbColumn):
        a = ArrowBinary(col)
        self._keep = [a]
        _check(lib().SpjJoinPushBuildArrow(self.h, C.byref(a.schema), C.byref(a.array)),
               "push_build", self._err)
        _check(lib().SpjJoinFinishBuild(self.h), "finish_build", self._err)

    def build_device(self, dcol: SpjDeviceWkb):
        _check(lib().SpjJoinBuildDevice(self.h, C.byref(dcol)), "build_device", self._err)

    def probe(self, col: WkbColumn, predicate: str = "intersects", distance: float = 0.0,
              probe_base: int = 0) -> Tuple[np.ndarray, np.ndarray]:
        a = ArrowBinary(col)
        out = {}

        def cb(b, p, n, _ud):
            out["b"] = np.ctypeslib.as_array(b, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
            out["p"] = np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
            return 0

        ccb = JOIN_CB(cb)
        rc = lib().SpjJoinProbeArrow(self.h, C.byref(a.schema), C.byref(a.array),
                                     PREDICATES[predicate], distance, probe_base, ccb, None)
        _check(rc, "probe", self._err)
        return out["b"], out["p"]

    def probe_host(self, col: WkbColumn, predicate: str, distance: float, out_b: np.ndarray,
                   out_p: np.ndarray, probe_base: int = 0) -> int:
        n = C.c_uint64(0)
        rc = lib().SpjJoinProbeHost(
            self.h, len(col), col.offsets.ctypes.data, int(col.offsets.dtype == np.int64),
            col.data.ctypes.data, col.validity.ctypes.data if col.validity is not None else None,
            PREDICATES[predicate], distance, probe_base, out_b.ctypes.data, out_p.ctypes.data,
            len(out_b), C.byref(n))
        _check(rc, "probe_host", self._err)
        return n.value

    def set_probe_distances(self, distances: Optional[np.ndarray]):
        """ST_DWithin distance column: one distance per probe row for the
        next probes (None clears it)."""
        if distances is None:
            _check(lib().SpjJoinSetProbeDistances(self.h, None, 0, 0), "set distances", self._err)
            return
        d = np.ascontiguousarray(distances, dtype=np.float64)
        _check(lib().SpjJoinSetProbeDistances(self.h, d.ctypes.data, len(d), 0),
               "set distances", self._err)

    def join_partitioned(self, build: WkbColumn, probe: WkbColumn, predicate: str = "intersects",
                         distance: float = 0.0, num_partitions: int = 0,
                         build_budget_bytes: int = 0, sample_rows: int = 0, seed: int = 0,
                         host_gather: bool = False, record_layout: bool = False):
        """The join of two host columns in partition passes (SpjJoinPartitioned):
        (build ids, probe ids, stats).  The join's build side is replaced."""
        keep = []

        def host(col):
            off = np.ascontiguousarray(col.offsets)
            data = np.ascontiguousarray(col.data) if len(col.data) else np.zeros(8, np.uint8)
            val = np.ascontiguousarray(col.validity) if col.validity is not None else None
            keep.extend([off, data, val])
            return SpjHostWkb(len(col), off.ctypes.data, int(off.dtype == np.int64),
                              data.ctypes.data, val.ctypes.data if val is not None else None, 0)

        hb, hp = host(build), host(probe)
        self._last_rows = (len(build), len(probe))
        chunks = []

        def cb(b, p, n, _ud):
            if n:
                chunks.append((np.ctypeslib.as_array(b, shape=(n,)).copy(),
                               np.ctypeslib.as_array(p, shape=(n,)).copy()))
            return 0

        ccb = JOIN_CB(cb)
        opt = SpjPartitionOptions(num_partitions, sample_rows, build_budget_bytes, seed,
                                  int(host_gather), int(record_layout))
        st = SpjPartitionStats()
        rc = lib().SpjJoinPartitioned(self.h, C.byref(hb), C.byref(hp), PREDICATES[predicate],
                                      distance, C.byref(opt), ccb, None, C.byref(st))
        _check(rc, "join_partitioned", self._err)
        b = np.concatenate([c[0] for c in chunks]) if chunks else np.zeros(0, np.uint32)
        p = np.concatenate([c[1] for c in chunks]) if chunks else np.zeros(0, np.uint32)
        return b, p, {f: getattr(st, f) for f, _ in SpjPartitionStats._fields_}

    def partition_layout(self) -> dict:
        """The last partitioned join's partitioning (SpjJoinPartitionLayout)."""
        counts = np.zeros(4, np.uint32)
        _check(lib().SpjJoinPartitionLayout(self.h, counts.ctypes.data, *[None] * 6), "layout",
               self._err)
        nl, ns = int(counts[0]), int(counts[1])
        extent = np.zeros(4, np.float32)
        leaves = np.zeros((max(nl, 1), 4), np.float32)
        bounds = np.zeros((max(nl, 1), 4), np.float32)
        samples = np.zeros((max(ns, 1), 4), np.float32)
        nb, npr = getattr(self, "_last_rows", (0, 0))
        bpart = np.zeros(max(nb, 1), np.uint32)
        ppart = np.zeros(max(npr, 1), np.uint32)
        _check(lib().SpjJoinPartitionLayout(self.h, counts.ctypes.data, extent.ctypes.data,
                                            leaves.ctypes.data, bounds.ctypes.data,
                                            samples.ctypes.data, bpart.ctypes.data,
                                            ppart.ctypes.data), "layout", self._err)
        return {"extent": extent, "leaves": leaves[:nl], "bounds": bounds[:nl],
                "samples": samples[:ns], "max_items": int(counts[2]),
                "max_levels": int(counts[3]), "build_part": bpart[:nb], "probe_part": ppart[:npr]}

    def probe_device(self, dcol: SpjDeviceWkb, predicate: str = "intersects",
                     distance: float = 0.0, probe_base: int = 0):
        db, dp, n = C.c_void_p(), C.c_void_p(), C.c_uint64()
        rc = lib().SpjJoinProbeDevice(self.h, C.byref(dcol), PREDICATES[predicate], distance,
                                      probe_base, C.byref(db), C.byref(dp), C.byref(n))
        _check(rc, "probe_device", self._err)
        return db.value, dp.value, n.value

    def stream(self) -> int:
        return lib().SpjJoinStream(self.h)

    def stats(self) -> dict:
        s = SpjJoinStats()
        _check(lib().SpjJoinGetStats(self.h, C.byref(s)), "stats", self._err)
        return {f: getattr(s, f) for f, _ in SpjJoinStats._fields_}

    def reset_stats(self):
        _check(lib().SpjJoinResetStats(self.h), "reset_stats", self._err)

    def __del__(self):
        if getattr(self, "h", None):
            lib().SpjJoinRelease(self.h)
            self.h = None


class StreamProbe:
    """Batched probe stream over device point batches (SpjStream*,
    include/spj_gb300.h): one CUDA-graph replay per run."""

    def __init__(self, join: "SpatialJoin"):
        self.join = join  # must outlive the stream
        self.h = C.c_void_p()
        if lib().SpjStreamCreate(join.h, C.byref(self.h)) != 0:
            raise GpuSpatialError(f"SpjStreamCreate: {lib().SpjJoinLastError(join.h).decode()}")

    def _err(self):
        return lib().SpjStreamLastError(self.h)

    def set_batches(self, dcols):
        arr = (SpjDeviceWkb * max(len(dcols), 1))(*dcols)
        self._cols = arr
        _check(lib().SpjStreamSetBatches(self.h, arr, len(dcols)), "set_batches", self._err)

    def run(self, predicate: str = "contains"):
        db, dp, n = C.c_void_p(), C.c_void_p(), C.c_uint64()
        _check(lib().SpjStreamRun(self.h, PREDICATES[predicate], C.byref(db), C.byref(dp),
                                  C.byref(n)), "run", self._err)
        return db.value, dp.value, n.value

    def set_params(self, block: int, chunk_rows: int, leaf_size: int):
        _check(lib().SpjStreamSetParams(self.h, block, chunk_rows, leaf_size), "set_params",
               self._err)

    def autotune(self, predicate: str, cache_path: Optional[str] = None):
        b, c, l = C.c_int32(), C.c_uint32(), C.c_uint32()
        _check(lib().SpjStreamAutotune(self.h, PREDICATES[predicate],
                                       cache_path.encode() if cache_path else None, C.byref(b),
                                       C.byref(c), C.byref(l)), "autotune", self._err)
        return b.value, c.value, l.value

    def stats(self):
        ms, esc, la = C.c_double(), C.c_uint64(), C.c_uint64()
        _check(lib().SpjStreamGetStats(self.h, C.byref(ms), C.byref(esc), C.byref(la)), "stats",
               self._err)
        return {"ms_last": ms.value, "escalations": esc.value, "launches_per_replay": la.value}

    def stream(self) -> int:
        return lib().SpjStreamCudaStream(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().SpjStreamRelease(self.h)
            self.h = None


class LearnedIndex:
    """Learned point index over a device point column (SpjLearned*,
    include/spj_gb300.h)."""

    def __init__(self, runtime: Optional[Runtime] = None, leaves: int = 4096, window: int = 4096):
        self.runtime = runtime or Runtime.get()
        self.h = C.c_void_p()
        cfg = SpjLearnedConfig(C.pointer(self.runtime.rt), leaves, window)
        if lib().SpjLearnedCreate(C.byref(cfg), C.byref(self.h)) != 0:
            raise GpuSpatialError("SpjLearnedCreate failed")
        self.leaves = leaves

    def _err(self):
        return lib().SpjLearnedLastError(self.h)

    def build_device(self, dcol: SpjDeviceWkb):
        _check(lib().SpjLearnedBuildDevice(self.h, C.byref(dcol)), "build", self._err)

    def set_trained(self, trained: bool):
        _check(lib().SpjLearnedSetTrained(self.h, int(trained)), "set_trained", self._err)

    def query_device(self, dcol: SpjDeviceWkb, predicate: str = "intersects", probe_base: int = 0):
        db, dp, n = C.c_void_p(), C.c_void_p(), C.c_uint64()
        _check(lib().SpjLearnedQueryDevice(self.h, C.byref(dcol), PREDICATES[predicate],
                                           probe_base, C.byref(db), C.byref(dp), C.byref(n)),
               "query", self._err)
        return db.value, dp.value, n.value

    def loss_and_grad(self, a: np.ndarray, b: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        loss = np.empty(self.leaves)
        ga = np.empty(self.leaves)
        gb = np.empty(self.leaves)
        _check(lib().SpjLearnedLossAndGrad(self.h, a.ctypes.data, b.ctypes.data, loss.ctypes.data,
                                           ga.ctypes.data, gb.ctypes.data), "loss_and_grad",
               self._err)
        return loss, ga, gb

    def export(self):
        st = self.stats()
        n, L = st["points"], self.leaves
        keys = np.empty(n, np.uint32)
        start = np.empty(L + 1, np.uint32)
        kc = np.empty(L, np.uint32)
        a = np.empty(L)
        b = np.empty(L)
        err = np.empty(L, np.uint32)
        _check(lib().SpjLearnedExport(self.h, keys.ctypes.data, start.ctypes.data, kc.ctypes.data,
                                      a.ctypes.data, b.ctypes.data, err.ctypes.data), "export",
               self._err)
        return {"keys": keys, "leaf_start": start, "leaf_kc": kc, "a": a, "b": b, "err": err}

    def stats(self) -> dict:
        s = SpjLearnedStats()
        _check(lib().SpjLearnedGetStats(self.h, C.byref(s)), "stats", self._err)
        return {f: getattr(s, f) for f, _ in SpjLearnedStats._fields_}

    def stream(self) -> int:
        return lib().SpjLearnedStream(self.h)

    def set_window(self, window: int):
        _check(lib().SpjLearnedSetWindow(self.h, window), "set_window", self._err)

    def autotune_window(self, samples, predicate: str = "intersects") -> int:
        arr = (SpjDeviceWkb * len(samples))(*samples)
        w = C.c_uint32()
        _check(lib().SpjLearnedAutotuneWindow(self.h, arr, len(samples), PREDICATES[predicate],
                                              C.byref(w)), "autotune_window", self._err)
        return w.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().SpjLearnedRelease(self.h)
            self.h = None


class KnnJoin:
    """KNN join over point columns (SpjKnn*, include/spj_gb300.h)."""

    def __init__(self, runtime: Optional[Runtime] = None, leaf_size: int = 0,
                 refine_form: int = 1):
        self.runtime = runtime or Runtime.get()
        self.h = C.c_void_p()
        cfg = SpjKnnConfig(C.pointer(self.runtime.rt), leaf_size, refine_form)
        if lib().SpjKnnCreate(C.byref(cfg), C.byref(self.h)) != 0:
            raise GpuSpatialError("SpjKnnCreate failed")

    def _err(self):
        return lib().SpjKnnLastError(self.h)

    def build(self, x: np.ndarray, y: np.ndarray):
        xy = np.ascontiguousarray(np.stack([x, y], 1), dtype=np.float64)
        _check(lib().SpjKnnBuild(self.h, xy.ctypes.data, len(xy)), "knn build", self._err)

    def query(self, x: np.ndarray, y: np.ndarray, k: int):
        xy = np.ascontiguousarray(np.stack([x, y], 1), dtype=np.float64)
        idx = np.empty((len(xy), k), dtype=np.uint32)
        dist = np.empty((len(xy), k), dtype=np.float64)
        _check(lib().SpjKnnQuery(self.h, xy.ctypes.data, len(xy), k, idx.ctypes.data,
                                 dist.ctypes.data, 0), "knn query", self._err)
        return idx, dist

    def query_device(self, d_xy: int, n: int, k: int, d_idx: int, d_dist: int):
        _check(lib().SpjKnnQuery(self.h, d_xy, n, k, d_idx, d_dist, 1), "knn query", self._err)

    def _ragged(self, call, n: int):
        """Runs a variable-length query (two tries: the first learns the size)."""
        offsets = np.zeros(n + 1, dtype=np.uint64)
        total = C.c_uint64(0)
        cap = max(16, n * 2)
        for _ in range(2):
            idx = np.empty(cap, dtype=np.uint32)
            dist = np.empty(cap, dtype=np.float64)
            rc = call(offsets, idx, dist, cap, total)
            if rc == 28:  # ENOSPC: retry with the reported size
                cap = int(total.value)
                continue
            _check(rc, "knn query", self._err)
            t = int(total.value)
            return offsets.astype(np.int64), idx[:t], dist[:t]
        raise GpuSpatialError("knn query: output size changed between calls")

    def query_ties(self, x: np.ndarray, y: np.ndarray, k: int, include_tie_breakers: bool = True):
        """Per probe i: idx / dist[offsets[i]:offsets[i+1]] are its k nearest
        and, with include_tie_breakers, every other build point within 1e-9
        of its k-th distance."""
        xy = np.ascontiguousarray(np.stack([x, y], 1), dtype=np.float64)
        return self._ragged(lambda o, i, d, cap, tot: lib().SpjKnnQueryTies(
            self.h, xy.ctypes.data, len(xy), k, int(include_tie_breakers), 0, o.ctypes.data,
            i.ctypes.data, d.ctypes.data, cap, C.byref(tot)), len(xy))

    def query_wkb(self, col: WkbColumn, k: int, include_tie_breakers: bool = False):
        """query_knn over a WKB point column (decoded on the device); empty
        and null rows get no results.  Returns (offsets, idx, dist)."""
        a = ArrowBinary(col)
        return self._ragged(lambda o, i, d, cap, tot: lib().SpjKnnQueryArrow(
            self.h, C.byref(a.schema), C.byref(a.array), k, int(include_tie_breakers),
            o.ctypes.data, i.ctypes.data, d.ctypes.data, cap, C.byref(tot)), len(col))

    def stream(self) -> int:
        return lib().SpjKnnStream(self.h)

    def stats(self) -> dict:
        v = [C.c_uint64() for _ in range(3)]
        _check(lib().SpjKnnGetStats(self.h, *[C.byref(x) for x in v]), "knn stats", self._err)
        return dict(zip(("queries", "exact_evals", "redone"), (x.value for x in v)))

    def __del__(self):
        if getattr(self, "h", None):
            lib().SpjKnnRelease(self.h)
            self.h = None
