"""Joined-batch materialisation on the device (SpjGather*, SpjVisited*).

The reference assembles each output batch of the spatial join on the host:
``build_batch_from_indices`` takes every output column from the build batch
or the probe batch by the refined index arrays
(rust/sedona-spatial-join/src/utils/join_utils.rs:346-405), and outer, semi,
anti and mark joins record the matched build rows in a visited bitmap
(stream.rs:1447-1455) whose unmatched / matched rows are emitted at the end
(get_final_indices_from_bit_map, join_utils.rs:95-124).  Here the same steps
run on device buffers (torch tensors as HBM plumbing), so the pairs the join
produced never leave the GPU.

Index tensors are int32 holding uint32 row ids; ``NULL_INDEX`` (-1 as int32)
gathers a null row, as a null entry of the reference's index arrays does.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Tuple

import torch

from .capi import GpuSpatialError, lib

NULL_INDEX = -1  # 0xFFFFFFFF as uint32
ENOSPC = 28


def _err():
    return lib().SpjMaterializeLastError()


def _check(rc: int, what: str):
    if rc != 0:
        raise GpuSpatialError(f"{what}: {_err().decode(errors='replace')}")


def _stream(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return t.data_ptr() if t is not None and t.numel() else None


def _index(idx: torch.Tensor) -> torch.Tensor:
    if idx.dtype not in (torch.int32,) or not idx.is_cuda:
        raise GpuSpatialError("index arrays are int32 device tensors (uint32 row ids)")
    return idx.contiguous()


@dataclass
class DeviceColumn:
    """One Arrow column on the device.  Fixed width: ``values`` (rows x
    item, 1-16 bytes per row).  Binary / utf8: ``offsets`` (int32 or int64,
    rows + 1) and ``data`` (uint8).  ``validity``: LSB bitmap (uint8) whose
    bit ``validity_offset + row`` is the row's, or None for no nulls."""
    length: int
    values: Optional[torch.Tensor] = None
    offsets: Optional[torch.Tensor] = None
    data: Optional[torch.Tensor] = None
    validity: Optional[torch.Tensor] = None
    validity_offset: int = 0
    null_count: int = 0

    @property
    def is_binary(self) -> bool:
        return self.offsets is not None


def take_fixed(values: torch.Tensor, idx: torch.Tensor) -> torch.Tensor:
    """values[idx] along dim 0; a null index gives a zero row."""
    idx = _index(idx)
    values = values.contiguous()
    n_values = values.shape[0]
    width = values.element_size()
    for d in values.shape[1:]:
        width *= d
    out = torch.empty((idx.numel(),) + tuple(values.shape[1:]), dtype=values.dtype,
                      device=values.device)
    _check(lib().SpjGatherFixed(_ptr(values), width, n_values, _ptr(idx), idx.numel(),
                                _ptr(out), _stream(values)), "gather")
    return out


def take_validity(validity: Optional[torch.Tensor], validity_offset: int, n_values: int,
                  idx: torch.Tensor) -> Tuple[torch.Tensor, int]:
    """The validity bitmap (uint8, whole 32-bit words) of the gathered rows
    and its null count."""
    idx = _index(idx)
    n = idx.numel()
    words = torch.empty(((n + 31) // 32,), dtype=torch.int32, device=idx.device)
    nulls = C.c_uint64(0)
    _check(lib().SpjGatherValidity(_ptr(validity), validity_offset, n_values, _ptr(idx), n,
                                   _ptr(words), C.byref(nulls), _stream(idx)), "gather validity")
    return words.view(torch.uint8), int(nulls.value)


def take_binary(offsets: torch.Tensor, data: torch.Tensor,
                idx: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
    """The gathered values of a binary column: (int64 offsets, uint8 data)."""
    idx = _index(idx)
    if offsets.dtype not in (torch.int32, torch.int64):
        raise GpuSpatialError("binary offsets are int32 or int64")
    offsets = offsets.contiguous()
    n = idx.numel()
    out_off = torch.empty((n + 1,), dtype=torch.int64, device=idx.device)
    total = C.c_uint64(0)
    args = (_ptr(offsets), int(offsets.dtype == torch.int64), _ptr(data), offsets.numel() - 1,
            _ptr(idx), n, _ptr(out_off))
    rc = lib().SpjGatherBinary(*args, None, 0, C.byref(total), _stream(idx))
    if rc not in (0, ENOSPC):
        _check(rc, "gather binary")
    out = torch.empty((int(total.value),), dtype=torch.uint8, device=idx.device)
    if out.numel():
        _check(lib().SpjGatherBinary(*args, _ptr(out), out.numel(), C.byref(total),
                                     _stream(idx)), "gather binary")
    return out_off, out


def take(col: DeviceColumn, idx: torch.Tensor) -> DeviceColumn:
    """Arrow ``take`` of one column by an index array with nulls."""
    if col.is_binary:
        off, data = take_binary(col.offsets, col.data, idx)
        out = DeviceColumn(idx.numel(), offsets=off, data=data)
    else:
        out = DeviceColumn(idx.numel(), values=take_fixed(col.values, idx))
    out.validity, out.null_count = take_validity(col.validity, col.validity_offset,
                                                 col.length, idx)
    return out


def build_joined_columns(build_cols, probe_cols, build_idx: torch.Tensor,
                         probe_idx: torch.Tensor):
    """The output columns of one joined batch, build side first then probe
    side (build_batch_from_indices with every column projected)."""
    return ([take(c, build_idx) for c in build_cols] +
            [take(c, probe_idx) for c in probe_cols])


class VisitedBitmap:
    """The build side's visited rows of an outer / semi / anti / mark join."""

    def __init__(self, n_rows: int, device="cuda"):
        self.n_rows = n_rows
        self.words = torch.zeros(((n_rows + 31) // 32,), dtype=torch.int32, device=device)

    def mark(self, idx: torch.Tensor):
        idx = _index(idx)
        _check(lib().SpjVisitedMark(_ptr(self.words), self.n_rows, _ptr(idx), idx.numel(),
                                    _stream(idx)), "visited mark")

    def collect(self, visited: bool) -> torch.Tensor:
        """Rows whose bit is set (visited=True: semi joins) or clear (left,
        left anti and full joins), ascending, as int32."""
        count = C.c_uint64(0)
        s = _stream(self.words)
        rc = lib().SpjVisitedCollect(_ptr(self.words), self.n_rows, int(visited), None, 0,
                                     C.byref(count), s)
        if rc not in (0, ENOSPC):
            _check(rc, "visited collect")
        out = torch.empty((int(count.value),), dtype=torch.int32, device=self.words.device)
        if out.numel():
            _check(lib().SpjVisitedCollect(_ptr(self.words), self.n_rows, int(visited),
                                           _ptr(out), out.numel(), C.byref(count), s),
                   "visited collect")
        return out

    def bitmap(self) -> torch.Tensor:
        """The mark column of a mark join: Arrow LSB bits, one per row."""
        return self.words.view(torch.uint8)[: (self.n_rows + 7) // 8]
