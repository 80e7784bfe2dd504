"""Device-buffer helpers for the GPU tests (torch owns the memory; the
library under test only sees raw pointers through its C ABI)."""
import numpy as np


def device_column(capi, col):
    """Uploads a WKB column; returns (SpjDeviceWkb, tensors keeping it alive)."""
    import torch
    off = torch.from_numpy(np.ascontiguousarray(col.offsets)).cuda()
    data = torch.from_numpy(np.ascontiguousarray(col.data) if len(col.data)
                            else np.zeros(8, np.uint8)).cuda()
    d = capi.SpjDeviceWkb(length=len(col), offsets=off.data_ptr(),
                          offsets_are_64bit=int(col.offsets.dtype == np.int64),
                          data=data.data_ptr(), data_length=len(col.data), validity=None,
                          validity_offset=0)
    return d, (off, data)


class _DevArray:
    """A raw device pointer exposed through __cuda_array_interface__."""

    def __init__(self, ptr, n, typestr="<i4"):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                         "data": (ptr, False), "version": 3, "strides": None}


def device_pairs(db, dp, n):
    """Copies n (build, probe) u32 pairs from device pointers to numpy."""
    import torch
    if n == 0:
        return np.zeros(0, np.uint32), np.zeros(0, np.uint32)
    torch.cuda.synchronize()
    b = torch.as_tensor(_DevArray(db, n), device="cuda").cpu().numpy().view(np.uint32)
    p = torch.as_tensor(_DevArray(dp, n), device="cuda").cpu().numpy().view(np.uint32)
    return b, p


def pairs(b, p):
    return sorted(zip(np.asarray(p).tolist(), np.asarray(b).tolist()))
