"""SpjIndexProbeNoAlloc: the index filter for callers that cannot allocate
device memory at probe time (an executor whose arena owns the device memory
budget, or a latency-critical loop that must not touch the CUDA allocator).
Its scratch is a static device array, so it takes at most
SPJ_NOALLOC_MAX_PROBES probe rects per call.

Checked through the C ABI against the regular SedonaFloatIndex2D probe (which
allocates) on two calls in a row: the pair sets must be identical (integer
results, exact).  Collected last (test_zz_*) so a failure here leaves every
other test already run; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PROBES = 1 << 18


@pytest.fixture(scope="module")
def env():
    import torch
    from sedona_gpuspatial import _build, capi
    _build.build()
    L = capi.lib()
    L.SpjIndexProbeNoAlloc.argtypes = [C.POINTER(capi.SedonaFloatIndex2D), C.c_void_p,
                                       C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint64,
                                       C.POINTER(C.c_uint64), C.c_void_p]
    L.SpjAllocationCount.restype = C.c_uint64
    L.SpjAllocationCount.argtypes = []
    return torch, capi, L


def _boxes(rng, n, points=False):
    x = rng.uniform(-180, 180, n)
    y = rng.uniform(-180, 180, n)
    w = 0 if points else rng.uniform(0, 30, n)
    h = 0 if points else rng.uniform(0, 30, n)
    return np.stack([x, y, x + w, y + h], 1).astype(np.float32)


def _pairs(b, p):
    return sorted(zip(np.asarray(p).tolist(), np.asarray(b).tolist()))


def _no_alloc_probe(torch, capi, L, idx, rects, capacity, warm=False):
    d_rects = torch.from_numpy(rects).cuda()
    d_b = torch.empty(max(capacity, 1), dtype=torch.int32, device="cuda")
    d_p = torch.empty(max(capacity, 1), dtype=torch.int32, device="cuda")
    n = C.c_uint64(0)
    torch.cuda.synchronize()
    # the library's own allocation count, read right around the call, may
    # not move; on a warm call (the static array's module already loaded by
    # an earlier call) the device's free memory may not move either
    allocs0 = L.SpjAllocationCount()
    free0 = torch.cuda.mem_get_info()[0]
    rc = L.SpjIndexProbeNoAlloc(C.byref(idx.idx), d_rects.data_ptr(), len(rects),
                                d_b.data_ptr(), d_p.data_ptr(), capacity, C.byref(n), None)
    free1 = torch.cuda.mem_get_info()[0]
    assert L.SpjAllocationCount() == allocs0, "the no-allocation probe allocated"
    if warm:
        assert free1 == free0, (free0, free1)
    b = d_b[: n.value].cpu().numpy().view(np.uint32) if rc == 0 else None
    p = d_p[: n.value].cpu().numpy().view(np.uint32) if rc == 0 else None
    return rc, n.value, b, p


def test_no_alloc_probe_matches_regular_probe_twice(env):
    torch, capi, L = env
    rng = np.random.default_rng(11)
    idx = capi.FloatIndex2D()
    idx.push_build(_boxes(rng, 20000))
    idx.finish_building()
    for call, rects in enumerate([_boxes(rng, 50000), _boxes(rng, 70000, points=True)]):
        eb, ep = idx.probe(rects)  # existing entry point (allocates)
        rc, n, b, p = _no_alloc_probe(torch, capi, L, idx, rects, capacity=len(eb) + 100,
                                      warm=call > 0)
        assert rc == 0, idx.idx.get_last_error(C.byref(idx.idx))
        assert n == len(eb) > 0
        assert _pairs(b, p) == _pairs(eb, ep), call
        # same grouping as the regular probe: ascending probe order
        assert np.all(np.diff(p.astype(np.int64)) >= 0)


def test_no_alloc_probe_limits(env):
    torch, capi, L = env
    rng = np.random.default_rng(12)
    idx = capi.FloatIndex2D()
    idx.push_build(_boxes(rng, 1000))
    idx.finish_building()
    rects = _boxes(rng, 5000)
    eb, _ = idx.probe(rects)
    # too small an output: ENOSPC, the count is still reported
    rc, n, _, _ = _no_alloc_probe(torch, capi, L, idx, rects, capacity=max(len(eb) - 1, 0))
    assert rc == 28 and n == len(eb)
    # more rects than the static scratch holds: rejected with a message
    big = np.zeros((MAX_PROBES + 1, 4), np.float32)
    rc, _, _, _ = _no_alloc_probe(torch, capi, L, idx, big, capacity=16)
    assert rc != 0
    assert b"maximum" in idx.idx.get_last_error(C.byref(idx.idx))
    # and the largest allowed batch works
    full = _boxes(rng, MAX_PROBES)
    eb, ep = idx.probe(full)
    rc, n, b, p = _no_alloc_probe(torch, capi, L, idx, full, capacity=len(eb))
    assert rc == 0 and _pairs(b, p) == _pairs(eb, ep)


def test_no_alloc_probe_rejects_misaligned_pointers(env):
    """A rect pointer off a 16-byte boundary (e.g. from an arena that aligns
    to 8 bytes) is rejected with EINVAL and a message before any launch."""
    torch, capi, L = env
    rng = np.random.default_rng(13)
    idx = capi.FloatIndex2D()
    idx.push_build(_boxes(rng, 500))
    idx.finish_building()
    rects = _boxes(rng, 64)
    buf = torch.zeros(len(rects) * 4 + 2, dtype=torch.float32, device="cuda")
    buf[2:].copy_(torch.from_numpy(rects.reshape(-1)))  # rects start 8 bytes in
    out = torch.empty(1024, dtype=torch.int32, device="cuda")
    n = C.c_uint64(0)
    torch.cuda.synchronize()
    rc = L.SpjIndexProbeNoAlloc(C.byref(idx.idx), buf.data_ptr() + 8, len(rects),
                                out.data_ptr(), out.data_ptr() + 2048, 256, C.byref(n), None)
    assert rc == 22
    assert b"16-byte" in idx.idx.get_last_error(C.byref(idx.idx))
    rc = L.SpjIndexProbeNoAlloc(C.byref(idx.idx), buf.data_ptr(), len(rects),
                                out.data_ptr() + 2, out.data_ptr() + 2048, 256, C.byref(n), None)
    assert rc == 22
    assert b"4-byte" in idx.idx.get_last_error(C.byref(idx.idx))
    # host memory is not accepted either
    host = np.ascontiguousarray(np.tile(rects, (1, 1)))
    rc = L.SpjIndexProbeNoAlloc(C.byref(idx.idx), host.ctypes.data, len(rects),
                                out.data_ptr(), out.data_ptr() + 2048, 256, C.byref(n), None)
    assert rc == 22
    # the index still answers afterwards
    eb, ep = idx.probe(rects)
    rc, n2, b, p = _no_alloc_probe(torch, capi, L, idx, rects, capacity=len(eb) + 1)
    assert rc == 0 and _pairs(b, p) == _pairs(eb, ep)
