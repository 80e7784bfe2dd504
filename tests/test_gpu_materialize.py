"""Joined-batch materialisation on the device (SpjGather*, SpjVisited*)
against numpy restatements of Arrow's take and the reference's visited
bitmap handling (build_batch_from_indices, join_utils.rs:346-405;
get_final_indices_from_bit_map, join_utils.rs:95-124).  All results are
integer / byte data and must match exactly."""
import numpy as np
import pytest

import gpu_util

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mat():
    from sedona_gpuspatial import _build
    _build.build()
    from sedona_gpuspatial import materialize
    return materialize


def _idx(rng, n, n_values, null_frac=0.1, oob=True):
    idx = rng.integers(0, max(n_values, 1), n).astype(np.int64)
    idx[rng.random(n) < null_frac] = 0xFFFFFFFF
    if oob and n:
        idx[rng.integers(0, n)] = n_values + 5  # past the end: a null row
    return idx.astype(np.uint32)


def _valid_rows(idx, n_values):
    return idx.astype(np.int64) < n_values


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("width", [1, 2, 4, 8, 16])
@pytest.mark.parametrize("n", [0, 1, 1000, 100003])
def test_take_fixed(mat, width, n):
    import torch
    rng = np.random.default_rng(width * 7 + n)
    n_values = 5000
    vals = rng.integers(0, 2**31, (n_values, 4), dtype=np.int64).astype(np.uint32)
    vals = vals.view(np.uint8).reshape(n_values, 16)[:, :width].copy()
    idx = _idx(rng, n, n_values)
    out = mat.take_fixed(_t(vals), _t(idx.view(np.int32))).cpu().numpy()
    ok = _valid_rows(idx, n_values)
    exp = np.zeros((n, width), np.uint8)
    exp[ok] = vals[idx[ok]]
    assert out.shape == (n, width)
    assert np.array_equal(out, exp)
    # a typed column: float64 values, one per row
    f = rng.standard_normal(n_values)
    got = mat.take_fixed(torch.from_numpy(f).cuda(), _t(idx.view(np.int32))).cpu().numpy()
    expf = np.zeros(n, np.float64)
    expf[ok] = f[idx[ok]]
    assert np.array_equal(got.view(np.uint64), expf.view(np.uint64))


@pytest.mark.parametrize("voff", [0, 3, 13])
@pytest.mark.parametrize("with_validity", [False, True])
def test_take_validity(mat, voff, with_validity):
    rng = np.random.default_rng(voff + 100 * with_validity)
    n_values, n = 7777, 50001
    bits = rng.random(n_values + voff) < 0.8
    validity = np.packbits(bits, bitorder="little")
    idx = _idx(rng, n, n_values)
    out, nulls = mat.take_validity(_t(validity) if with_validity else None, voff, n_values,
                                   _t(idx.view(np.int32)))
    got = np.unpackbits(out.cpu().numpy(), bitorder="little")[:n].astype(bool)
    ok = _valid_rows(idx, n_values)
    exp = ok.copy()
    if with_validity:
        exp[ok] &= bits[voff + idx[ok].astype(np.int64)]
    assert np.array_equal(got, exp)
    assert nulls == int((~exp).sum())
    # bits past n in the last word stay clear
    tail = np.unpackbits(out.cpu().numpy(), bitorder="little")[n:]
    assert not tail.any()


@pytest.mark.parametrize("off64", [False, True])
@pytest.mark.parametrize("maxlen", [0, 7, 300])
def test_take_binary(mat, off64, maxlen):
    rng = np.random.default_rng(int(off64) * 1000 + maxlen)
    n_values, n = 3001, 20000
    lens = rng.integers(0, maxlen + 1, n_values)
    offsets = np.zeros(n_values + 1, np.int64)
    np.cumsum(lens, out=offsets[1:])
    data = rng.integers(0, 256, max(int(offsets[-1]), 1), dtype=np.uint8)
    idx = _idx(rng, n, n_values)
    off = offsets if off64 else offsets.astype(np.int32)
    o, d = mat.take_binary(_t(off), _t(data), _t(idx.view(np.int32)))
    o, d = o.cpu().numpy(), d.cpu().numpy()
    ok = _valid_rows(idx, n_values)
    ii = idx.astype(np.int64)
    exp_lens = np.where(ok, lens[np.where(ok, ii, 0)], 0)
    exp_off = np.zeros(n + 1, np.int64)
    np.cumsum(exp_lens, out=exp_off[1:])
    assert np.array_equal(o, exp_off)
    exp = b"".join(data[offsets[j]:offsets[j + 1]].tobytes() if k else b""
                   for j, k in zip(ii, ok))
    assert d.tobytes() == exp


def test_take_binary_too_small(mat):
    """The ABI reports ENOSPC with the needed size and writes only offsets."""
    import ctypes as C
    import torch
    from sedona_gpuspatial import capi
    off = _t(np.array([0, 5, 9], np.int32))
    data = _t(np.arange(9, dtype=np.uint8))
    idx = _t(np.array([1, 0, 1], np.uint32).view(np.int32))
    out_off = torch.empty(4, dtype=torch.int64, device="cuda")
    out = torch.full((8,), 77, dtype=torch.uint8, device="cuda")
    total = C.c_uint64(0)
    rc = capi.lib().SpjGatherBinary(off.data_ptr(), 0, data.data_ptr(), 2, idx.data_ptr(), 3,
                                    out_off.data_ptr(), out.data_ptr(), 8, C.byref(total),
                                    None)
    assert rc == 28 and total.value == 13
    assert b"capacity" in capi.lib().SpjMaterializeLastError()
    assert out_off.cpu().tolist() == [0, 4, 9, 13]
    assert (out.cpu().numpy() == 77).all()


def test_gather_rejects_bad_width(mat):
    from sedona_gpuspatial import capi
    import torch
    v = torch.zeros(12, dtype=torch.uint8, device="cuda")
    i = torch.zeros(1, dtype=torch.int32, device="cuda")
    o = torch.zeros(12, dtype=torch.uint8, device="cuda")
    rc = capi.lib().SpjGatherFixed(v.data_ptr(), 3, 4, i.data_ptr(), 1, o.data_ptr(), None)
    assert rc == 22 and b"width" in capi.lib().SpjMaterializeLastError()


@pytest.mark.parametrize("n_rows", [0, 1, 31, 32, 33, 100000])
def test_visited_bitmap(mat, n_rows):
    rng = np.random.default_rng(n_rows)
    vb = mat.VisitedBitmap(n_rows)
    marked = np.zeros(n_rows, bool)
    for _ in range(3):  # several probe batches mark the same bitmap
        ids = rng.integers(0, max(n_rows, 1) + 3, rng.integers(0, 3 * n_rows + 2))
        ids = ids.astype(np.uint32)
        vb.mark(_t(ids.view(np.int32)))
        inb = ids[ids < n_rows]
        marked[inb] = True
    semi = vb.collect(True).cpu().numpy()
    anti = vb.collect(False).cpu().numpy()
    assert np.array_equal(semi, np.flatnonzero(marked).astype(np.int32))
    assert np.array_equal(anti, np.flatnonzero(~marked).astype(np.int32))
    bits = np.unpackbits(vb.bitmap().cpu().numpy(), bitorder="little")[:n_rows].astype(bool)
    assert np.array_equal(bits, marked)


def test_visited_collect_too_small(mat):
    import ctypes as C
    import torch
    from sedona_gpuspatial import capi
    vb = mat.VisitedBitmap(100)
    vb.mark(_t(np.array([3, 50, 99], np.int32)))
    out = torch.full((2,), -5, dtype=torch.int32, device="cuda")
    cnt = C.c_uint64(0)
    rc = capi.lib().SpjVisitedCollect(vb.words.data_ptr(), 100, 1, out.data_ptr(), 2,
                                      C.byref(cnt), None)
    assert rc == 28 and cnt.value == 3
    assert out.cpu().tolist() == [-5, -5]


def test_joined_batch_and_left_outer_join(mat, oracle_lib):
    """One probe of the fused join, its pairs left on the device, then the
    joined batch (build WKB + build id column + probe WKB) and the unmatched
    build rows of a left join, against the host restatement."""
    import torch
    from sedona_gpuspatial import capi, datagen
    inp = datagen.workload1(n_points=40000, n_polys=600)
    j = capi.SpatialJoin()
    j.build(inp.build)
    dcol, keep = gpu_util.device_column(capi, inp.probe)
    db, dp, n = j.probe_device(dcol, "intersects")
    torch.cuda.synchronize()
    b_np, p_np = gpu_util.device_pairs(db, dp, n)
    assert gpu_util.pairs(b_np, p_np) == gpu_util.pairs(
        *oracle_lib.join(oracle_lib.Geoms(inp.build), oracle_lib.Geoms(inp.probe),
                         "intersects", 0.0, nthreads=4))
    bi = torch.as_tensor(gpu_util._DevArray(db, n), device="cuda")
    pi = torch.as_tensor(gpu_util._DevArray(dp, n), device="cuda")
    build = mat.DeviceColumn(len(inp.build), offsets=_t(inp.build.offsets),
                             data=_t(inp.build.data))
    ids = mat.DeviceColumn(len(inp.build), values=_t(np.arange(len(inp.build), dtype=np.int64)))
    probe = mat.DeviceColumn(len(inp.probe), offsets=_t(inp.probe.offsets),
                             data=_t(inp.probe.data))
    cols = mat.build_joined_columns([build, ids], [probe], bi, pi)
    exp_b = inp.build.take(b_np.astype(np.int64))
    exp_p = inp.probe.take(p_np.astype(np.int64))
    assert np.array_equal(cols[0].offsets.cpu().numpy(), exp_b.offsets.astype(np.int64))
    assert np.array_equal(cols[0].data.cpu().numpy(), exp_b.data)
    assert np.array_equal(cols[1].values.cpu().numpy(), b_np.astype(np.int64))
    assert np.array_equal(cols[2].offsets.cpu().numpy(), exp_p.offsets.astype(np.int64))
    assert np.array_equal(cols[2].data.cpu().numpy(), exp_p.data)
    assert all(c.null_count == 0 for c in cols)
    # left join: unmatched build rows, probe side all null
    vb = mat.VisitedBitmap(len(inp.build))
    vb.mark(bi)
    un = vb.collect(False)
    exp_un = np.setdiff1d(np.arange(len(inp.build)), b_np)
    assert np.array_equal(un.cpu().numpy(), exp_un.astype(np.int32))
    nulls = torch.full((un.numel(),), -1, dtype=torch.int32, device="cuda")
    tail = mat.build_joined_columns([ids], [probe], un, nulls)
    assert np.array_equal(tail[0].values.cpu().numpy(), exp_un.astype(np.int64))
    assert tail[1].null_count == un.numel()
    assert int(tail[1].offsets[-1]) == 0
    del keep
