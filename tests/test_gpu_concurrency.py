"""Concurrent callers through the reference ABI.

The reference's provider shares one SedonaFloatIndex2D and one
SedonaSpatialRefiner between its probe partitions and calls probe and refine
from probe_threads_count threads at once, each probe with its own
SedonaSpatialIndexContext
(rust/sedona-spatial-join-gpu/src/index/gpu_spatial_index_builder.rs:165).
Here four host threads do the same on one GPU (ctypes releases the GIL for the
calls): every thread's pairs must equal the oracle's, and a probe that fails
in one thread's context (its callback returns non-zero) must leave an error
in that context only.
"""
import ctypes as C
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    from sedona_gpuspatial import _build, capi
    _build.build()
    return capi


def test_four_threads_probe_and_refine_one_index(capi):
    import oracle
    from sedona_gpuspatial import datagen
    oracle.build(with_ref=False)
    inp = datagen.workload1(n_points=40000, n_polys=800)
    B = oracle.Geoms(inp.build)
    build_boxes = B.boxes(1)
    idx = capi.FloatIndex2D(concurrency=4)
    idx.push_build(build_boxes)
    idx.finish_building()
    ref = capi.Refiner(concurrency=4)
    ref.init_build_schema()
    ref.push_build(inp.build)
    ref.finish_building()

    nthreads, rounds = 4, 3
    parts = np.array_split(np.arange(len(inp.probe)), nthreads)
    expected = []
    for rows in parts:
        col = inp.probe.take(rows)
        ob, op = oracle.join(B, oracle.Geoms(col), "intersects", nthreads=2)
        expected.append(sorted(zip(op.tolist(), ob.tolist())))
    probe_cols = [inp.probe.take(rows) for rows in parts]
    probe_boxes = [oracle.Geoms(c).boxes(1) for c in probe_cols]

    start = threading.Barrier(nthreads)
    results, errors = {}, []

    def worker(t):
        try:
            for r in range(rounds):
                start.wait()
                cb, cp = idx.probe(probe_boxes[t])
                b, p = ref.refine(probe_cols[t], "intersects", cb, cp)
                results[(t, r)] = sorted(zip(p.tolist(), b.tolist()))
        except Exception as e:  # surfaced by the main thread
            errors.append((t, repr(e)))

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(nthreads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join(timeout=600)
    assert not errors, errors
    for t in range(nthreads):
        for r in range(rounds):
            assert results[(t, r)] == expected[t], (t, r)


def test_probe_errors_stay_in_their_context(capi):
    """Two threads probe one index at once: one with a null rect buffer (an
    error, EINVAL with a message in its own context), the other normally
    (pairs delivered, no message in its context).  A callback that returns
    non-zero stops the probe and its value comes back unchanged, as in the
    reference (c/sedona-libgpuspatial/libgpuspatial/src/gpuspatial_c.cc:191-213)."""
    rng = np.random.default_rng(3)
    xy = rng.uniform(0, 100, (2000, 2)).astype(np.float32)
    boxes = np.concatenate([xy, xy + 2.0], 1)
    idx = capi.FloatIndex2D(concurrency=2)
    idx.push_build(boxes)
    idx.finish_building()
    probes = np.ascontiguousarray(np.concatenate([xy[:500] - 1.0, xy[:500] + 1.0], 1),
                                  dtype=np.float32)
    good_ctx, bad_ctx = capi.SedonaSpatialIndexContext(), capi.SedonaSpatialIndexContext()
    idx.idx.create_context(C.byref(good_ctx))
    idx.idx.create_context(C.byref(bad_ctx))
    try:
        seen = {"good": 0}
        go = threading.Barrier(2)
        rcs = {}

        def ok_cb(b, p, n, _ud):
            seen["good"] += n
            return 0

        ok_c = capi.PROBE_CB(ok_cb)

        def run(name, ctx, buf):
            go.wait()
            rcs[name] = idx.idx.probe(C.byref(idx.idx), C.byref(ctx), buf, len(probes), ok_c,
                                      None)

        good_buf = probes.ctypes.data_as(C.POINTER(C.c_float))
        null_buf = C.POINTER(C.c_float)()
        ths = [threading.Thread(target=run, args=("good", good_ctx, good_buf)),
               threading.Thread(target=run, args=("bad", bad_ctx, null_buf))]
        for th in ths:
            th.start()
        for th in ths:
            th.join(timeout=300)
        assert rcs["good"] == 0 and seen["good"] > 0
        assert rcs["bad"] == 22
        assert b"null" in idx.idx.context_get_last_error(C.byref(bad_ctx))
        assert idx.idx.context_get_last_error(C.byref(good_ctx)) in (b"", None)

        def stop_cb(b, p, n, _ud):
            return 7

        stop_c = capi.PROBE_CB(stop_cb)
        rc = idx.idx.probe(C.byref(idx.idx), C.byref(good_ctx), good_buf, len(probes), stop_c,
                           None)
        assert rc == 7
    finally:
        idx.idx.destroy_context(C.byref(good_ctx))
        idx.idx.destroy_context(C.byref(bad_ctx))
