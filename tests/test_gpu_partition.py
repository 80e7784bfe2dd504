"""The partitioned (out-of-core) join (SpjJoinPartitioned): its pair set
against the oracle and against the one-pass join, every pair delivered once,
and its partitioning against the reference's rules restated in
partition_ref.py (the KDB tree from the same sample, partition_no_multi for
the build rows, the flat partitioner over the partitions' bounds for the
probe rows)."""
import numpy as np
import pytest

import gpu_util
import partition_ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    from sedona_gpuspatial import _build, capi
    _build.build()
    return capi


def _oracle_pairs(oracle_lib, build, probe, pred, distance=0.0):
    ob, op = oracle_lib.join(oracle_lib.Geoms(build), oracle_lib.Geoms(probe), pred, distance,
                             nthreads=4)
    return gpu_util.pairs(ob, op)


def _inputs(kind):
    from sedona_gpuspatial import datagen
    if kind == "pip":
        return datagen.workload1(n_points=60000, n_polys=800)
    if kind == "polys":
        return datagen.workload2(n_buildings=40000, n_zones=600)
    return datagen.workload4(n_probe=40000, n_build=20000)


@pytest.mark.parametrize("host_gather", [False, True])
@pytest.mark.parametrize("parts", [1, 4, 16])
@pytest.mark.parametrize("kind,pred", [("pip", "intersects"), ("polys", "intersects"),
                                       ("polys", "contains"), ("points", "dwithin")])
def test_partitioned_pairs_match_oracle(capi, oracle_lib, kind, pred, parts, host_gather):
    inp = _inputs(kind)
    d = float(inp.params.get("distance", 0.0)) if pred == "dwithin" else 0.0
    j = capi.SpatialJoin()
    b, p, st = j.join_partitioned(inp.build, inp.probe, pred, d, num_partitions=parts,
                                  seed=7, host_gather=host_gather)
    got = gpu_util.pairs(b, p)
    assert len(got) == len(set(got)), "a pair delivered twice"
    assert got == _oracle_pairs(oracle_lib, inp.build, inp.probe, pred, d)
    assert st["pairs"] == len(got)
    if parts > 1:
        assert st["partitions"] > 1
    if host_gather:
        assert st["direct_host_reads"] == 0


def test_partitioning_follows_reference_rules(capi, oracle_lib):
    inp = _inputs("polys")
    j = capi.SpatialJoin()
    j.join_partitioned(inp.build, inp.probe, "intersects", num_partitions=12, sample_rows=3000,
                       seed=3, record_layout=True)
    L = j.partition_layout()
    # the tree: rebuilt from the exported sample with the same parameters
    kdb = partition_ref.Kdb(L["max_items"], L["max_levels"], L["extent"])
    for r in L["samples"]:
        kdb.insert(r)
    leaves = kdb.leaves()
    assert np.array_equal(leaves, L["leaves"])
    assert L["max_items"] == max(1, len(L["samples"]) // 12) and L["max_levels"] == 12
    bbox = oracle_lib.Geoms(inp.build).boxes(1)
    pbox = oracle_lib.Geoms(inp.probe).boxes(1)
    ext = np.array([np.nanmin(bbox[:, 0]), np.nanmin(bbox[:, 1]), np.nanmax(bbox[:, 2]),
                    np.nanmax(bbox[:, 3])], np.float32)
    assert np.array_equal(L["extent"], ext)
    # build rows: partition_no_multi
    assert np.array_equal(L["build_part"], partition_ref.no_multi(bbox, leaves))
    # bounds: the union of each partition's build boxes
    for k in range(len(leaves)):
        sel = bbox[L["build_part"] == k]
        if len(sel):
            exp = [sel[:, 0].min(), sel[:, 1].min(), sel[:, 2].max(), sel[:, 3].max()]
            assert np.array_equal(L["bounds"][k], np.array(exp, np.float32))
        else:
            assert np.isnan(L["bounds"][k]).all()
    # probe rows: the flat partitioner over the bounds (NaN bounds meet nothing)
    assert np.array_equal(L["probe_part"], partition_ref.flat(pbox, L["bounds"]))


def test_partitioned_edge_cases(capi, oracle_lib):
    from sedona_gpuspatial import datagen, wkb
    inp = datagen.workload1(n_points=5000, n_polys=100)
    j = capi.SpatialJoin()
    empty = wkb.WkbColumn(np.zeros(1, np.int32), np.zeros(0, np.uint8))
    b, p, st = j.join_partitioned(empty, inp.probe, "intersects", num_partitions=4)
    assert len(b) == 0 and st["passes"] == 0
    b, p, st = j.join_partitioned(inp.build, empty, "intersects", num_partitions=4)
    assert len(b) == 0
    # nulls on both sides, and more partitions than sampled rows
    rng = np.random.default_rng(5)
    bv = np.packbits(rng.random(len(inp.build)) > 0.3, bitorder="little")
    pv = np.packbits(rng.random(len(inp.probe)) > 0.3, bitorder="little")
    B = wkb.WkbColumn(inp.build.offsets, inp.build.data, bv)
    P = wkb.WkbColumn(inp.probe.offsets, inp.probe.data, pv)
    b, p, st = j.join_partitioned(B, P, "intersects", num_partitions=64, sample_rows=50)
    assert gpu_util.pairs(b, p) == _oracle_pairs(oracle_lib, B, P, "intersects")
    assert st["probe_rows_none"] >= int((~np.unpackbits(pv, bitorder="little")[:len(P)]
                                         .astype(bool)).sum())


def test_partitioned_budget_and_callback_stop(capi):
    import ctypes as C
    from sedona_gpuspatial import datagen
    inp = datagen.workload1(n_points=50000, n_polys=2000)
    j = capi.SpatialJoin()
    # a budget below the build side's size gives several partitions
    b, p, st = j.join_partitioned(inp.build, inp.probe, "intersects",
                                  build_budget_bytes=inp.build.nbytes // 2)
    assert st["partitions"] >= 2
    # a callback that returns non-zero stops the join with its value
    keep = []

    def host(col):
        off = np.ascontiguousarray(col.offsets)
        data = np.ascontiguousarray(col.data)
        keep.extend([off, data])
        return capi.SpjHostWkb(len(col), off.ctypes.data, 0, data.ctypes.data, None, 0)

    hb, hp = host(inp.build), host(inp.probe)
    calls = []

    def cb(bb, pp, n, _ud):
        calls.append(n)
        return 9

    rc = capi.lib().SpjJoinPartitioned(j.h, C.byref(hb), C.byref(hp), 5, 0.0,
                                       C.byref(capi.SpjPartitionOptions(8, 0, 0, 0, 0, 0)),
                                       capi.JOIN_CB(cb), None, None)
    assert rc == 9 and len(calls) == 1
