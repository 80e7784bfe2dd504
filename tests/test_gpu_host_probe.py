"""Host-buffer probe (SpjJoinProbeHost).  A column of at least 2 x 262,144
rows is cut into row slices that are probed on two workspaces in turn, with
the copies of the neighbouring slices in flight; it must return exactly the
pairs, in the same order, that one call over the whole column returns."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    from sedona_gpuspatial import _build, capi
    _build.build()
    return capi


def _with_nulls(col, seed, frac=0.01):
    from sedona_gpuspatial.wkb import WkbColumn
    keep = np.random.default_rng(seed).random(len(col)) >= frac
    return WkbColumn(col.offsets, col.data, np.packbits(keep, bitorder="little"))


def _inputs(shape):
    from sedona_gpuspatial import datagen
    if shape == "points":
        inp = datagen.workload1(n_points=700_000, n_polys=3_000, seed=7)
        return inp.build, inp.probe, inp.predicate, 0.0
    if shape == "polygons":
        inp = datagen.workload2(n_buildings=600_000, n_zones=2_000, seed=7)
        return inp.build, inp.probe, inp.predicate, 0.0
    inp = datagen.workload4(n_probe=800_000, n_build=40_000, seed=7)
    return inp.build, inp.probe, "dwithin", 250.0


@pytest.mark.parametrize("shape", ["points", "polygons", "dwithin"])
@pytest.mark.parametrize("large_offsets", [False, True])
def test_sliced_host_probe_same_pairs_and_order(capi, shape, large_offsets):
    from sedona_gpuspatial.wkb import WkbColumn
    build, probe, pred, d = _inputs(shape)
    probe = _with_nulls(probe, seed=3)
    if large_offsets:
        probe = WkbColumn(probe.offsets.astype(np.int64), probe.data, probe.validity)
    j = capi.SpatialJoin()
    j.build(build)
    ref_b, ref_p = j.probe(probe, pred, distance=d, probe_base=5)
    assert len(ref_b) > 0
    cap = len(ref_b) + 100
    ob = np.full(cap, 0xFFFFFFFF, np.uint32)
    op = np.full(cap, 0xFFFFFFFF, np.uint32)
    n = j.probe_host(probe, pred, d, ob, op, probe_base=5)
    assert n == len(ref_b)
    np.testing.assert_array_equal(ob[:n], ref_b)
    np.testing.assert_array_equal(op[:n], ref_p)
    assert (ob[n:] == 0xFFFFFFFF).all() and (op[n:] == 0xFFFFFFFF).all()
    # again on the same join: the second workspace is reused
    n2 = j.probe_host(probe, pred, d, ob, op, probe_base=5)
    assert n2 == n
    np.testing.assert_array_equal(op[:n], ref_p)


@pytest.mark.parametrize("slices", [1, 3, 64])
def test_host_probe_slice_counts(capi, slices):
    build, probe, pred, d = _inputs("polygons")
    probe = probe.slice(0, 200_000)
    j = capi.SpatialJoin()
    j.set_option("host_slices", slices)
    j.build(build)
    ref_b, ref_p = j.probe(probe, pred, distance=d)
    ob = np.zeros(len(ref_b) + 1, np.uint32)
    op = np.zeros(len(ref_b) + 1, np.uint32)
    n = j.probe_host(probe, pred, d, ob, op)
    assert n == len(ref_b)
    np.testing.assert_array_equal(ob[:n], ref_b)
    np.testing.assert_array_equal(op[:n], ref_p)


def test_sliced_host_probe_capacity_error(capi):
    build, probe, pred, d = _inputs("points")
    j = capi.SpatialJoin()
    j.build(build)
    ref_b, _ = j.probe(probe, pred)
    small = len(ref_b) // 2
    ob = np.zeros(small, np.uint32)
    op = np.zeros(small, np.uint32)
    with pytest.raises(capi.GpuSpatialError, match=f"need {len(ref_b)} pairs"):
        j.probe_host(probe, pred, d, ob, op)
    # the join still answers afterwards
    ob = np.zeros(len(ref_b), np.uint32)
    op = np.zeros(len(ref_b), np.uint32)
    assert j.probe_host(probe, pred, d, ob, op) == len(ref_b)
    np.testing.assert_array_equal(ob, ref_b)
