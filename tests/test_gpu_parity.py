"""CUDA path vs the oracle (and the reference's own tg outcomes frozen in the
golden fixtures), through the C ABI.  Integer / index results must be
bit-exact: pair sets are compared as sorted (probe, build) lists."""
import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu

PREDS = ["intersects", "contains", "covers", "within", "coveredby", "touches", "equals"]


@pytest.fixture(scope="module")
def capi():
    from sedona_gpuspatial import _build, capi
    _build.build()
    return capi


@pytest.fixture(scope="module")
def oracle_mod():
    import oracle
    oracle.build(with_ref=False)
    return oracle


def pairs(b, p):
    return sorted(zip(np.asarray(p).tolist(), np.asarray(b).tolist()))


def oracle_pairs(oracle_mod, build, probe, pred, distance=0.0):
    ob, op = oracle_mod.join(oracle_mod.Geoms(build), oracle_mod.Geoms(probe), pred, distance,
                             nthreads=4)
    return pairs(ob, op)


# ---------------------------------------------------------------------------
# fused join (SpjJoin): workload-shaped inputs at small sizes

@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("pred", PREDS)
def test_point_in_polygon_join(capi, oracle_mod, form, pred):
    from sedona_gpuspatial import datagen
    inp = datagen.workload1(n_points=30000, n_polys=500)
    j = capi.SpatialJoin(refine_form=form)
    j.build(inp.build)
    b, p = j.probe(inp.probe, pred)
    assert pairs(b, p) == oracle_pairs(oracle_mod, inp.build, inp.probe, pred)


def _staircase_rings():
    # integer-vertex rings with 24 to 80 segments (cell grids are built from
    # 12 segments up): a staircase, a comb with 1-wide teeth, and a diamond
    st = [(0, 0)]
    for k in range(12):
        st += [(k + 1, k), (k + 1, k + 1)]
    st += [(0, 12), (0, 0)]
    comb = [(0, 0), (40, 0), (40, 3)]
    for k in range(19, -1, -1):
        comb += [(2 * k + 1, 3), (2 * k + 1, 10), (2 * k, 10), (2 * k, 3)] if k else [(1, 3), (1, 10), (0, 10)]
    comb += [(0, 0)]
    dia = [(20, 0), (40, 20), (20, 40), (0, 20), (20, 0)]
    dia = [tuple(np.array(a) + (np.array(b) - np.array(a)) * t / 8) for a, b in zip(dia[:-1], dia[1:])
           for t in range(8)] + [(20, 0)]
    return [st, comb, dia]


@pytest.mark.parametrize("pred", PREDS)
def test_cell_grid_edges_vertices_and_cell_boundaries(capi, oracle_mod, pred):
    """Points on edges, on vertices, on grid-cell boundaries and strictly
    inside / outside many-segment integer rings: the FP32 form with cell
    grids (and without) against the oracle, and polygon-polygon pairs whose
    boxes sit in clean cells or straddle edges."""
    from sedona_gpuspatial import wkb
    rings = _staircase_rings()
    build = wkb.column_from_values([wkb.wkb_polygon([np.array(r, dtype=np.float64)]) for r in rings])
    g = np.arange(-1, 41.5, 0.25)
    px, py = [a.ravel() for a in np.meshgrid(g, g)]
    probe = wkb.points_column(px, py)
    exp = oracle_pairs(oracle_mod, build, probe, pred)
    for grid in (1, 0):
        j = capi.SpatialJoin(refine_form=1)
        j.set_option("cell_grid", grid)
        j.build(build)
        b, p = j.probe(probe, pred)
        assert pairs(b, p) == exp, grid
    if pred == "intersects":
        rng = np.random.default_rng(9)
        sq = []
        for _ in range(3000):
            x, y = rng.integers(-2, 42, 2) / 2.0
            w = rng.integers(0, 5) / 2.0 + 0.25
            sq.append(wkb.wkb_polygon([np.array([(x, y), (x + w, y), (x + w, y + w), (x, y + w),
                                                 (x, y)])]))
        probe2 = wkb.column_from_values(sq)
        exp2 = oracle_pairs(oracle_mod, build, probe2, "intersects")
        for grid in (1, 0):
            j = capi.SpatialJoin(refine_form=1)
            j.set_option("cell_grid", grid)
            j.build(build)
            assert pairs(*j.probe(probe2, "intersects")) == exp2, grid


@pytest.mark.parametrize("form", [0, 1])
def test_polygon_polygon_intersects(capi, oracle_mod, form):
    from sedona_gpuspatial import datagen
    inp = datagen.workload2(n_buildings=20000, n_zones=300)
    j = capi.SpatialJoin(refine_form=form)
    j.build(inp.build)
    b, p = j.probe(inp.probe, "intersects")
    exp = oracle_pairs(oracle_mod, inp.build, inp.probe, "intersects")
    assert len(exp) > 1000
    assert pairs(b, p) == exp


RELATIONS = ["contains", "within", "covers", "coveredby", "touches", "equals", "intersects"]


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("pred", RELATIONS)
def test_polygon_polygon_relations_zones_build(capi, oracle_mod, form, pred):
    """Workload-2 shape with the zones as the build side: SQL
    ST_Within(building, zone) reaches the refiner as contains(zone, building)
    (pred(build, probe), rust/sedona-query-planner/src/spatial_predicate.rs:218-230)."""
    from sedona_gpuspatial import datagen
    inp = datagen.workload2(n_buildings=20000, n_zones=300)
    j = capi.SpatialJoin(refine_form=form)
    j.build(inp.build)
    b, p = j.probe(inp.probe, pred)
    exp = oracle_pairs(oracle_mod, inp.build, inp.probe, pred)
    if pred in ("contains", "covers", "intersects"):
        assert len(exp) > 100
    assert pairs(b, p) == exp


@pytest.mark.parametrize("pred", ["within", "coveredby", "touches", "intersects"])
def test_polygon_polygon_relations_buildings_build(capi, oracle_mod, pred):
    """The same shapes with the buildings as the build side: within(building,
    zone) evaluates tg's ring-in-ring test the other way round."""
    from sedona_gpuspatial import datagen
    inp = datagen.workload2(n_buildings=8000, n_zones=200)
    j = capi.SpatialJoin()
    j.build(inp.probe)
    b, p = j.probe(inp.build, pred)
    exp = oracle_pairs(oracle_mod, inp.probe, inp.build, pred)
    if pred != "touches":
        assert len(exp) > 50
    assert pairs(b, p) == exp


def test_contains_stream_batches(capi, oracle_mod):
    """Workload-3 shape: probe batches of uneven size, probe ids offset by the
    batch start (probe_base), concatenated in probe order."""
    from sedona_gpuspatial import datagen
    inp = datagen.workload3(n_points=60000, n_zones=400)
    j = capi.SpatialJoin()
    j.build(inp.build)
    got = []
    start = 0
    rng = np.random.default_rng(5)
    while start < len(inp.probe):
        n = int(min(len(inp.probe) - start, rng.integers(1000, 9000)))
        b, p = j.probe(inp.probe.slice(start, start + n), "contains", probe_base=start)
        assert np.all(np.diff(p.astype(np.int64)) >= 0)  # ascending probe order
        got += pairs(b, p)
        start += n
    assert sorted(got) == oracle_pairs(oracle_mod, inp.build, inp.probe, "contains")


@pytest.mark.parametrize("form", [0, 1])
def test_dwithin(capi, oracle_mod, form):
    from sedona_gpuspatial import datagen
    inp = datagen.workload4(n_probe=20000, n_build=20000)
    j = capi.SpatialJoin(refine_form=form)
    j.build(inp.build)
    b, p = j.probe(inp.probe, "dwithin", distance=250.0)
    exp = oracle_pairs(oracle_mod, inp.build, inp.probe, "dwithin", 250.0)
    assert len(exp) > 10000
    assert pairs(b, p) == exp


@pytest.mark.parametrize("order", [-1, 1])
def test_dwithin_fused_same_output(capi, oracle_mod, order):
    """ST_DWithin decided inside the traversal (fuse_dwithin) writes the same
    pairs at the same positions as filter + refine + compact, and matches the
    oracle, including pairs exactly at the distance (Pythagorean triples)."""
    from sedona_gpuspatial import datagen, wkb
    inp = datagen.workload4(n_probe=20000, n_build=20000)
    out = {}
    # (fuse_dwithin, dwithin_slots, dwithin_arena): result slots of the
    # counting pass and its overflow arena (of the slots' size, at least 1024
    # chunks); with few slots the arena runs out and the probes it could not
    # hold are traversed again by the scatter pass, without it every probe
    # past its slots is
    variants = [(0, 64, 1), (1, 64, 1), (1, 64, 0), (1, 4, 1), (1, 1, 1), (1, 4, 0), (1, 0, 1),
                (1, 64, 2)]
    for v in variants:
        j = capi.SpatialJoin(probe_order=order)
        j.set_option("fuse_dwithin", v[0])
        j.set_option("dwithin_slots", v[1])
        j.set_option("dwithin_arena", v[2])
        j.build(inp.build)
        out[v] = j.probe(inp.probe, "dwithin", distance=250.0)
        assert j.stats()["kernel_launches"] > 0
    for v in variants[1:]:
        np.testing.assert_array_equal(out[v][0], out[variants[0]][0])
        np.testing.assert_array_equal(out[v][1], out[variants[0]][1])
    assert pairs(*out[(1, 64, 1)]) == oracle_pairs(oracle_mod, inp.build, inp.probe, "dwithin",
                                                   250.0)
    bx = np.array([0, 3, 5, 8, 20, 7, 24], dtype=np.float64)
    by = np.array([0, 4, 12, 15, 21, 24, 7], dtype=np.float64)
    build = wkb.points_column(bx, by)
    probe = wkb.points_column(np.array([0.0, 10.0]), np.array([0.0, 3.0]))
    j = capi.SpatialJoin(probe_order=order)
    j.set_option("fuse_dwithin", 1)
    j.build(build)
    for d in (5.0, 13.0, 17.0, 25.0, 29.0, 4.999999999999999):
        b, p = j.probe(probe, "dwithin", distance=d)
        assert pairs(b, p) == oracle_pairs(oracle_mod, build, probe, "dwithin", d), d


@pytest.mark.parametrize("shape", ["pip", "polygons", "dwithin"])
def test_probe_order_keeps_pairs_and_layout(capi, oracle_mod, shape):
    """Traversal in Morton order of the probe boxes (probe_order=1) writes the
    same pairs at the same positions as traversal in row order (-1)."""
    from sedona_gpuspatial import datagen
    if shape == "pip":
        inp, pred, d = datagen.workload1(n_points=40000, n_polys=500), "within", 0.0
    elif shape == "polygons":
        inp, pred, d = datagen.workload2(n_buildings=20000, n_zones=300), "intersects", 0.0
    else:
        inp, pred, d = datagen.workload4(n_probe=20000, n_build=20000), "dwithin", 250.0
    out = {}
    # (probe_order, candidate_order, refine_min_blocks, cell_grid, refine_split)
    variants = [(-1, 0, 4, 0, 0), (1, 2, 6, 1, 0), (1, 3, 0, 1, 1), (0, 2, 0, 1, 1),
                (-1, 0, 4, 1, 1), (1, 2, 6, 0, 1), (1, 3, 0, 1, 2), (-1, 0, 0, 1, 2),
                (-1, 2, 4, 0, 1), (1, 0, 6, 1, 1), (1, 2, 6, 1, 3), (-1, 0, 4, 1, 3)]
    for v in variants:
        j = capi.SpatialJoin(probe_order=v[0])
        j.set_option("candidate_order", v[1])
        j.set_option("refine_min_blocks", v[2])
        j.set_option("cell_grid", v[3])
        j.set_option("refine_split", v[4])
        j.build(inp.build)
        out[v] = j.probe(inp.probe, pred, distance=d)
    for v in variants[1:]:
        np.testing.assert_array_equal(out[v][0], out[variants[0]][0])
        np.testing.assert_array_equal(out[v][1], out[variants[0]][1])
    assert pairs(*out[variants[0]]) == oracle_pairs(oracle_mod, inp.build, inp.probe, pred, d)


@pytest.mark.parametrize("tiles", [1, 3, 6, 10])
def test_order_tiles_same_pairs(capi, oracle_mod, tiles):
    """Build-major order within tiles of the Morton-ordered candidate list
    (each tile sorted in place by the segmented radix sort) refines a
    permutation of the candidates: the same pairs at the same positions as
    the candidates taken as listed."""
    from sedona_gpuspatial import datagen
    inp = datagen.workload2(n_buildings=30000, n_zones=400)
    out = {}
    for order, t in [(0, 0), (2, tiles)]:
        j = capi.SpatialJoin(probe_order=1)
        j.set_option("candidate_order", order)
        j.set_option("order_tiles", t)
        j.build(inp.build)
        out[t] = j.probe(inp.probe, "intersects")
    np.testing.assert_array_equal(out[tiles][0], out[0][0])
    np.testing.assert_array_equal(out[tiles][1], out[0][1])
    assert pairs(*out[0]) == oracle_pairs(oracle_mod, inp.build, inp.probe, "intersects", 0.0)


def test_unknown_option_is_an_error(capi):
    j = capi.SpatialJoin()
    with pytest.raises(capi.GpuSpatialError, match="unknown option"):
        j.set_option("no_such_option", 1)
    with pytest.raises(capi.GpuSpatialError, match="refine_min_blocks"):
        j.set_option("refine_min_blocks", 1)


def test_dwithin_exact_boundary(capi, oracle_mod):
    """Integer Pythagorean triples put pairs exactly at distance d."""
    from sedona_gpuspatial import wkb
    bx = np.array([0, 3, 5, 8, 20, 7, 24], dtype=np.float64)
    by = np.array([0, 4, 12, 15, 21, 24, 7], dtype=np.float64)
    build = wkb.points_column(bx, by)
    probe = wkb.points_column(np.array([0.0, 10.0]), np.array([0.0, 3.0]))
    j = capi.SpatialJoin()
    j.build(build)
    for d in (5.0, 13.0, 17.0, 25.0, 29.0, 4.999999999999999):
        b, p = j.probe(probe, "dwithin", distance=d)
        assert pairs(b, p) == oracle_pairs(oracle_mod, build, probe, "dwithin", d), d


@pytest.mark.parametrize("form", [0, 1])
def test_knn(capi, oracle_mod, form):
    from sedona_gpuspatial import datagen
    inp = datagen.workload4(n_probe=5000, n_build=40000)
    bx, by = _points(oracle_mod, inp.build)
    px, py = _points(oracle_mod, inp.probe)
    kj = capi.KnnJoin(refine_form=form)
    kj.build(bx, by)
    idx, dist = kj.query(px, py, 8)
    oi, od = oracle_mod.knn(oracle_mod.Geoms(inp.build), oracle_mod.Geoms(inp.probe), 8, nthreads=4)
    assert np.array_equal(idx, oi)
    np.testing.assert_allclose(dist, od, rtol=1e-12, atol=0)


@pytest.mark.parametrize("case", ["lattice", "offset", "huge"])
@pytest.mark.parametrize("k", [1, 5, 12, 20])
def test_knn_split_pass_cases(capi, oracle_mod, case, k):
    """The split-FP32 pass against the oracle where it must hand probes to the
    exact kernel: exact distance ties on an integer lattice (ties at rank k),
    points 1e-3 apart at 1e5 offsets (the hi/lo split carries the digits FP32
    alone loses), and coordinates beyond the split range (exact kernel)."""
    from sedona_gpuspatial import wkb
    rng = np.random.default_rng(11 + k)
    if case == "lattice":
        g = np.arange(60, dtype=np.float64)
        bx, by = [a.ravel() for a in np.meshgrid(g, g)]
        px = rng.integers(0, 120, 3000) / 2.0
        py = rng.integers(0, 120, 3000) / 2.0
    elif case == "offset":
        bx = 1e5 + rng.uniform(0, 3.0, 4000).round(3)
        by = -1e5 + rng.uniform(0, 3.0, 4000).round(3)
        px = 1e5 + rng.uniform(0, 3.0, 3000)
        py = -1e5 + rng.uniform(0, 3.0, 3000)
    else:
        bx = rng.uniform(-1e20, 1e20, 3000)
        by = rng.uniform(-1e20, 1e20, 3000)
        px = rng.uniform(-1e20, 1e20, 1000)
        py = rng.uniform(-1e20, 1e20, 1000)
    kj = capi.KnnJoin(refine_form=1)
    kj.build(bx, by)
    idx, dist = kj.query(px, py, k)
    oi, od = oracle_mod.knn(oracle_mod.Geoms(wkb.points_column(bx, by)),
                            oracle_mod.Geoms(wkb.points_column(px, py)), k, nthreads=4)
    assert np.array_equal(idx, oi)
    np.testing.assert_allclose(dist, od, rtol=1e-12, atol=0)


def test_knn_ties_by_row_id(capi, oracle_mod):
    from sedona_gpuspatial import wkb
    # duplicated build points: equal distances must come back in row order
    bx = np.array([1.0, 1.0, 2.0, 1.0, -1.0, 0.0, 0.0]); by = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 1.0, -1.0])
    kj = capi.KnnJoin()
    kj.build(bx, by)
    idx, dist = kj.query(np.array([0.0]), np.array([0.0]), 6)
    oi, od = oracle_mod.knn(oracle_mod.Geoms(wkb.points_column(bx, by)),
                            oracle_mod.Geoms(wkb.points_column(np.array([0.0]), np.array([0.0]))), 6)
    assert idx.tolist() == oi.tolist()
    assert idx[0].tolist()[:6] == [0, 1, 3, 4, 5, 6]


def test_knn_k_larger_than_build(capi):
    kj = capi.KnnJoin()
    kj.build(np.array([0.0, 1.0]), np.array([0.0, 0.0]))
    idx, dist = kj.query(np.array([0.2]), np.array([0.0]), 4)
    assert idx[0].tolist() == [0, 1, 0xFFFFFFFF, 0xFFFFFFFF]
    assert np.isinf(dist[0, 2:]).all()


def _points(oracle_mod, col):
    g = oracle_mod.Geoms(col)
    import ctypes as C
    L = oracle_mod.lib()
    x = np.empty(len(col)); y = np.empty(len(col))
    xx, yy = C.c_double(), C.c_double()
    for i in range(len(col)):
        L.spjo_point(g.ptr, i, C.byref(xx), C.byref(yy))
        x[i], y[i] = xx.value, yy.value
    return x, y


# ---------------------------------------------------------------------------
# golden fixtures: the reference's own tg outcomes, through the refiner ABI

@pytest.mark.parametrize("name", list(golden_io.SHAPES))
@pytest.mark.parametrize("form", [0, 1])
def test_refiner_matches_reference_tg_golden(capi, name, form):
    z, cols = golden_io.load()
    preds, brows, prows, exp = golden_io.cube(z, cols, name)
    bname, pname = golden_io.SHAPES[name]
    j = capi.SpatialJoin(refine_form=form)
    j.build(cols[bname])
    probe = cols[pname]
    for k, code in enumerate(preds):
        pred = [n for n, c in capi.PREDICATES.items() if c == code][0]
        if pred == "disjoint":
            continue  # not a join predicate (the planner never plans it)
        b, p = j.probe(probe, pred)
        got = np.zeros((len(cols[bname]), len(probe)), dtype=np.uint8)
        got[b, p] = 1
        sub = got[np.ix_(brows, prows)]
        bad = np.argwhere(sub != exp[k])
        assert len(bad) == 0, (pred, [(int(brows[i]), int(prows[j])) for i, j in bad[:5]])


def test_refiner_abi_known_answer(capi):
    """gpu_spatial_index.rs:647-746 through index probe + refiner refine:
    3 squares x 4 points -> probe indices [0, 2, 3]."""
    from sedona_gpuspatial import wkb
    squares = [[(0, 0), (10, 0), (10, 10), (0, 10), (0, 0)],
               [(20, 20), (30, 20), (30, 30), (20, 30), (20, 20)],
               [(40, 40), (50, 40), (50, 50), (40, 50), (40, 40)]]
    build = wkb.column_from_values([wkb.wkb_polygon([[(float(x), float(y)) for x, y in s]])
                                    for s in squares])
    pts = [(5, 5), (15, 15), (25, 25), (45, 45)]
    probe = wkb.column_from_values([wkb.wkb_point(float(x), float(y)) for x, y in pts])
    idx = capi.FloatIndex2D()
    idx.push_build(np.array([[0, 0, 10, 10], [20, 20, 30, 30], [40, 40, 50, 50]], np.float32))
    idx.finish_building()
    cb, cp = idx.probe(np.array([[x, y, x, y] for x, y in pts], np.float32))
    ref = capi.Refiner()
    ref.init_build_schema()
    ref.push_build(build)
    ref.finish_building()
    b, p = ref.refine(probe, "intersects", cb, cp)
    assert p.tolist() == [0, 2, 3]
    assert b.tolist() == [0, 1, 2]


def test_index_matches_rect_join(capi, oracle_mod):
    """index_test.cu:52-86 recipe: mt19937-style uniform boxes in
    [-180,180], sizes U(0,100), box-box and point-box."""
    rng = np.random.default_rng(0)

    def boxes(n, points=False):
        x = rng.uniform(-180, 180, n); y = rng.uniform(-180, 180, n)
        w = 0 if points else rng.uniform(0, 100, n)
        h = 0 if points else rng.uniform(0, 100, n)
        return np.stack([x, y, x + w, y + h], 1).astype(np.float32)

    for nb, npb, pts in [(1, 1, False), (7, 100, False), (1000, 3000, False), (5000, 8192, True),
                         (8192, 1000, False)]:
        B, P = boxes(nb), boxes(npb, pts)
        idx = capi.FloatIndex2D()
        idx.push_build(B[: nb // 2])
        idx.push_build(B[nb // 2:])  # two pushes concatenate
        idx.finish_building()
        b, p = idx.probe(P)
        ob, op = oracle_mod.rect_join(B, P, nthreads=4)
        assert pairs(b, p) == pairs(ob, op), (nb, npb)


def test_index_empty_and_nan(capi):
    idx = capi.FloatIndex2D()
    idx.finish_building()
    b, p = idx.probe(np.array([[0, 0, 1, 1]], np.float32))
    assert len(b) == 0
    idx2 = capi.FloatIndex2D()
    idx2.push_build(np.array([[np.nan] * 4, [0, 0, 1, 1]], np.float32))
    idx2.finish_building()
    b, p = idx2.probe(np.array([[0.5, 0.5, 0.5, 0.5], [np.nan] * 4], np.float32))
    assert b.tolist() == [1] and p.tolist() == [0]


def test_nulls_empties_bigendian_large_binary(capi, oracle_mod):
    from sedona_gpuspatial import wkb
    sq = [[(0.0, 0.0), (4.0, 0.0), (4.0, 4.0), (0.0, 4.0), (0.0, 0.0)]]
    build_vals = [wkb.wkb_polygon(sq), None, wkb.wkb_polygon(sq, big_endian=True),
                  wkb.wkb_polygon([]), wkb.wkb_multipolygon([sq, [[(10.0, 10.0), (12.0, 10.0),
                                                                   (12.0, 12.0), (10.0, 10.0)]]])]
    probe_vals = [wkb.wkb_point(1, 1), None, wkb.wkb_point(float("nan"), float("nan")),
                  wkb.wkb_point(11.5, 10.5, big_endian=True), wkb.wkb_point(4, 2)]
    for large in (False, True):
        build = wkb.column_from_values(build_vals, large=large)
        probe = wkb.column_from_values(probe_vals, large=large)
        j = capi.SpatialJoin()
        j.build(build)
        for pred in ("intersects", "contains", "covers"):
            b, p = j.probe(probe, pred)
            assert pairs(b, p) == oracle_pairs(oracle_mod, build, probe, pred), (large, pred)


def test_sliced_arrow_array(capi, oracle_mod):
    """A probe array with a non-zero Arrow offset (a slice of a batch)."""
    from sedona_gpuspatial import capi as c, datagen
    inp = datagen.workload1(n_points=5000, n_polys=200)
    j = capi.SpatialJoin()
    j.build(inp.build)
    a = c.ArrowBinary(inp.probe, offset=1000, length=2000)
    import ctypes as C
    out = {}

    def cb(b, p, n, _):
        out["b"] = np.ctypeslib.as_array(b, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
        out["p"] = np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
        return 0

    rc = c.lib().SpjJoinProbeArrow(j.h, C.byref(a.schema), C.byref(a.array), 5, 0.0, 0,
                                   c.JOIN_CB(cb), None)
    assert rc == 0
    exp = oracle_pairs(oracle_mod, inp.build, inp.probe.slice(1000, 3000), "intersects")
    assert pairs(out["b"], out["p"]) == exp


def test_malformed_wkb_reports_row(capi):
    from sedona_gpuspatial import wkb
    good = wkb.wkb_point(1, 1)
    bad = good[:10]  # truncated
    j = capi.SpatialJoin()
    j.build(wkb.column_from_values([wkb.wkb_polygon([[(0.0, 0.0), (2.0, 0.0), (2.0, 2.0), (0.0, 0.0)]])]))
    with pytest.raises(capi.GpuSpatialError, match="row 1"):
        j.probe(wkb.column_from_values([good, bad, good]), "intersects")
    # the object stays usable after the error
    b, p = j.probe(wkb.column_from_values([good]), "intersects")
    assert p.tolist() == [0]


def test_empty_probe_and_build(capi):
    from sedona_gpuspatial import wkb
    j = capi.SpatialJoin()
    j.build(wkb.column_from_values([]))
    b, p = j.probe(wkb.column_from_values([wkb.wkb_point(0, 0)]), "intersects")
    assert len(b) == 0
    j2 = capi.SpatialJoin()
    j2.build(wkb.column_from_values([wkb.wkb_point(0, 0)]))
    b, p = j2.probe(wkb.column_from_values([]), "intersects")
    assert len(b) == 0


# ---------------------------------------------------------------------------
# batched probe stream (one CUDA-graph replay over uneven record batches)

def _device_batches(capi, col, sizes):
    import torch
    keep, dcols = [], []
    start = 0
    for n in sizes:
        part = col.slice(start, start + n)
        off = torch.from_numpy(np.ascontiguousarray(part.offsets)).cuda()
        data = torch.from_numpy(np.ascontiguousarray(part.data)).cuda()
        keep.append((off, data))
        dcols.append(capi.SpjDeviceWkb(length=n, offsets=off.data_ptr(),
                                       offsets_are_64bit=int(part.offsets.dtype == np.int64),
                                       data=data.data_ptr(), data_length=len(part.data),
                                       validity=None, validity_offset=0))
        start += n
    return dcols, keep


class _DevArray:
    """A raw device pointer exposed through __cuda_array_interface__."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (ptr, False),
                                         "version": 3, "strides": None}


def _device_pairs(db, dp, n):
    import torch
    if n == 0:
        return np.zeros(0, np.uint32), np.zeros(0, np.uint32)
    torch.cuda.synchronize()
    b = torch.as_tensor(_DevArray(db, n), device="cuda").cpu().numpy().view(np.uint32)
    p = torch.as_tensor(_DevArray(dp, n), device="cuda").cpu().numpy().view(np.uint32)
    return b, p


@pytest.mark.parametrize("params", [None, (128, 256, 2), (256, 8192, 8)])
def test_stream_matches_oracle(capi, oracle_mod, params):
    from sedona_gpuspatial import datagen
    inp = datagen.workload3(n_points=80000, n_zones=400)
    j = capi.SpatialJoin()
    j.build(inp.build)
    rng = np.random.default_rng(9)
    sizes, left = [], len(inp.probe)
    while left:
        s = int(min(left, np.floor(np.exp(rng.uniform(np.log(64), np.log(20000))))))
        sizes.append(s)
        left -= s
    dcols, keep = _device_batches(capi, inp.probe, sizes)
    st = capi.StreamProbe(j)
    if params:
        st.set_params(*params)
    st.set_batches(dcols)
    exp = oracle_pairs(oracle_mod, inp.build, inp.probe, "contains")
    for _ in range(2):  # two replays of the same graph
        db, dp, n = st.run("contains")
        b, p = _device_pairs(db, dp, n)
        assert np.all(np.diff(p.astype(np.int64)) >= 0)
        assert pairs(b, p) == exp


def test_stream_probe_order_same_arrays(capi):
    """From 65,536 rows the stream graph traverses and refines the rows in
    Morton order; the pairs and their positions must equal the unordered
    graph's (probe_order = -1)."""
    from sedona_gpuspatial import datagen
    inp = datagen.workload3(n_points=150000, n_zones=600, seed=3)
    rng = np.random.default_rng(4)
    sizes, left = [], len(inp.probe)
    while left:
        s = int(min(left, rng.integers(100, 30000)))
        sizes.append(s)
        left -= s
    dcols, keep = _device_batches(capi, inp.probe, sizes)
    out = {}
    for po in (-1, 0, 1):
        j = capi.SpatialJoin(probe_order=po)
        j.build(inp.build)
        st = capi.StreamProbe(j)
        st.set_batches(dcols)
        for pred in ("contains", "intersects"):
            db, dp, n = st.run(pred)
            out[(po, pred)] = _device_pairs(db, dp, n)
    for pred in ("contains", "intersects"):
        for po in (0, 1):
            np.testing.assert_array_equal(out[(po, pred)][0], out[(-1, pred)][0])
            np.testing.assert_array_equal(out[(po, pred)][1], out[(-1, pred)][1])


def test_stream_autotune_and_cache(capi, oracle_mod, tmp_path):
    from sedona_gpuspatial import datagen
    inp = datagen.workload3(n_points=20000, n_zones=200)
    j = capi.SpatialJoin()
    j.build(inp.build)
    dcols, keep = _device_batches(capi, inp.probe, [5000, 7000, 8000])
    st = capi.StreamProbe(j)
    st.set_batches(dcols)
    cache = str(tmp_path / "tune.txt")
    best = st.autotune("intersects", cache)
    assert best[0] in (64, 128, 256) and best[2] in (2, 4, 8)
    assert best == st.autotune("intersects", cache)  # served from the cache
    db, dp, n = st.run("intersects")
    b, p = _device_pairs(db, dp, n)
    assert pairs(b, p) == oracle_pairs(oracle_mod, inp.build, inp.probe, "intersects")


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("name", golden_io.FIXTURE_JOINS)
def test_reference_fixtures(capi, form, name):
    """The reference's own test data (c/sedona-libgpuspatial/libgpuspatial/
    test/data: natural-earth countries, multipolygons with holes, and their
    generated points; the synthetic PIP and polygon sets) through the fused
    join, against the pair sets the reference's tg returns for each
    predicate (tests/golden/gen_fixtures.py)."""
    build, probe, exp = golden_io.load_fixtures()[name]
    j = capi.SpatialJoin(refine_form=form)
    j.build(build)
    for pred, want in exp.items():
        b, p = j.probe(probe, pred)
        assert pairs(b, p) == want, pred


@pytest.mark.parametrize("k", [1, 4, 8])
def test_knn_tie_breakers(capi, k):
    """include_tie_breakers (rust/sedona-spatial-join/src/index/
    default_spatial_index.rs:378-470): on an integer lattice with probes on
    the lattice and half-lattice, many build points tie at the k-th
    distance; each probe gets its k nearest by (distance, row id), then every
    other point within 1e-9 of the k-th distance (brute force in FP64)."""
    g = np.arange(30.0)
    bx, by = [a.ravel() for a in np.meshgrid(g, g)]
    rng = np.random.default_rng(9)
    px = rng.integers(-4, 64, 300) / 2.0
    py = rng.integers(-4, 64, 300) / 2.0
    kj = capi.KnnJoin()
    kj.build(bx, by)
    off, idx, dist = kj.query_ties(px, py, k, True)
    ids = np.arange(len(bx))
    extra = 0
    for i in range(len(px)):
        d = np.hypot(px[i] - bx, py[i] - by)
        order = np.lexsort((ids, d))
        kth = d[order[k - 1]]
        exp = set(order[:k].tolist()) | set(np.nonzero(d - kth <= 1e-9)[0].tolist())
        got = idx[off[i]:off[i + 1]]
        assert got[:k].tolist() == order[:k].tolist(), i
        assert len(got) == len(exp) and set(got.tolist()) == exp, i
        np.testing.assert_allclose(dist[off[i]:off[i + 1]], d[got], rtol=1e-12, atol=0)
        extra += len(got) - k
    assert extra > 0  # the lattice does produce ties
    off0, idx0, _ = kj.query_ties(px, py, k, False)
    ri, _ = kj.query(px, py, k)
    assert np.array_equal(np.diff(off0), np.full(len(px), k))
    assert np.array_equal(idx0.reshape(-1, k), ri)


def test_knn_wkb_column(capi, oracle_mod):
    """query_knn over a WKB point column decoded on the device; empty (POINT
    EMPTY) and null rows get no results, as in the reference
    (default_spatial_index.rs:331-339)."""
    from sedona_gpuspatial import wkb
    rng = np.random.default_rng(10)
    bx, by = rng.uniform(0, 100, 5000), rng.uniform(0, 100, 5000)
    px, py = rng.uniform(-5, 105, 700), rng.uniform(-5, 105, 700)
    vals = [wkb.wkb_point(float(x), float(y)) for x, y in zip(px, py)]
    vals[3] = None
    vals[10] = wkb.wkb_point(float("nan"), float("nan"))
    vals[11] = wkb.wkb_point(float(px[11]), float(py[11]), big_endian=True)
    kj = capi.KnnJoin()
    kj.build(bx, by)
    off, idx, dist = kj.query_wkb(wkb.column_from_values(vals), 6)
    assert off[4] - off[3] == 0 and off[11] - off[10] == 0
    keep = [i for i in range(len(vals)) if i not in (3, 10)]
    B = oracle_mod.Geoms(wkb.points_column(bx, by))
    P = oracle_mod.Geoms(wkb.points_column(px[keep], py[keep]))
    ob, od = oracle_mod.knn(B, P, 6, nthreads=4)
    for r, i in enumerate(keep):
        assert idx[off[i]:off[i + 1]].tolist() == ob[r].tolist(), i
        np.testing.assert_allclose(dist[off[i]:off[i + 1]], od[r], rtol=1e-12, atol=0)
    poly = wkb.wkb_polygon([[(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 0.0)]])
    with pytest.raises(capi.GpuSpatialError, match="points"):
        kj.query_wkb(wkb.column_from_values([vals[0], poly]), 2)


@pytest.mark.parametrize("form", [0, 1])
def test_dwithin_with_polygons(capi, oracle_mod, form):
    """ST_DWithin between points and polygons and between polygons: the
    reference's build.distance_ext(probe) <= d (refine/geo.rs:312-321, the
    distances of sedona-geo-generic-alg's euclidean/utils.rs), probe rects
    expanded by d; point build sides against polygon probes too."""
    from sedona_gpuspatial import datagen
    inp = datagen.workload1(n_points=20000, n_polys=300)
    for build, probe, d in ((inp.build, inp.probe, 2.0), (inp.probe, inp.build, 1.5)):
        j = capi.SpatialJoin(refine_form=form)
        j.build(build)
        b, p = j.probe(probe, "dwithin", distance=d)
        exp = oracle_pairs(oracle_mod, build, probe, "dwithin", d)
        assert len(exp) > 100
        assert pairs(b, p) == exp
    inp2 = datagen.workload2(n_buildings=4000, n_zones=80)
    j = capi.SpatialJoin(refine_form=form)
    j.build(inp2.build)
    b, p = j.probe(inp2.probe, "dwithin", distance=120.0)
    exp = oracle_pairs(oracle_mod, inp2.build, inp2.probe, "dwithin", 120.0)
    assert len(exp) > 100
    assert pairs(b, p) == exp


def test_dwithin_distance_column(capi, oracle_mod):
    """A distance per probe row (operand_evaluator.rs:556-627): point pairs
    (decided inside the traversal) and polygon pairs, with null (NaN) and
    negative distances matching nothing."""
    from sedona_gpuspatial import datagen
    rng = np.random.default_rng(21)
    inp = datagen.workload4(n_probe=20000, n_build=20000)
    d = rng.uniform(0, 400, len(inp.probe))
    d[::17] = np.nan
    d[5::23] = -1.0
    j = capi.SpatialJoin()
    j.build(inp.build)
    j.set_probe_distances(d)
    b, p = j.probe(inp.probe, "dwithin", distance=0.0)
    ob, op = oracle_mod.join_dists(oracle_mod.Geoms(inp.build), oracle_mod.Geoms(inp.probe), d,
                                   nthreads=4)
    assert len(ob) > 1000
    assert pairs(b, p) == pairs(ob, op)
    j.set_probe_distances(None)
    b2, p2 = j.probe(inp.probe, "dwithin", distance=100.0)
    assert pairs(b2, p2) == oracle_pairs(oracle_mod, inp.build, inp.probe, "dwithin", 100.0)
    inp1 = datagen.workload1(n_points=10000, n_polys=200)
    dp = rng.uniform(0, 3, len(inp1.probe))
    dp[::11] = np.nan
    j1 = capi.SpatialJoin()
    j1.build(inp1.build)
    j1.set_probe_distances(dp)
    b, p = j1.probe(inp1.probe, "dwithin", distance=0.0)
    ob, op = oracle_mod.join_dists(oracle_mod.Geoms(inp1.build), oracle_mod.Geoms(inp1.probe),
                                   dp, nthreads=4)
    assert pairs(b, p) == pairs(ob, op)
    with pytest.raises(capi.GpuSpatialError, match="distance column"):
        j1.probe(inp1.probe.slice(0, 100), "dwithin", distance=0.0)
