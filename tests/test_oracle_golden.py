"""The oracle restatement against the reference's own tg outcomes (golden
fixtures made by tests/golden/gen_golden.py) and known-answer cases."""
import numpy as np
import pytest

import golden_io


@pytest.fixture(scope="module")
def golden(oracle_lib):
    z, cols = golden_io.load()
    geoms = {k: oracle_lib.Geoms(v) for k, v in cols.items()}
    return z, cols, geoms


@pytest.mark.parametrize("name", list(golden_io.SHAPES))
def test_predicates_match_reference_tg(golden, oracle_lib, name):
    z, cols, geoms = golden
    preds, brows, prows, exp = golden_io.cube(z, cols, name)
    bname, pname = golden_io.SHAPES[name]
    L = oracle_lib.lib()
    bad = []
    for k, code in enumerate(preds):
        for a, i in enumerate(brows):
            for b, j in enumerate(prows):
                r = L.spjo_predicate(geoms[bname].ptr, int(i), geoms[pname].ptr, int(j), int(code))
                if r != exp[k, a, b]:
                    bad.append((int(code), int(i), int(j), r, int(exp[k, a, b])))
    assert not bad, bad[:10]


def test_golden_tables_hold_every_relation(golden):
    """The polygon-polygon tables carry positive outcomes for every predicate
    (so the parity above is not vacuous), and contains equals covers between
    polygons as in tg (tg_poly_contains_poly, tg.c:4094-4096)."""
    z, cols, _ = golden
    for name in ("rel_rel", "poly_poly_all"):
        preds, _, _, exp = golden_io.cube(z, cols, name)
        sums = {int(c): int(exp[k].sum()) for k, c in enumerate(preds)}
        assert all(v > 0 for v in sums.values()), (name, sums)
        assert sums[3] == sums[4] and sums[6] == sums[7], sums


def test_raycast_known_answers(golden, oracle_lib):
    z, _, _ = golden
    got = [oracle_lib.raycast(*map(float, s)) for s in z["raycast_in"]]
    assert np.array_equal(np.array(got), z["raycast_out"])


def test_segment_intersects_known_answers(golden, oracle_lib):
    z, _, _ = golden
    got = [oracle_lib.segment_intersects(*map(float, s)) for s in z["segx_in"]]
    assert np.array_equal(np.array(got), z["segx_out"])


def test_gpu_index_known_answer(oracle_lib):
    """rust/sedona-spatial-join-gpu/src/index/gpu_spatial_index.rs:647-746:
    three squares x four points -> 3 matches with probe indices [0, 2, 3]."""
    from sedona_gpuspatial import wkb
    squares = [[(0, 0), (10, 0), (10, 10), (0, 10), (0, 0)],
               [(20, 20), (30, 20), (30, 30), (20, 30), (20, 20)],
               [(40, 40), (50, 40), (50, 50), (40, 50), (40, 40)]]
    build = wkb.column_from_values([wkb.wkb_polygon([[(float(x), float(y)) for x, y in s]])
                                    for s in squares])
    probe = wkb.column_from_values([wkb.wkb_point(5, 5), wkb.wkb_point(15, 15),
                                    wkb.wkb_point(25, 25), wkb.wkb_point(45, 45)])
    b, p = oracle_lib.join(oracle_lib.Geoms(build), oracle_lib.Geoms(probe), "intersects")
    assert sorted(p.tolist()) == [0, 2, 3]
    assert sorted(zip(p.tolist(), b.tolist())) == [(0, 0), (2, 1), (3, 2)]


def test_outward_rounding(oracle_lib):
    """rust/sedona-spatial-join/src/utils/bounds.rs:164-351: f32 boxes enclose the f64 bounds."""
    from sedona_gpuspatial import wkb
    vals = [wkb.wkb_polygon([[(0.1, 0.2), (1e5 + 0.3, 0.2), (1e5 + 0.3, 7.7), (0.1, 0.2)]]),
            wkb.wkb_point(0.1, -0.3), None]
    g = oracle_lib.Geoms(wkb.column_from_values(vals))
    b = g.boxes(0)
    assert b[0, 0] <= 0.1 and b[0, 2] >= 1e5 + 0.3 and b[0, 1] <= 0.2 and b[0, 3] >= 7.7
    assert np.float64(b[1, 0]) <= 0.1 <= np.float64(b[1, 2])
    assert np.isnan(b[2]).all()
    rn = g.boxes(1)  # GPU factory: points round to nearest, degenerate
    assert rn[1, 0] == np.float32(0.1) and rn[1, 2] == np.float32(0.1)


def test_rect_join_matches_bruteforce(oracle_lib):
    rng = np.random.default_rng(0)
    # index_test.cu:52-86 recipe: coords U(-180,180), box size U(0,100)
    def boxes(n):
        x = rng.uniform(-180, 180, n); y = rng.uniform(-180, 180, n)
        w = rng.uniform(0, 100, n); h = rng.uniform(0, 100, n)
        return np.stack([x, y, x + w, y + h], 1).astype(np.float32)
    B, P = boxes(700), boxes(500)
    P[::7, 2] = P[::7, 0]; P[::7, 3] = P[::7, 1]  # some points
    b, p = oracle_lib.rect_join(B, P, nthreads=3)
    hit = ~((B[None, :, 0] > P[:, None, 2]) | (B[None, :, 2] < P[:, None, 0]) |
            (B[None, :, 1] > P[:, None, 3]) | (B[None, :, 3] < P[:, None, 1]))
    pp, bb = np.nonzero(hit)
    assert np.array_equal(p, pp) and np.array_equal(b, bb)


def test_knn_bruteforce(oracle_lib):
    from sedona_gpuspatial import wkb
    rng = np.random.default_rng(3)
    bx = np.round(rng.uniform(0, 100, 3000), 1); by = np.round(rng.uniform(0, 100, 3000), 1)
    px = np.round(rng.uniform(-10, 110, 400), 1); py = np.round(rng.uniform(-10, 110, 400), 1)
    B = oracle_lib.Geoms(wkb.points_column(bx, by)); P = oracle_lib.Geoms(wkb.points_column(px, py))
    ob, od = oracle_lib.knn(B, P, 8, nthreads=2)
    for i in range(0, 400, 13):
        d = np.hypot(px[i] - bx, py[i] - by)
        order = np.lexsort((np.arange(len(bx)), d))[:8]
        assert np.array_equal(ob[i], order.astype(np.uint32))
        assert np.array_equal(od[i], d[order])


@pytest.mark.parametrize("case", ["offset", "lattice"])
def test_knn_bruteforce_cell_edges_and_ties(oracle_lib, case):
    """Points at 1e5 offsets on a 1e-3 lattice (outward f32 boxes straddle
    grid cells, so one point sits in several cells) and exact distance ties
    on an integer lattice: each build row at most once, ties by row id."""
    from sedona_gpuspatial import wkb
    rng = np.random.default_rng(8)
    if case == "offset":
        bx = 1e5 + rng.uniform(0, 3.0, 4000).round(3)
        by = -1e5 + rng.uniform(0, 3.0, 4000).round(3)
        px = 1e5 + rng.uniform(0, 3.0, 300)
        py = -1e5 + rng.uniform(0, 3.0, 300)
    else:
        g = np.arange(40, dtype=np.float64)
        bx, by = [a.ravel() for a in np.meshgrid(g, g)]
        px = rng.integers(0, 80, 300) / 2.0
        py = rng.integers(0, 80, 300) / 2.0
    B = oracle_lib.Geoms(wkb.points_column(bx, by)); P = oracle_lib.Geoms(wkb.points_column(px, py))
    for k in (1, 5, 12, 20):
        ob, od = oracle_lib.knn(B, P, k, nthreads=2)
        for i in range(0, 300, 7):
            d = np.hypot(px[i] - bx, py[i] - by)
            order = np.lexsort((np.arange(len(bx)), d))[:k]
            assert np.array_equal(ob[i], order.astype(np.uint32)), (case, k, i)
            assert np.array_equal(od[i], d[order])


def test_dwithin_bruteforce(oracle_lib):
    from sedona_gpuspatial import wkb
    rng = np.random.default_rng(4)
    bx = rng.uniform(0, 100, 2000); by = rng.uniform(0, 100, 2000)
    px = rng.uniform(0, 100, 300); py = rng.uniform(0, 100, 300)
    B = oracle_lib.Geoms(wkb.points_column(bx, by)); P = oracle_lib.Geoms(wkb.points_column(px, py))
    b, p = oracle_lib.join(B, P, "dwithin", distance=3.0, nthreads=2)
    d = np.hypot(bx[None, :] - px[:, None], by[None, :] - py[:, None])
    pp, bb = np.nonzero(d <= 3.0)
    assert np.array_equal(p, pp) and np.array_equal(b, bb)


@pytest.mark.parametrize("name", ["countries_points", "pip_points", "poly_poly",
                                  "countries_countries"])
def test_oracle_matches_reference_fixtures(oracle_lib, name):
    """The reference's own test data (natural-earth countries with their
    generated points, the synthetic PIP and polygon sets): the oracle's join
    returns the pair set the reference's tg returns for every predicate."""
    build, probe, exp = golden_io.load_fixtures()[name]
    B, P = oracle_lib.Geoms(build), oracle_lib.Geoms(probe)
    assert exp
    for pred, pairs in exp.items():
        b, p = oracle_lib.join(B, P, pred, nthreads=4)
        assert sorted(zip(p.tolist(), b.tolist())) == pairs, pred


def test_geo_distance_known_answers(oracle_lib):
    """build.distance_ext(probe) as restated from the reference's
    sedona-geo-generic-alg (euclidean/utils.rs): point-polygon, polygon-
    polygon, a polygon inside another's hole, multipolygons."""
    from sedona_gpuspatial import wkb

    def sq(x0, y0, x1, y1):
        return [(x0, y0), (x1, y0), (x1, y1), (x0, y1), (x0, y0)]

    build = wkb.column_from_values([
        wkb.wkb_polygon([sq(0.0, 0.0, 1.0, 1.0)]),
        wkb.wkb_polygon([sq(0.0, 0.0, 10.0, 10.0), sq(2.0, 2.0, 8.0, 8.0)]),
        wkb.wkb_multipolygon([[sq(0.0, 0.0, 1.0, 1.0)], [sq(5.0, 0.0, 6.0, 1.0)]]),
        wkb.wkb_point(0.0, 0.0),
    ])
    probe = wkb.column_from_values([
        wkb.wkb_point(3.0, 0.5), wkb.wkb_point(0.5, 0.5), wkb.wkb_point(4.0, 5.0),
        wkb.wkb_polygon([sq(3.0, 0.0, 4.0, 1.0)]), wkb.wkb_polygon([sq(4.0, 4.0, 5.0, 6.0)]),
        wkb.wkb_point(3.0, 4.0),
    ])
    B, P = oracle_lib.Geoms(build), oracle_lib.Geoms(probe)
    d = lambda b, p: oracle_lib.geo_distance(B, b, P, p)  # noqa: E731
    assert d(0, 0) == 2.0 and d(0, 1) == 0.0 and d(0, 3) == 2.0
    assert d(1, 2) == 2.0            # a point in the hole: 2 to the hole's edge
    assert d(1, 4) == 2.0            # a polygon inside the hole: 2 to the hole's edge
    assert d(2, 0) == 2.0 and d(2, 3) == 1.0   # the nearest part of a multipolygon
    assert d(3, 5) == 5.0            # points: hypot
    b, p = oracle_lib.join_dists(B, P, np.array([2.0, 0.0, 0.5, 1.0, 2.0, 4.0]), nthreads=2)
    got = sorted(zip(p.tolist(), b.tolist()))
    assert (0, 0) in got and (1, 0) in got and (4, 1) in got and (3, 2) in got
    assert (5, 3) not in got and (3, 0) not in got
