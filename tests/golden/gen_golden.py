"""Generate the golden predicate fixtures from the reference's own tg library.

Run in a container where the reference tree is mounted:

    SPJ_REFERENCE_TREE=/path/to/sedona-db python tests/golden/gen_golden.py

It compiles the reference's vendored tg (c/sedona-tg/src/tg/tg.c) through
oracle/Makefile into oracle/_ref/, evaluates tg_geom_<pred>(build, probe) on
seeded degenerate and random inputs, and writes tests/golden/tg_predicates.npz:
the WKB columns plus the expected 0/1 outcome per (pred, build, probe) triple.
The argument order follows the reference refiner
(rust/sedona-spatial-join/src/refine/tg.rs:322-357).  The fixtures let the
oracle and the CUDA path be pinned to the reference on machines without the
reference tree.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "sedona-db_gb300"))

import oracle  # noqa: E402
from sedona_gpuspatial import wkb  # noqa: E402

PREDS = ["equals", "disjoint", "touches", "contains", "covers", "intersects", "within",
         "coveredby"]


def build_cases(seed=20260101):
    rng = np.random.default_rng(seed)

    def rand_ring(n, grid):
        pts = [(float(rng.integers(0, grid)), float(rng.integers(0, grid))) for _ in range(n)]
        return pts + [pts[0]]

    polys = []
    # integer-grid rings: shared vertices, collinear edges, self-intersections
    for _ in range(120):
        polys.append(wkb.wkb_polygon([rand_ring(int(rng.integers(3, 8)), 6)]))
    # axis-aligned rectangles (horizontal and vertical edges)
    for _ in range(40):
        x0, y0 = rng.integers(0, 5, 2)
        w, h = rng.integers(1, 4, 2)
        r = [(x0, y0), (x0 + w, y0), (x0 + w, y0 + h), (x0, y0 + h), (x0, y0)]
        polys.append(wkb.wkb_polygon([[(float(a), float(b)) for a, b in r]]))
    # polygons with a hole, and multipolygons (for point predicates)
    holed = []
    for _ in range(20):
        x0, y0 = rng.integers(0, 3, 2)
        outer = [(x0, y0), (x0 + 4, y0), (x0 + 4, y0 + 4), (x0, y0 + 4), (x0, y0)]
        hole = [(x0 + 1, y0 + 1), (x0 + 1, y0 + 3), (x0 + 3, y0 + 3), (x0 + 3, y0 + 1),
                (x0 + 1, y0 + 1)]
        holed.append(wkb.wkb_polygon([[(float(a), float(b)) for a, b in outer],
                                      [(float(a), float(b)) for a, b in hole]]))
    for _ in range(20):
        parts = [[rand_ring(int(rng.integers(3, 6)), 6)] for _ in range(int(rng.integers(1, 4)))]
        holed.append(wkb.wkb_multipolygon(parts))
    # big-endian encodings of a few shapes
    for _ in range(10):
        polys.append(wkb.wkb_polygon([rand_ring(5, 6)], big_endian=True))
    # star polygons with random FP64 coordinates
    for _ in range(30):
        n = int(rng.integers(8, 40))
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        rad = rng.uniform(0.6, 1.0, n) * 2.0
        cx, cy = rng.uniform(1, 5, 2)
        ring = [(cx + r * np.cos(a), cy + r * np.sin(a)) for a, r in zip(ang, rad)]
        ring.append(ring[0])
        polys.append(wkb.wkb_polygon([ring]))

    pts = [wkb.wkb_point(x / 2.0, y / 2.0) for x in range(0, 13) for y in range(0, 13)]
    pts += [wkb.wkb_point(float(rng.uniform(0, 6)), float(rng.uniform(0, 6)))
            for _ in range(150)]
    pts += [wkb.wkb_point(1.0, 2.0, big_endian=True)]
    return polys, holed, pts


def build_relate_cases(seed=20260202):
    """Polygons and multipolygons for the polygon-polygon relations
    (contains / within / covers / coveredby / touches / equals, holes on both
    sides): shapes on a small integer grid that share edges, corners and
    whole rings, nest inside each other and inside holes, in both windings,
    plus generic FP64 stars and rings of 32+ points (which tg indexes)."""
    rng = np.random.default_rng(seed)
    out = []

    def rect(x0, y0, x1, y1):
        return [(float(x0), float(y0)), (float(x1), float(y0)), (float(x1), float(y1)),
                (float(x0), float(y1)), (float(x0), float(y0))]

    def rev(ring):
        return list(reversed(ring))

    def rotate(ring, k):
        body = ring[:-1]
        body = body[k:] + body[:k]
        return body + [body[0]]

    # rectangles on a 0..8 grid (shared edges and corners are common)
    for _ in range(50):
        x0, y0 = rng.integers(0, 7, 2)
        x1 = x0 + rng.integers(1, 4)
        y1 = y0 + rng.integers(1, 4)
        r = rect(x0, y0, x1, y1)
        out.append(wkb.wkb_polygon([rev(r) if rng.random() < 0.3 else r]))
    # polygons with one or two holes, what fills each hole exactly, and what
    # sits strictly inside or touches the hole's boundary from inside
    for _ in range(14):
        x0, y0 = rng.integers(0, 3, 2)
        outer = rect(x0, y0, x0 + 6, y0 + 6)
        hx, hy = x0 + rng.integers(1, 3), y0 + rng.integers(1, 3)
        hw, hh = rng.integers(1, 3), rng.integers(1, 3)
        hole = rect(hx, hy, hx + hw, hy + hh)
        rings = [outer, rev(hole) if rng.random() < 0.5 else hole]
        if rng.random() < 0.4 and hy + hh + 2 <= y0 + 5:
            rings.append(rect(hx, hy + hh + 1, hx + 1, hy + hh + 2))
        out.append(wkb.wkb_polygon(rings))
        out.append(wkb.wkb_polygon([hole]))
        out.append(wkb.wkb_polygon([rect(hx, hy, hx + hw, hy + 0.5 * hh)]))
        out.append(wkb.wkb_polygon([[(hx + 0.25 * hw, hy + 0.25 * hh),
                                     (hx + 0.75 * hw, hy + 0.25 * hh),
                                     (hx + 0.5 * hw, hy + 0.75 * hh),
                                     (hx + 0.25 * hw, hy + 0.25 * hh)]]))
    # concave L / U shapes
    for _ in range(14):
        x0, y0 = rng.integers(0, 5, 2)
        a, b = rng.integers(2, 4, 2)
        if rng.random() < 0.5:
            ring = [(x0, y0), (x0 + a, y0), (x0 + a, y0 + 1), (x0 + 1, y0 + 1), (x0 + 1, y0 + b),
                    (x0, y0 + b), (x0, y0)]
        else:
            ring = [(x0, y0), (x0 + 3, y0), (x0 + 3, y0 + b), (x0 + 2, y0 + b), (x0 + 2, y0 + 1),
                    (x0 + 1, y0 + 1), (x0 + 1, y0 + b), (x0, y0 + b), (x0, y0)]
        ring = [(float(x), float(y)) for x, y in ring]
        out.append(wkb.wkb_polygon([rev(ring) if rng.random() < 0.5 else ring]))
    # triangles (convex) in both windings, with vertices on edges of others
    for _ in range(20):
        pts = [(float(rng.integers(0, 9)), float(rng.integers(0, 9))) for _ in range(3)]
        out.append(wkb.wkb_polygon([pts + [pts[0]]]))
    # the same shape again: identical, another start vertex, reversed
    base = [wkb.wkb_polygon([rect(1, 1, 4, 3)]), wkb.wkb_polygon([rect(2, 2, 5, 6)])]
    out += base
    out.append(wkb.wkb_polygon([rotate(rect(1, 1, 4, 3), 2)]))
    out.append(wkb.wkb_polygon([rev(rect(2, 2, 5, 6))]))
    out.append(wkb.wkb_polygon([rect(1, 1, 4, 3)]))
    # multipolygons: touching, disjoint and overlapping rectangle parts, a
    # part with a hole, parts equal to single polygons above, empty parts
    for _ in range(18):
        parts = []
        for _ in range(int(rng.integers(2, 4))):
            x0, y0 = rng.integers(0, 7, 2)
            parts.append([rect(x0, y0, x0 + rng.integers(1, 3), y0 + rng.integers(1, 3))])
        if rng.random() < 0.3:
            parts.append([rect(0, 0, 6, 6), rect(2, 2, 4, 4)])
        out.append(wkb.wkb_multipolygon(parts))
    out.append(wkb.wkb_multipolygon([[rect(1, 1, 4, 3)], [rect(2, 2, 5, 6)]]))
    out.append(wkb.wkb_multipolygon([[rect(1, 1, 4, 3)], []]))
    out.append(wkb.wkb_multipolygon([[], [rect(0, 0, 2, 2)], [rect(2, 0, 4, 2)]]))
    # generic FP64 stars, some large (32+ points: tg builds its ring index)
    for _ in range(16):
        n = int(rng.integers(6, 60))
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        rad = rng.uniform(0.5, 1.0, n) * rng.uniform(1.0, 3.5)
        cx, cy = rng.uniform(1, 7, 2)
        ring = [(float(cx + r * np.cos(t)), float(cy + r * np.sin(t))) for t, r in zip(ang, rad)]
        ring.append(ring[0])
        out.append(wkb.wkb_polygon([rev(ring) if rng.random() < 0.5 else ring]))
    # regular polygons (convex, building-like) with FP64 vertices
    for _ in range(10):
        n = int(rng.integers(4, 13))
        rot = rng.uniform(0, 2 * np.pi)
        r = rng.uniform(0.3, 2.0)
        cx, cy = rng.uniform(1, 7, 2)
        ring = [(float(cx + r * np.cos(rot + 2 * np.pi * k / n)),
                 float(cy + r * np.sin(rot + 2 * np.pi * k / n))) for k in range(n)]
        ring.append(ring[0])
        out.append(wkb.wkb_polygon([ring]))
    # integer-grid rings (self-intersections, collinear and repeated points)
    for _ in range(16):
        pts = [(float(rng.integers(0, 7)), float(rng.integers(0, 7)))
               for _ in range(int(rng.integers(3, 8)))]
        out.append(wkb.wkb_polygon([pts + [pts[0]]]))
    # a 40-point circle with a 36-point hole (indexed rings on both levels)
    ring = [(4.0 + 3.5 * np.cos(2 * np.pi * k / 40), 4.0 + 3.5 * np.sin(2 * np.pi * k / 40))
            for k in range(40)]
    hole = [(4.0 + 1.5 * np.cos(2 * np.pi * k / 36), 4.0 + 1.5 * np.sin(2 * np.pi * k / 36))
            for k in range(36)]
    out.append(wkb.wkb_polygon([ring + [ring[0]], hole + [hole[0]]]))
    out.append(wkb.wkb_polygon([hole + [hole[0]]]))
    return out


def main():
    oracle.build(with_ref=True)
    assert oracle.ref_available(), "reference tg could not be built"
    polys, holed, pts = build_cases()
    rel = build_relate_cases()
    out = {}

    def col_arrays(prefix, values):
        c = wkb.column_from_values(values)
        out[prefix + "_offsets"] = c.offsets.astype(np.int64)
        out[prefix + "_data"] = c.data

    col_arrays("polys", polys)
    col_arrays("holed", holed)
    col_arrays("pts", pts)
    col_arrays("rel", rel)

    def table(name, build, probe, preds, stride_b=1, stride_p=1, index=3):
        """Dense outcome cube [pred, build row, probe row] over the strided
        rows, stored bit-packed; row i of the cube is build row i*stride_b."""
        res = []
        for pred in preds:
            for i in range(0, len(build), stride_b):
                for j in range(0, len(probe), stride_p):
                    r = oracle.ref_predicate(build[i], probe[j], pred, index)
                    assert r in (0, 1), (pred, i, j, r)
                    if index != 3 and (i + j) % 3 == 0:
                        # the natural index and the reference refiner's
                        # default (y-stripes) decide alike
                        assert oracle.ref_predicate(build[i], probe[j], pred, 1) == r
                    res.append(r)
        out[name + "_preds"] = np.array([oracle.PRED[p] for p in preds], dtype=np.int32)
        out[name + "_stride"] = np.array([stride_b, stride_p], dtype=np.int32)
        out[name + "_res"] = np.packbits(np.array(res, dtype=np.uint8), bitorder="little")
        out[name + "_count"] = np.array([len(res)], dtype=np.int64)

    # polygon build x point probe: every predicate (C1/C3 shape)
    table("poly_point", polys, pts, PREDS, 1, 2)
    # holed / multipolygon build x point probe
    table("holed_point", holed, pts, PREDS, 1, 1)
    # polygon x polygon: intersects (C2 shape)
    table("poly_poly", polys, polys, ["intersects"], 1, 1)
    # point build x polygon probe (C5 shape: range box probe)
    table("point_poly", pts, polys, ["intersects", "within", "coveredby", "touches"], 3, 2)
    # point x point
    table("point_point", pts, pts, ["intersects", "equals", "contains", "touches"], 7, 5)
    # polygon-polygon relations under the reference refiner's default ring
    # index (y-stripes, rust/sedona-common/src/option.rs:213): every predicate
    table("rel_rel", rel, rel, PREDS, 1, 1, index=2)
    table("poly_poly_all", polys, polys, PREDS, 1, 1, index=2)
    table("rel_point", rel, pts, PREDS, 1, 2, index=2)
    table("point_rel", pts, rel, PREDS, 3, 1, index=2)

    # raycast / segment-intersection known answers on integer grids
    rng = np.random.default_rng(7)
    segs = rng.integers(0, 4, size=(4000, 6)).astype(np.float64)
    segs[:, 4:] += rng.integers(0, 2, size=(4000, 2)) * 0.5
    segs = segs.astype(np.float32)  # exact: small halves
    rc = [oracle.ref().tgref_raycast(*map(float, s)) for s in segs]
    out["raycast_in"] = segs
    out["raycast_out"] = np.array(rc, dtype=np.int8)
    s2 = rng.integers(0, 4, size=(4000, 8)).astype(np.float32)
    si = [oracle.ref().tgref_segment_intersects(*map(float, s)) for s in s2]
    out["segx_in"] = s2
    out["segx_out"] = np.array(si, dtype=np.int8)

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tg_predicates.npz")
    np.savez_compressed(path, **out)
    sizes = {k: int(v[0]) for k, v in out.items() if k.endswith("_count")}
    print("wrote", path, os.path.getsize(path), "bytes", sizes)


if __name__ == "__main__":
    main()
