"""Generate the golden predicate fixtures from the reference's own tg library.

Run in a container where the reference tree is mounted:

    python tests/golden/gen_golden.py

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


def main():
    oracle.build(with_ref=True)
    assert oracle.ref_available(), "reference tg could not be built"
    polys, holed, pts = build_cases()
    out = {}

    def col_arrays(prefix, values):
        c = wkb.column_from_values(values)
        out[prefix + "_offsets"] = c.offsets.astype(np.int64)
        out[prefix + "_data"] = c.data

    col_arrays("polys", polys)
    col_arrays("holed", holed)
    col_arrays("pts", pts)

    def table(name, build, probe, preds, stride_b=1, stride_p=1):
        """Dense outcome cube [pred, build row, probe row] over the strided
        rows, stored bit-packed; row i of the cube is build row i*stride_b."""
        res = []
        for pred in preds:
            for i in range(0, len(build), stride_b):
                for j in range(0, len(probe), stride_p):
                    r = oracle.ref_predicate(build[i], probe[j], pred)
                    assert r in (0, 1), (pred, i, j, r)
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
