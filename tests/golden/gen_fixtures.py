"""Golden outcomes on the reference's own test data.

The reference's GPU library tests read six parquet files
(c/sedona-libgpuspatial/libgpuspatial/test/data/{synthetic_pip,synthetic_poly,
countries}).  This script reads them with pyarrow where the reference tree is
mounted, keeps seeded subsets of the synthetic ones (the countries and their
generated points in full), and stores, per join and predicate, the pair set
the reference CPU join's refiner returns: every (build, probe) pair whose f32
boxes intersect, refined by the reference's own tg (compiled from the
reference tree into oracle/_ref) as tg_geom_<pred>(build, probe) under the
refiner's default y-stripes ring index
(rust/sedona-spatial-join/src/refine/tg.rs:322-357,
rust/sedona-common/src/option.rs:213).

    SPJ_REFERENCE_TREE=/path/to/sedona-db python tests/golden/gen_fixtures.py

writes tests/golden/reference_fixtures.npz (WKB columns + expected pairs).
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

DATA = "c/sedona-libgpuspatial/libgpuspatial/test/data"
PREDS = ["intersects", "contains", "covers", "within", "coveredby", "touches", "equals"]
# join name: (build file, probe file, build rows kept, probe rows kept, predicates)
JOINS = {
    "countries_points": ("countries/natural-earth_countries_geo.parquet",
                         "countries/generated_points.parquet", None, None,
                         ["intersects", "contains", "covers", "touches"]),
    "pip_points": ("synthetic_pip/polygons.parquet", "synthetic_pip/points.parquet", 1500, None,
                   ["intersects", "contains", "covers", "touches"]),
    "poly_poly": ("synthetic_poly/polygons1.parquet", "synthetic_poly/polygons2.parquet", 1500,
                  1500, PREDS),
    "countries_countries": ("countries/natural-earth_countries_geo.parquet",
                            "countries/natural-earth_countries_geo.parquet", None, None, PREDS),
}


def read_geometry(path, keep, seed):
    import pyarrow.parquet as pq
    vals = pq.read_table(path).column("geometry").combine_chunks().to_pylist()
    if keep is not None and keep < len(vals):
        rows = np.sort(np.random.default_rng(seed).choice(len(vals), keep, replace=False))
        vals = [vals[i] for i in rows]
    return vals


def main():
    tree = os.environ.get("SPJ_REFERENCE_TREE", "")
    assert tree, "set SPJ_REFERENCE_TREE to the reference source tree"
    oracle.build(with_ref=True)
    assert oracle.ref_available(), "the reference's tg could not be built"
    out = {}
    cols = {}
    for name, (bf, pf, bk, pk, preds) in JOINS.items():
        for side, f, keep, seed in (("build", bf, bk, 11), ("probe", pf, pk, 12)):
            # each distinct column is stored once, under a short name
            key = os.path.basename(f).split(".")[0] + ("" if keep is None else f"_{keep}_{seed}")
            if key not in cols:
                cols[key] = read_geometry(os.path.join(tree, DATA, f), keep, seed)
                c = wkb.column_from_values(cols[key])
                out[f"col_{key}_offsets"] = c.offsets.astype(np.int64)
                out[f"col_{key}_data"] = c.data
            out[f"{name}_{side}"] = np.array(key)
        build, probe = cols[str(out[f"{name}_build"])], cols[str(out[f"{name}_probe"])]
        B = oracle.Geoms(wkb.column_from_values(build))
        P = oracle.Geoms(wkb.column_from_values(probe))
        # candidates: f32 box filter (outward boxes, points to nearest)
        cb, cp = oracle.rect_join(B.boxes(1), P.boxes(1), nthreads=os.cpu_count() or 1)
        for pred in preds:
            keep_b, keep_p = [], []
            for b, p in zip(cb.tolist(), cp.tolist()):
                r = oracle.ref_predicate(build[b], probe[p], pred, 2)
                assert r in (0, 1), (name, pred, b, p, r)
                if r:
                    keep_b.append(b)
                    keep_p.append(p)
            out[f"{name}_{pred}_build"] = np.array(keep_b, dtype=np.uint32)
            out[f"{name}_{pred}_probe"] = np.array(keep_p, dtype=np.uint32)
            print(name, pred, len(cb), "candidates", len(keep_b), "pairs")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_fixtures.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
