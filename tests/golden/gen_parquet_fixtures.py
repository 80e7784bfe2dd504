"""Writes the GeoParquet fixtures of the device reader's tests with pyarrow
(Arrow's own Parquet writer, as the reference's files are made) and the
expected WKB values next to them.

    python tests/golden/gen_parquet_fixtures.py

Outputs tests/golden/parquet/*.parquet and tests/golden/parquet_expected.npz.
The files cover what pyarrow writes by default and its options: SNAPPY and
stored pages, data page v1 and v2, dictionary pages with RLE_DICTIONARY data
pages, a dictionary that falls back to PLAIN in the middle of a chunk, a
REQUIRED large_binary column, nulls, several row groups and pages, and other
columns around the geometry.  The values are synthetic (seeded) WKB points
and polygons.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "sedona-db_gb300"))

import pyarrow as pa  # noqa: E402
import pyarrow.parquet as pq  # noqa: E402

from sedona_gpuspatial import wkb  # noqa: E402


def polygon_wkb(rng, n):
    out = []
    for _ in range(n):
        k = int(rng.integers(3, 12))
        cx, cy = rng.uniform(-170, 170), rng.uniform(-80, 80)
        ang = np.sort(rng.uniform(0, 2 * np.pi, k))
        r = rng.uniform(0.1, 2.0, k)
        xs, ys = cx + r * np.cos(ang), cy + r * np.sin(ang)
        ring = np.stack([np.append(xs, xs[0]), np.append(ys, ys[0])], 1)
        out.append(b"\x01" + np.uint32(3).tobytes() + np.uint32(1).tobytes() +
                   np.uint32(len(ring)).tobytes() + ring.astype("<f8").tobytes())
    return out


def point_wkb(rng, n):
    x, y = rng.uniform(-180, 180, n), rng.uniform(-90, 90, n)
    col = wkb.points_column(x, y)
    return [col.value(i) for i in range(n)]


def geo_meta(column):
    return json.dumps({"version": "1.1.0", "primary_column": column,
                       "columns": {column: {"encoding": "WKB", "geometry_types": []}}})


def write(path, table, column, **kw):
    md = dict(table.schema.metadata or {})
    md[b"geo"] = geo_meta(column).encode()
    pq.write_table(table.replace_schema_metadata(md), path, **kw)


def main():
    rng = np.random.default_rng(20260301)
    outdir = os.path.join(HERE, "parquet")
    os.makedirs(outdir, exist_ok=True)
    expected = {}

    def keep(name, values):
        off = np.zeros(len(values) + 1, np.int64)
        off[1:] = np.cumsum([len(v) if v is not None else 0 for v in values])
        expected[f"off_{name}"] = off
        expected[f"data_{name}"] = np.frombuffer(b"".join(v for v in values if v is not None),
                                                 np.uint8)
        expected[f"valid_{name}"] = np.array([v is not None for v in values])

    distinct = polygon_wkb(rng, 40) + point_wkb(rng, 10)
    pick = rng.integers(0, len(distinct), 3000)
    vals = [distinct[i] if rng.random() > 0.1 else None for i in pick]
    t = pa.table({"geometry": pa.array(vals, pa.binary())})
    write(os.path.join(outdir, "dict_snappy_v1.parquet"), t, "geometry", compression="snappy",
          use_dictionary=True, row_group_size=1000, data_page_size=2048,
          data_page_version="1.0")
    keep("dict_snappy_v1", vals)
    write(os.path.join(outdir, "dict_none_v2.parquet"), t, "geometry", compression="none",
          use_dictionary=True, row_group_size=1300, data_page_size=1024,
          data_page_version="2.0")
    keep("dict_none_v2", vals)

    mixed = point_wkb(rng, 1200) + polygon_wkb(rng, 800)
    order = rng.permutation(len(mixed))
    vals = [mixed[i] if rng.random() > 0.05 else None for i in order]
    t = pa.table({"id": pa.array(np.arange(len(vals), dtype=np.int64)),
                  "name": pa.array([f"row{i}" for i in range(len(vals))]),
                  "geom": pa.array(vals, pa.binary())})
    write(os.path.join(outdir, "plain_snappy_v2.parquet"), t, "geom", compression="snappy",
          use_dictionary=False, row_group_size=700, data_page_size=4096,
          data_page_version="2.0")
    keep("plain_snappy_v2", vals)
    # the dictionary outgrows its limit early in each chunk: later pages PLAIN
    write(os.path.join(outdir, "dict_fallback_v1.parquet"), t, "geom", compression="snappy",
          use_dictionary=True, dictionary_pagesize_limit=3000, row_group_size=1000,
          data_page_size=2048, data_page_version="1.0")
    keep("dict_fallback_v1", vals)

    pts = point_wkb(rng, 3000)
    schema = pa.schema([pa.field("geometry", pa.large_binary(), nullable=False)])
    t = pa.table({"geometry": pa.array(pts, pa.large_binary())}, schema=schema)
    write(os.path.join(outdir, "required_none_v1.parquet"), t, "geometry", compression="none",
          use_dictionary=False, row_group_size=2000, data_page_size=8192,
          data_page_version="1.0")
    keep("required_none_v1", pts)

    np.savez_compressed(os.path.join(HERE, "parquet_expected.npz"), **expected)
    for f in sorted(os.listdir(outdir)):
        md = pq.ParquetFile(os.path.join(outdir, f)).metadata
        encs = sorted({e for g in range(md.num_row_groups)
                       for c in range(md.num_columns)
                       for e in md.row_group(g).column(c).encodings})
        print(f, os.path.getsize(os.path.join(outdir, f)), md.num_row_groups, encs)


if __name__ == "__main__":
    main()
