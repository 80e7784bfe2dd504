"""Writes the GeoParquet fixtures of the device reader's tests with pyarrow
(Arrow's own Parquet writer, as the reference's files are made) and the
expected WKB values next to them.

    python tests/golden/gen_parquet_fixtures.py

Outputs tests/golden/parquet/*.parquet and tests/golden/parquet_expected.npz.
The files cover what pyarrow writes by default and its options: SNAPPY and
stored pages, data page v1 and v2, dictionary pages with RLE_DICTIONARY data
pages, a dictionary that falls back to PLAIN in the middle of a chunk, a
REQUIRED large_binary column, nulls, several row groups and pages, and other
columns around the geometry.  Two more files are built by hand (checked by
reading them with pyarrow).  In one, a Snappy page holds a copy that reaches
back across a 64 KiB block, which the format allows and Snappy writers do not
emit.  The other has a data page header with 3,000-byte min / max statistics,
longer than the device reader's window for page headers.
The values are synthetic (seeded) WKB points and polygons.
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


# --- a file built by hand: its Snappy page has a copy that reaches back
# across a 64 KiB block, which Snappy writers never emit but the format
# allows (the device reader decodes such pages with one warp per page)

def _varint(v):
    out = bytearray()
    while v >= 0x80:
        out.append((v & 0x7F) | 0x80)
        v >>= 7
    out.append(v)
    return bytes(out)


def _zz(v):
    return _varint((v << 1) ^ (v >> 63))


class _T:
    """Thrift compact protocol writer (the subset Parquet metadata needs)."""

    def __init__(self):
        self.b = bytearray()
        self.last = [0]

    def field(self, fid, t):
        d = fid - self.last[-1]
        self.b += bytes([(d << 4) | t]) if 0 < d <= 15 else bytes([t]) + _zz(fid)
        self.last[-1] = fid

    def i32(self, fid, v):
        self.field(fid, 5)
        self.b += _zz(v)

    def i64(self, fid, v):
        self.field(fid, 6)
        self.b += _zz(v)

    def string(self, fid, s):
        s = s.encode() if isinstance(s, str) else s
        self.field(fid, 8)
        self.b += _varint(len(s)) + s

    def begin(self, fid=None):
        if fid is not None:
            self.field(fid, 12)
        self.last.append(0)

    def end(self):
        self.b.append(0)
        self.last.pop()

    def list(self, fid, etype, n):
        self.field(fid, 9)
        self.b += bytes([(n << 4) | etype]) if n < 15 else bytes([0xF0 | etype]) + _varint(n)


def _snappy_literal(data):
    n = len(data) - 1
    if n < 60:
        return bytes([n << 2]) + data
    nb = (n.bit_length() + 7) // 8
    return bytes([(59 + nb) << 2]) + n.to_bytes(nb, "little") + data


def cross_block_file(path, rng, stats_bytes=0):
    """stats_bytes > 0: no cross-block copy, but a data page header that
    carries min / max statistics of that many bytes each (a header longer
    than the reader's window for page headers)."""
    vals = [rng.integers(0, 256, int(rng.integers(200, 500)), dtype=np.uint8).tobytes()
            for _ in range(300)]
    levels = _varint(len(vals) << 1) + b"\x01"  # one RLE run of definition level 1
    body = bytearray(np.uint32(len(levels)).tobytes() + levels)
    starts = []
    for v in vals:
        body += np.uint32(len(v)).tobytes()
        starts.append(len(body))
        body += v
    if stats_bytes:
        # literals only, split at the block end
        comp = (_varint(len(body)) + _snappy_literal(bytes(body[:65536])) +
                _snappy_literal(bytes(body[65536:])))
    else:
        # a destination inside a value of block 1 copies bytes from a value of block 0
        d = next(s for s in starts if s > 65536 + 8) + 4
        src = starts[3] + 2
        L = 48
        body[d:d + L] = body[src:src + L]
        # the first literal ends exactly at the block end, so only the copy
        # crosses blocks (the block-parallel pass finds it and hands the page
        # to the per-page pass)
        comp = (_varint(len(body)) + _snappy_literal(bytes(body[:65536])) +
                _snappy_literal(bytes(body[65536:d])) +
                bytes([2 | ((L - 1) << 2)]) + (d - src).to_bytes(2, "little") +
                _snappy_literal(bytes(body[d + L:])))
        assert d - src < 65536 and d - src > d - 65536
    # the values as written, re-read from the body
    out, q = [], 4 + len(levels)
    for _ in vals:
        n = int(np.frombuffer(bytes(body[q:q + 4]), np.uint32)[0])
        out.append(bytes(body[q + 4:q + 4 + n]))
        q += 4 + n
    h = _T()
    h.i32(1, 0)
    h.i32(2, len(body))
    h.i32(3, len(comp))
    h.begin(5)
    h.i32(1, len(vals))
    h.i32(2, 0)
    h.i32(3, 3)
    h.i32(4, 3)
    if stats_bytes:
        h.begin(5)  # Statistics: max_value (5), min_value (6)
        h.string(5, rng.integers(0, 256, stats_bytes, dtype=np.uint8).tobytes())
        h.string(6, rng.integers(0, 256, stats_bytes, dtype=np.uint8).tobytes())
        h.end()
    h.end()
    h.b.append(0)
    chunk = bytes(h.b) + comp
    m = _T()
    m.i32(1, 1)
    m.list(2, 12, 2)
    m.begin()
    m.string(4, "schema")
    m.i32(5, 1)
    m.end()
    m.begin()
    m.i32(1, 6)
    m.i32(3, 1)
    m.string(4, "geometry")
    m.end()
    m.i64(3, len(vals))
    m.list(4, 12, 1)
    m.begin()
    m.list(1, 12, 1)
    m.begin()
    m.i64(2, 4)
    m.begin(3)
    m.i32(1, 6)
    m.list(2, 5, 2)
    m.b += _zz(0) + _zz(3)
    m.list(3, 8, 1)
    m.b += _varint(8) + b"geometry"
    m.i32(4, 1)
    m.i64(5, len(vals))
    m.i64(6, len(h.b) + len(body))
    m.i64(7, len(chunk))
    m.i64(9, 4)
    m.end()
    m.end()
    m.i64(2, len(h.b) + len(body))
    m.i64(3, len(vals))
    m.end()
    m.list(5, 12, 1)
    m.begin()
    m.string(1, "geo")
    m.string(2, geo_meta("geometry"))
    m.end()
    m.b.append(0)
    with open(path, "wb") as f:
        f.write(b"PAR1" + chunk + bytes(m.b) + np.uint32(len(m.b)).tobytes() + b"PAR1")
    return out


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

    vals = cross_block_file(os.path.join(outdir, "cross_block_snappy_v1.parquet"), rng)
    got = pq.read_table(os.path.join(outdir, "cross_block_snappy_v1.parquet")).column(
        "geometry").to_pylist()
    assert got == vals, "pyarrow reads the hand-built file differently"
    keep("cross_block_snappy_v1", vals)

    vals = cross_block_file(os.path.join(outdir, "big_header_snappy_v1.parquet"), rng,
                            stats_bytes=3000)
    got = pq.read_table(os.path.join(outdir, "big_header_snappy_v1.parquet")).column(
        "geometry").to_pylist()
    assert got == vals, "pyarrow reads the hand-built file differently"
    keep("big_header_snappy_v1", vals)

    np.savez_compressed(os.path.join(HERE, "parquet_expected.npz"), **expected)
    for f in sorted(os.listdir(outdir)):
        md = pq.ParquetFile(os.path.join(outdir, f)).metadata
        encs = sorted({e for g in range(md.num_row_groups)
                       for c in range(md.num_columns)
                       for e in md.row_group(g).column(c).encodings})
        print(f, os.path.getsize(os.path.join(outdir, f)), md.num_row_groups, encs)


if __name__ == "__main__":
    main()
