"""GeoParquet host side without a GPU: the footer / schema / "geo" metadata
parser and the writer of the device reader's path, against pyarrow (Arrow's
own Parquet implementation) where it is installed, and the committed
fixtures against their expected values."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXDIR = os.path.join(HERE, "golden", "parquet")
FIXTURES = sorted(f[:-8] for f in os.listdir(FIXDIR) if f.endswith(".parquet"))


@pytest.fixture(scope="module")
def gp():
    from sedona_gpuspatial import _build
    _build.build()
    from sedona_gpuspatial import geoparquet
    return geoparquet


def _expected(name):
    z = np.load(os.path.join(HERE, "golden", "parquet_expected.npz"))
    return z[f"off_{name}"], z[f"data_{name}"], z[f"valid_{name}"]


@pytest.mark.parametrize("name", FIXTURES)
def test_fixture_values_match_pyarrow(name):
    pq = pytest.importorskip("pyarrow.parquet")
    off, data, valid = _expected(name)
    f = pq.ParquetFile(os.path.join(FIXDIR, name + ".parquet"))
    geo = json.loads(f.metadata.metadata[b"geo"])
    vals = f.read().column(geo["primary_column"]).to_pylist()
    assert len(vals) == len(valid)
    for i, v in enumerate(vals):
        assert (v is not None) == bool(valid[i])
        if v is not None:
            assert v == data[off[i]:off[i + 1]].tobytes()


@pytest.mark.parametrize("name", FIXTURES)
def test_footer_parse_matches_pyarrow(gp, name):
    pq = pytest.importorskip("pyarrow.parquet")
    path = os.path.join(FIXDIR, name + ".parquet")
    md = pq.ParquetFile(path).metadata
    with gp.GeoParquetFile(path) as f:
        info = f.info()
        assert info == {"num_rows": md.num_rows, "num_row_groups": md.num_row_groups,
                        "num_columns": md.num_columns}
        assert f.column_names() == [md.schema.column(i).path for i in range(md.num_columns)]
        assert f.primary_column() == json.loads(md.metadata[b"geo"])["primary_column"]
        for g in range(md.num_row_groups):
            assert f.row_group_rows(g) == md.row_group(g).num_rows


def _column(n, seed, nulls):
    from sedona_gpuspatial import wkb
    rng = np.random.default_rng(seed)
    vals = []
    for i in range(n):
        k = int(rng.integers(0, 4))
        if k == 0:
            vals.append(b"")  # an empty value (not a null)
        else:
            vals.append(rng.integers(0, 256, int(rng.integers(1, 300)), dtype=np.uint8).tobytes())
    off = np.zeros(n + 1, np.int32)
    off[1:] = np.cumsum([len(v) for v in vals])
    data = np.frombuffer(b"".join(vals), np.uint8) if off[-1] else np.zeros(0, np.uint8)
    validity = None
    if nulls:
        validity = np.packbits(rng.random(n) > 0.2, bitorder="little")
    return wkb.WkbColumn(off, data, validity), vals


@pytest.mark.parametrize("compression", ["snappy", "none"])
@pytest.mark.parametrize("page_version", [1, 2])
@pytest.mark.parametrize("nulls", [False, True])
def test_writer_output_reads_in_pyarrow(gp, tmp_path, compression, page_version, nulls):
    pq = pytest.importorskip("pyarrow.parquet")
    col, vals = _column(1500, page_version * 10 + nulls, nulls)
    path = str(tmp_path / "w.parquet")
    gp.write_wkb(path, col, column="geom", compression=compression, page_version=page_version,
                 row_group_rows=600, page_bytes=5000)
    f = pq.ParquetFile(path)
    assert f.metadata.num_row_groups == 3
    geo = json.loads(f.metadata.metadata[b"geo"])
    assert geo["primary_column"] == "geom" and geo["columns"]["geom"]["encoding"] == "WKB"
    got = f.read().column("geom").to_pylist()
    for i, v in enumerate(got):
        if col.is_valid(i):
            assert v == vals[i]
        else:
            assert v is None
    with gp.GeoParquetFile(path) as g:
        assert g.info()["num_rows"] == 1500 and g.primary_column() == "geom"


def test_snappy_compresses_repetitive_pages(gp, tmp_path):
    """Snappy elements beyond literals: repeated WKB values shrink."""
    from sedona_gpuspatial import wkb
    col = wkb.points_column(np.tile(np.arange(50.0), 200), np.zeros(10000))
    a, b = str(tmp_path / "s.parquet"), str(tmp_path / "n.parquet")
    gp.write_wkb(a, col, compression="snappy")
    gp.write_wkb(b, col, compression="none")
    assert os.path.getsize(a) < os.path.getsize(b) / 4
    pq = pytest.importorskip("pyarrow.parquet")
    got = pq.read_table(a).column("geometry").to_pylist()
    assert all(v == col.value(i) for i, v in enumerate(got))


def test_empty_file(gp, tmp_path):
    from sedona_gpuspatial import wkb
    path = str(tmp_path / "e.parquet")
    gp.write_wkb(path, wkb.WkbColumn(np.zeros(1, np.int32), np.zeros(0, np.uint8)))
    with gp.GeoParquetFile(path) as f:
        assert f.info() == {"num_rows": 0, "num_row_groups": 0, "num_columns": 1}
    pq = pytest.importorskip("pyarrow.parquet")
    assert pq.read_table(path).num_rows == 0


def test_malformed_files_raise(gp, tmp_path):
    from sedona_gpuspatial.capi import GpuSpatialError
    src = open(os.path.join(FIXDIR, "dict_snappy_v1.parquet"), "rb").read()
    cases = {
        "short": b"PAR1",
        "magic": src[:-4] + b"XXXX",
        "footer_len": src[:-8] + np.uint32(len(src) * 2).tobytes() + b"PAR1",
        "truncated_footer": src[:-40] + src[-8:],
    }
    for name, blob in cases.items():
        p = tmp_path / f"{name}.parquet"
        p.write_bytes(blob)
        with pytest.raises(GpuSpatialError):
            gp.GeoParquetFile(str(p))
    with pytest.raises(GpuSpatialError, match="cannot open"):
        gp.GeoParquetFile(str(tmp_path / "missing.parquet"))


def test_reference_parquet_metadata(gp):
    """The reference's own GeoParquet test files (when its tree is at hand)."""
    ref = os.environ.get("SPJ_REFERENCE_TREE", "")
    pq = pytest.importorskip("pyarrow.parquet")
    files = []
    for root in ("c/sedona-libgpuspatial/libgpuspatial/test/data", "r/sedonadb/inst/files"):
        d = os.path.join(ref, root)
        if ref and os.path.isdir(d):
            for dp, _, fs in os.walk(d):
                files += [os.path.join(dp, f) for f in fs if f.endswith(".parquet")]
    if not files:
        pytest.skip("reference tree not available")
    for path in files:
        md = pq.ParquetFile(path).metadata
        with gp.GeoParquetFile(path) as f:
            assert f.info()["num_rows"] == md.num_rows
            assert f.column_names() == [md.schema.column(i).path for i in range(md.num_columns)]
            geo = md.metadata.get(b"geo") if md.metadata else None
            if geo:
                assert f.primary_column() == json.loads(geo)["primary_column"]


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_reader_matches_fixtures(oracle_lib, name):
    off, data, valid = _expected(name)
    o_off, o_data, o_valid = oracle_lib.parquet_read(os.path.join(FIXDIR, name + ".parquet"))
    exp_off = np.zeros(len(valid) + 1, np.int64)
    exp_off[1:] = np.cumsum(np.where(valid, np.diff(off), 0))
    assert np.array_equal(o_valid, valid)
    assert np.array_equal(o_off, exp_off)
    assert np.array_equal(o_data, data)


@pytest.mark.parametrize("compression", ["snappy", "none"])
@pytest.mark.parametrize("page_version", [1, 2])
def test_oracle_reader_reads_writer_output(gp, oracle_lib, tmp_path, compression,
                                           page_version):
    col, vals = _column(3000, 7 + page_version, True)
    path = str(tmp_path / "w.parquet")
    gp.write_wkb(path, col, compression=compression, page_version=page_version,
                 row_group_rows=1000, page_bytes=8000)
    off, data, valid = oracle_lib.parquet_read(path)
    for i in range(len(vals)):
        assert bool(valid[i]) == col.is_valid(i)
        if valid[i]:
            assert data[off[i]:off[i + 1]].tobytes() == vals[i]
        else:
            assert off[i] == off[i + 1]


def test_oracle_reader_on_reference_files(oracle_lib):
    """The oracle against pyarrow on the reference's own GeoParquet files."""
    ref = os.environ.get("SPJ_REFERENCE_TREE", "")
    pq = pytest.importorskip("pyarrow.parquet")
    d = os.path.join(ref, "c/sedona-libgpuspatial/libgpuspatial/test/data")
    if not ref or not os.path.isdir(d):
        pytest.skip("reference tree not available")
    n = 0
    for dp, _, fs in os.walk(d):
        for f in fs:
            if not f.endswith(".parquet"):
                continue
            path = os.path.join(dp, f)
            t = pq.read_table(path)
            off, data, valid = oracle_lib.parquet_read(path, "geometry")
            vals = t.column("geometry").to_pylist()
            assert len(vals) == len(valid)
            for i, v in enumerate(vals):
                assert (v is not None) == bool(valid[i])
                if v is not None:
                    assert data[off[i]:off[i + 1]].tobytes() == v
            n += 1
    assert n >= 6


def test_oracle_reader_errors(oracle_lib, tmp_path):
    src = open(os.path.join(FIXDIR, "plain_snappy_v2.parquet"), "rb").read()
    p = tmp_path / "bad.parquet"
    p.write_bytes(src[:-4] + b"XXXX")
    with pytest.raises(ValueError):
        oracle_lib.parquet_read(str(p))
    with pytest.raises(ValueError, match="no such column"):
        oracle_lib.parquet_read(os.path.join(FIXDIR, "plain_snappy_v2.parquet"), "nope")
