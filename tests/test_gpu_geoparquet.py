"""GeoParquet read onto the device (SpjParquetReadWkb) against the values
pyarrow wrote into the committed fixtures, against the writer's input on
round trips, and through a join against the same columns given directly.
Byte data: results must match exactly."""
import os

import numpy as np
import pytest

import gpu_util

pytestmark = pytest.mark.gpu

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


def _assert_column(got, off, data, valid):
    """got: a host WkbColumn with int64 offsets; nulls are empty values."""
    n = len(valid)
    assert len(got) == n
    lens = np.diff(off)
    exp_off = np.zeros(n + 1, np.int64)
    exp_off[1:] = np.cumsum(np.where(valid, lens, 0))
    assert np.array_equal(got.offsets, exp_off)
    assert np.array_equal(got.data, data)
    if valid.all():
        assert got.validity is None
    else:
        bits = np.unpackbits(got.validity, bitorder="little")[:n].astype(bool)
        assert np.array_equal(bits, valid)


@pytest.mark.parametrize("name", FIXTURES)
def test_fixture_read_matches_pyarrow_values(gp, name):
    off, data, valid = _expected(name)
    with gp.GeoParquetFile(os.path.join(FIXDIR, name + ".parquet")) as f:
        for _ in range(2):  # a second read reuses the handle's buffers
            d = f.read_wkb()
            _assert_column(gp.device_to_host(d), off, data, valid)
        st = f.stats()
        assert st["value_bytes"] == len(data) and st["ms_device"] > 0


@pytest.mark.parametrize("name", ["dict_snappy_v1", "plain_snappy_v2"])
def test_row_group_ranges(gp, name):
    off, data, valid = _expected(name)
    with gp.GeoParquetFile(os.path.join(FIXDIR, name + ".parquet")) as f:
        nrg = f.info()["num_row_groups"]
        r0 = 0
        for g in range(nrg):
            rows = f.row_group_rows(g)
            d = f.read_wkb(rg_begin=g, rg_end=g + 1)
            sub_off = off[r0:r0 + rows + 1]
            _assert_column(gp.device_to_host(d), sub_off - sub_off[0],
                           data[sub_off[0]:sub_off[-1]], valid[r0:r0 + rows])
            r0 += rows
        d = f.read_wkb(rg_begin=1, rg_end=1)
        assert d.length == 0


@pytest.mark.parametrize("compression", ["snappy", "none"])
@pytest.mark.parametrize("page_version", [1, 2])
def test_writer_round_trip(gp, tmp_path, compression, page_version):
    from sedona_gpuspatial import datagen, wkb
    inp = datagen.workload1(n_points=200000, n_polys=3000)
    rng = np.random.default_rng(page_version)
    for col, nulls in ((inp.probe, True), (inp.build, False)):
        validity = np.packbits(rng.random(len(col)) > 0.1, bitorder="little") if nulls else None
        c = wkb.WkbColumn(col.offsets, col.data, validity)
        path = str(tmp_path / "rt.parquet")
        gp.write_wkb(path, c, compression=compression, page_version=page_version,
                     row_group_rows=70000, page_bytes=1 << 18)
        with gp.GeoParquetFile(path) as f:
            got = gp.device_to_host(f.read_wkb())
        valid = (np.unpackbits(validity, bitorder="little")[:len(c)].astype(bool)
                 if nulls else np.ones(len(c), bool))
        off = col.offsets.astype(np.int64)
        keep = np.repeat(valid, np.diff(off))
        _assert_column(got, off, col.data[keep], valid)


def test_join_from_geoparquet(gp, tmp_path):
    """Build and probe sides read from GeoParquet give the pairs of the same
    columns passed directly."""
    from sedona_gpuspatial import capi, datagen
    inp = datagen.workload1(n_points=100000, n_polys=1000)
    pb, pp = str(tmp_path / "b.parquet"), str(tmp_path / "p.parquet")
    gp.write_wkb(pb, inp.build, compression="snappy")
    gp.write_wkb(pp, inp.probe, compression="snappy", page_version=2)
    j0 = capi.SpatialJoin()
    j0.build(inp.build)
    exp = gpu_util.pairs(*j0.probe(inp.probe, "intersects"))
    fb, fp = gp.GeoParquetFile(pb), gp.GeoParquetFile(pp)
    j = capi.SpatialJoin()
    import ctypes as C
    rc = capi.lib().SpjJoinBuildDevice(j.h, C.byref(fb.read_wkb()))
    assert rc == 0, capi.lib().SpjJoinLastError(j.h)
    db, dp, n = j.probe_device(fp.read_wkb(), "intersects")
    assert gpu_util.pairs(*gpu_util.device_pairs(db, dp, n)) == exp
    fb.close()
    fp.close()


def test_corrupt_page_is_an_error(gp, tmp_path):
    """A PLAIN length word that runs past its page fails the read with a
    message; the handle then reads a good file's column again."""
    from sedona_gpuspatial import datagen
    from sedona_gpuspatial.capi import GpuSpatialError
    inp = datagen.workload1(n_points=5000, n_polys=50)
    path = str(tmp_path / "c.parquet")
    gp.write_wkb(path, inp.build, compression="none")
    blob = bytearray(open(path, "rb").read())
    first = inp.build.value(0)
    at = bytes(blob).find(first)
    assert at > 4 and blob[at - 4:at] == np.uint32(len(first)).tobytes()
    blob[at - 4:at] = np.uint32(0x7FFFFFF0).tobytes()
    bad = str(tmp_path / "bad.parquet")
    open(bad, "wb").write(bytes(blob))
    with gp.GeoParquetFile(bad) as f:
        with pytest.raises(GpuSpatialError, match="PLAIN"):
            f.read_wkb()
    with gp.GeoParquetFile(path) as f:
        got = gp.device_to_host(f.read_wkb())
    assert np.array_equal(got.data, inp.build.data)


@pytest.mark.parametrize("page_version", [1, 2])
def test_device_matches_oracle(gp, oracle_lib, tmp_path, page_version):
    """The device reader against the CPU oracle's reading of the same file."""
    from sedona_gpuspatial import datagen, wkb
    inp = datagen.workload2(n_buildings=100000, n_zones=2000)
    col = inp.probe
    rng = np.random.default_rng(11)
    validity = np.packbits(rng.random(len(col)) > 0.05, bitorder="little")
    c = wkb.WkbColumn(col.offsets, col.data, validity)
    path = str(tmp_path / "o.parquet")
    gp.write_wkb(path, c, compression="snappy", page_version=page_version,
                 row_group_rows=40000, page_bytes=1 << 17)
    off, data, valid = oracle_lib.parquet_read(path)
    with gp.GeoParquetFile(path) as f:
        got = gp.device_to_host(f.read_wkb())
    _assert_column(got, off, data, valid)
