"""Loader for tests/golden/tg_predicates.npz (made by tests/golden/gen_golden.py)."""
import os

import numpy as np

from sedona_gpuspatial.wkb import WkbColumn

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tg_predicates.npz")


def load():
    z = np.load(PATH)
    cols = {}
    for name in ("polys", "holed", "pts", "rel"):
        cols[name] = WkbColumn(z[name + "_offsets"].astype(np.int32), z[name + "_data"])
    return z, cols


def table(z, name):
    """Yields (pred_code, build_rows, probe_rows, expected[nb, np]) per predicate."""
    preds = z[name + "_preds"]
    sb, sp = (int(v) for v in z[name + "_stride"])
    count = int(z[name + "_count"][0])
    res = np.unpackbits(z[name + "_res"], bitorder="little")[:count]
    return preds, sb, sp, res


SHAPES = {
    # table name: (build column, probe column)
    "poly_point": ("polys", "pts"),
    "holed_point": ("holed", "pts"),
    "poly_poly": ("polys", "polys"),
    "point_poly": ("pts", "polys"),
    "point_point": ("pts", "pts"),
    "rel_rel": ("rel", "rel"),
    "poly_poly_all": ("polys", "polys"),
    "rel_point": ("rel", "pts"),
    "point_rel": ("pts", "rel"),
}


def cube(z, cols, name):
    preds, sb, sp, res = table(z, name)
    bname, pname = SHAPES[name]
    nb = len(range(0, len(cols[bname]), sb))
    np_ = len(range(0, len(cols[pname]), sp))
    return preds, np.arange(0, len(cols[bname]), sb), np.arange(0, len(cols[pname]), sp), \
        res.reshape(len(preds), nb, np_)


FIXTURES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                        "reference_fixtures.npz")
FIXTURE_JOINS = ["countries_points", "pip_points", "poly_poly", "countries_countries"]


def load_fixtures():
    """The reference's own test data (tests/golden/gen_fixtures.py): per join,
    (build column, probe column, {predicate: expected sorted (probe, build)
    pairs})."""
    z = np.load(FIXTURES)

    def col(key):
        return WkbColumn(z[f"col_{key}_offsets"].astype(np.int32), z[f"col_{key}_data"])

    joins = {}
    for name in FIXTURE_JOINS:
        exp = {}
        for k in z.files:
            if k.startswith(name + "_") and k.endswith("_build") and k != name + "_build":
                pred = k[len(name) + 1:-len("_build")]
                b, p = z[k], z[f"{name}_{pred}_probe"]
                exp[pred] = sorted(zip(p.tolist(), b.tolist()))
        joins[name] = (col(str(z[name + "_build"])), col(str(z[name + "_probe"])), exp)
    return joins
