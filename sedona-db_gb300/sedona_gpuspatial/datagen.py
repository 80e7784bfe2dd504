"""Seeded synthetic inputs for the five spatial-join workloads.

The public data the reference measures on (SpatialBench SF1) is not available,
so these generators stand in for it with the shapes, sizes and value
distributions of each workload.  Every generator takes its seed
(default 20260101 + workload number) and optional size overrides so tests can
run the same distributions at small sizes.

Workloads:
  1  1M uniform points  x  10k star polygons, ST_Intersects(poly, pt)
  2  2M building polygons (GMM-clustered)  x  50k star zones, ST_Intersects
  3  10M GMM points in uneven record batches  x  the workload-2 zones, ST_Contains
  4  20M probe points  x  1M build points (GMM), KNN k=8 and ST_DWithin(d=25)
  5  100M GMM build points  x  10M range boxes + 10M exact-point lookups
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .wkb import WkbColumn, points_column, polygons_column

BASE_SEED = 20260101


@dataclass
class JoinInputs:
    name: str
    build: WkbColumn
    probe: WkbColumn
    predicate: str
    params: dict = field(default_factory=dict)
    batches: Optional[List[int]] = None  # probe record-batch row counts


def _rng(workload: int, seed: Optional[int]) -> np.random.Generator:
    return np.random.default_rng(BASE_SEED + workload if seed is None else seed)


def star_polygons(rng, n, nv_lo, nv_hi, cx, cy, r_lo, r_hi):
    """Star-shaped simple polygons: n_i ~ U{nv_lo..nv_hi} vertices at sorted
    uniform angles, radii R*U(0.6, 1.0), R ~ U(r_lo, r_hi); rings are closed."""
    nv = rng.integers(nv_lo, nv_hi + 1, size=n)
    R = rng.uniform(r_lo, r_hi, size=n)
    tot = int(nv.sum())
    poly_of = np.repeat(np.arange(n), nv)
    ang = rng.uniform(0.0, 2 * np.pi, size=tot)
    # sort angles within each polygon
    order = np.lexsort((ang, poly_of))
    ang = ang[order]
    rad = R[poly_of] * rng.uniform(0.6, 1.0, size=tot)
    x = cx[poly_of] + rad * np.cos(ang)
    y = cy[poly_of] + rad * np.sin(ang)
    return _close_rings(nv, x, y)


def regular_polygons(rng, n, nv_lo, nv_hi, cx, cy, side_lo, side_hi):
    """Regular n-gons (n ~ U{nv_lo..nv_hi}) with side ~ U(side_lo, side_hi)
    and rotation ~ U[0, 2pi); rings are closed."""
    nv = rng.integers(nv_lo, nv_hi + 1, size=n)
    side = rng.uniform(side_lo, side_hi, size=n)
    rot = rng.uniform(0.0, 2 * np.pi, size=n)
    circ = side / (2.0 * np.sin(np.pi / nv))
    poly_of = np.repeat(np.arange(n), nv)
    start = np.zeros(n, dtype=np.int64)
    np.cumsum(nv[:-1], out=start[1:])
    k = np.arange(int(nv.sum())) - start[poly_of]
    ang = rot[poly_of] + 2 * np.pi * k / nv[poly_of]
    x = cx[poly_of] + circ[poly_of] * np.cos(ang)
    y = cy[poly_of] + circ[poly_of] * np.sin(ang)
    return _close_rings(nv, x, y)


def _close_rings(nv, x, y):
    """Append each ring's first vertex at its end; returns (npts, xy)."""
    n = len(nv)
    start = np.zeros(n, dtype=np.int64)
    np.cumsum(nv[:-1], out=start[1:])
    npts = nv + 1
    tot = int(npts.sum())
    out = np.empty((tot, 2), dtype=np.float64)
    dst_start = start + np.arange(n)
    poly_of = np.repeat(np.arange(n), nv)
    k = np.arange(len(x)) - start[poly_of]
    dst = dst_start[poly_of] + k
    out[dst, 0] = x
    out[dst, 1] = y
    close = dst_start + nv
    out[close, 0] = x[start]
    out[close, 1] = y[start]
    return npts, out


def gmm_points(rng, n, ncomp, lo, hi, sig_lo, sig_hi):
    """n points from an equal-weight Gaussian mixture; means U[lo,hi]^2,
    sigma ~ U(sig_lo, sig_hi); clipped to the square."""
    mx = rng.uniform(lo, hi, size=ncomp)
    my = rng.uniform(lo, hi, size=ncomp)
    sg = rng.uniform(sig_lo, sig_hi, size=ncomp)
    c = rng.integers(0, ncomp, size=n)
    x = np.clip(mx[c] + sg[c] * rng.standard_normal(n), lo, hi)
    y = np.clip(my[c] + sg[c] * rng.standard_normal(n), lo, hi)
    return x, y, (mx, my, sg)


def batch_sizes(rng, total, lo=1024, hi=131072):
    """Record-batch row counts floor(exp(U(ln lo, ln hi))); remainder last."""
    sizes = []
    left = total
    while left > 0:
        s = int(np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        s = min(s, left)
        sizes.append(s)
        left -= s
    return sizes


def workload1(n_points=1_000_000, n_polys=10_000, seed=None) -> JoinInputs:
    rng = _rng(1, seed)
    cx = rng.uniform(0, 1000, size=n_polys)
    cy = rng.uniform(0, 1000, size=n_polys)
    npts, xy = star_polygons(rng, n_polys, 8, 64, cx, cy, 0.5, 5.0)
    px = rng.uniform(0, 1000, size=n_points)
    py = rng.uniform(0, 1000, size=n_points)
    return JoinInputs("pip_uniform_1m_x_10k", polygons_column(npts, xy),
                      points_column(px, py), "intersects")


def zones(rng, n_zones):
    cx = rng.uniform(0, 1e5, size=n_zones)
    cy = rng.uniform(0, 1e5, size=n_zones)
    return star_polygons(rng, n_zones, 32, 256, cx, cy, 500.0, 3000.0)


def workload2(n_buildings=2_000_000, n_zones=50_000, seed=None) -> JoinInputs:
    rng = _rng(2, seed)
    znpts, zxy = zones(rng, n_zones)
    bx, by, _ = gmm_points(rng, n_buildings, 64, 0.0, 1e5, 200.0, 2000.0)
    bnpts, bxy = regular_polygons(rng, n_buildings, 4, 12, bx, by, 5.0, 50.0)
    return JoinInputs("polygon_intersects_2m_x_50k", polygons_column(znpts, zxy),
                      polygons_column(bnpts, bxy), "intersects")


def workload3(n_points=10_000_000, n_zones=50_000, seed=None) -> JoinInputs:
    # same zones as workload 2 (same seed stream position)
    rng2 = _rng(2, None if seed is None else seed - 1)
    znpts, zxy = zones(rng2, n_zones)
    rng = _rng(3, seed)
    px, py, _ = gmm_points(rng, n_points, 64, 0.0, 1e5, 200.0, 2000.0)
    sizes = batch_sizes(rng, n_points)
    return JoinInputs("contains_stream_10m_x_50k", polygons_column(znpts, zxy),
                      points_column(px, py), "contains", batches=sizes)


def workload4(n_probe=20_000_000, n_build=1_000_000, seed=None, k=8, distance=25.0) -> JoinInputs:
    rng = _rng(4, seed)
    mx = rng.uniform(0, 1e5, size=128)
    my = rng.uniform(0, 1e5, size=128)
    sg = rng.uniform(50.0, 500.0, size=128)

    def draw(n):
        c = rng.integers(0, 128, size=n)
        x = np.clip(mx[c] + sg[c] * rng.standard_normal(n), 0, 1e5)
        y = np.clip(my[c] + sg[c] * rng.standard_normal(n), 0, 1e5)
        return x, y

    bx, by = draw(n_build)
    px, py = draw(n_probe)
    return JoinInputs("knn8_dwithin25_20m_x_1m", points_column(bx, by),
                      points_column(px, py), "knn",
                      params={"k": k, "distance": distance, "build_xy": (bx, by),
                              "probe_xy": (px, py)})


def workload5(n_build=100_000_000, n_boxes=10_000_000, n_lookups=10_000_000, seed=None):
    """Returns (build points column, box-probe column, lookup-probe column, build xy)."""
    rng = _rng(5, seed)
    bx, by, (mx, my, sg) = gmm_points(rng, n_build, 256, 0.0, 1e5, 50.0, 500.0)
    c = rng.integers(0, 256, size=n_boxes)
    cx = np.clip(mx[c] + sg[c] * rng.standard_normal(n_boxes), 0, 1e5)
    cy = np.clip(my[c] + sg[c] * rng.standard_normal(n_boxes), 0, 1e5)
    side = np.exp(rng.uniform(np.log(0.01), np.log(10.0), size=n_boxes))
    h = side / 2
    ring = np.stack([
        np.stack([cx - h, cy - h], 1), np.stack([cx + h, cy - h], 1),
        np.stack([cx + h, cy + h], 1), np.stack([cx - h, cy + h], 1),
        np.stack([cx - h, cy - h], 1)], 1).reshape(-1, 2)
    boxes = polygons_column(np.full(n_boxes, 5), ring)
    pick = rng.integers(0, n_build, size=n_lookups)
    lookups = points_column(bx[pick], by[pick])
    return points_column(bx, by), boxes, lookups, (bx, by)
