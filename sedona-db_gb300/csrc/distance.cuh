// distance.cuh — the Euclidean distance of the reference's ST_DWithin
// refine, build.distance_ext(probe) <= d (rust/sedona-spatial-join/src/refine/
// geo.rs:312-321), as the reference's sedona-geo-generic-alg computes it
// (rust/sedona-geo-generic-alg/src/algorithm/line_measures/metric_spaces/
// euclidean/utils.rs, distance.rs), for point, polygon and multipolygon rows.
// Every step is the reference's FP64 operation (the library is built without
// multiply-add contraction); hypot is CUDA's, within an ulp or two of the host
// libm's.  The reference's intersects tests are geo's (exact predicates); tg's
// stand in for them, and the two differ only where a distance is within FP64
// rounding of zero.
#pragma once
#include <cfloat>

#include "relate.cuh"

namespace spj {
namespace pred {
namespace {

// utils.rs:127-165 distance_coord_to_line_generic
__device__ __forceinline__ double coord_line_dist(double2 p, double2 a, double2 b) {
  if (a.x == b.x && a.y == b.y) return hypot(p.x - a.x, p.y - a.y);
  const double dx = b.x - a.x, dy = b.y - a.y;
  const double d2 = dx * dx + dy * dy;
  const double r = ((p.x - a.x) * dx + (p.y - a.y) * dy) / d2;
  if (r <= 0) return hypot(p.x - a.x, p.y - a.y);
  if (r >= 1) return hypot(p.x - b.x, p.y - b.y);
  const double s = ((a.y - p.y) * dx - (a.x - p.x) * dy) / d2;
  return fabs(s) * hypot(dx, dy);
}

// utils.rs:291-314 distance_line_to_line_generic
__device__ __forceinline__ double line_line_dist(double2 a1, double2 b1, double2 a2, double2 b2) {
  if (seg_intersects_seg(a1, b1, a2, b2)) return 0;
  const double d1 = coord_line_dist(a1, a2, b2), d2 = coord_line_dist(b1, a2, b2);
  const double d3 = coord_line_dist(a2, a1, b1), d4 = coord_line_dist(b2, a1, b1);
  return fmin(fmin(fmin(d1, d2), d3), d4);
}

// distance.rs:486-505 LineString to LineString (and utils.rs:36-73
// nearest_neighbour_distance, whose vertex passes cannot go below the segment
// pairs' minimum): min over segment pairs, 0 at the first pair that meets
__device__ __noinline__ double ring_ring_dist(const GeomsView& G1, uint32_t r1,
                                              const GeomsView& G2, uint32_t r2) {
  double m = DBL_MAX;
  const uint32_t V1 = G1.ring_vtx[r1], V2 = G2.ring_vtx[r2];
  const int n1 = G1.ring_nsegs[r1], n2 = G2.ring_nsegs[r2];
  for (int i = 0; i < n1; i++) {
    const double2 a1 = G1.xy[V1 + i], b1 = G1.xy[V1 + i + 1];
    for (int j = 0; j < n2; j++) {
      const double d = line_line_dist(a1, b1, G2.xy[V2 + j], G2.xy[V2 + j + 1]);
      if (d == 0) return 0;
      m = fmin(m, d);
    }
  }
  return m == DBL_MAX ? 0 : m;
}

// utils.rs:231-289 distance_point_to_polygon_generic (part q of G)
template <bool kFast>
__device__ __noinline__ double point_poly_dist(const GeomsView& G, uint32_t q, double2 p,
                                               float2 p32, uint32_t& esc) {
  if (poly_contains_point<kFast>(G, q, p, p32, true, esc)) return 0;
  double m = DBL_MAX;
  for (uint32_t r = G.part_ring[q]; r < G.part_ring[q + 1]; r++) {
    const uint32_t V = G.ring_vtx[r];
    const int ns = G.ring_nsegs[r];
    for (int i = 0; i < ns; i++) m = fmin(m, coord_line_dist(p, G.xy[V + i], G.xy[V + i + 1]));
  }
  return m;
}

// utils.rs:567-657 distance_polygon_to_polygon_generic (parts qa, qb)
template <bool kFast>
__device__ __noinline__ double poly_poly_dist(const GeomsView& GA, uint32_t qa,
                                              const GeomsView& GB, uint32_t qb, uint32_t& esc) {
  if (poly_intersects_poly<kFast>(GA, qa, GB, qb, esc)) return 0;
  const uint32_t a0 = GA.part_ring[qa], a1 = GA.part_ring[qa + 1];
  const uint32_t b0 = GB.part_ring[qb], b1 = GB.part_ring[qb + 1];
  if (a1 - a0 == 1 && b1 - b0 == 1) return ring_ring_dist(GA, a0, GB, b0);
  // b inside a (strictly inside a's shell at b's first point): the nearest
  // of a's holes; the same the other way round
  if (a1 - a0 > 1) {
    const uint32_t Vb = GB.ring_vtx[b0];
    if (ring_pip<kFast>(GA, a0, GB.xy[Vb], GB.xy32[Vb], false, esc).hit) {
      double m = DBL_MAX;
      for (uint32_t h = a0 + 1; h < a1; h++) m = fmin(m, ring_ring_dist(GB, b0, GA, h));
      return m;
    }
  }
  if (b1 - b0 > 1) {
    const uint32_t Va = GA.ring_vtx[a0];
    if (ring_pip<kFast>(GB, b0, GA.xy[Va], GA.xy32[Va], false, esc).hit) {
      double m = DBL_MAX;
      for (uint32_t h = b0 + 1; h < b1; h++) m = fmin(m, ring_ring_dist(GA, a0, GB, h));
      return m;
    }
  }
  return ring_ring_dist(GA, a0, GB, b0);
}

// build.distance_ext(probe) between two rows of which at least one is not
// a point: a multipolygon is the minimum over its parts (distance.rs:224-246);
// an empty part has distance 0 (utils.rs:236-238)
template <bool kFast>
__device__ __noinline__ double row_distance(const GeomsView& GA, uint32_t ia, const GeomsView& GB,
                                            uint32_t ib, uint32_t& esc) {
  const uint8_t ka = GA.kind[ia], kb = GB.kind[ib];
  if (ka == kEmpty || kb == kEmpty) return 0;
  if (has_empty_parts(GA, ia) || has_empty_parts(GB, ib)) return 0;
  double m = DBL_MAX;
  if (ka == kPoint || kb == kPoint) {
    const GeomsView& GY = ka == kPoint ? GB : GA;
    const GeomsView& GP = ka == kPoint ? GA : GB;
    const uint32_t iy = ka == kPoint ? ib : ia, ip = ka == kPoint ? ia : ib;
    const double2 p = GP.pt[ip];
    const float4 pb = GP.box[ip];
    for (uint32_t q = GY.row_part[iy]; q < GY.row_part[iy + 1]; q++)
      m = fmin(m, point_poly_dist<kFast>(GY, q, p, make_float2(pb.x, pb.y), esc));
    return m;
  }
  for (uint32_t qa = GA.row_part[ia]; qa < GA.row_part[ia + 1]; qa++)
    for (uint32_t qb = GB.row_part[ib]; qb < GB.row_part[ib + 1]; qb++)
      m = fmin(m, poly_poly_dist<kFast>(GA, qa, GB, qb, esc));
  return m;
}

}  // namespace
}  // namespace pred
}  // namespace spj
