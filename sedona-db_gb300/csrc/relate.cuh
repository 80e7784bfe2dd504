// relate.cuh — device restatement of tg's polygon-polygon relations, which the
// reference CPU join's default refiner evaluates as tg_geom_<pred>(build,
// probe) (rust/sedona-spatial-join/src/refine/tg.rs:322-357):
//   ring contains segment / ring    tg.c:2910-3039, 3120-3156
//   ring intersects segment / ring  tg.c:3046-3113, 3166-3192
//   polygon covers / intersects / touches polygon (holes)  tg.c:4040-4262
//   dispatch over polygons and multipolygons               tg.c:5544-6789
// Every decision repeats tg's FP64 operation sequence (predicates.cuh).  The
// FP32 tiers only skip work whose FP64 outcome they prove: a segment whose
// RN32 rect is strictly separated from the query's fails tg's first test, and
// decided orientations (orient32) prove a segment pair disjoint, or crossing
// properly (then no endpoint of either lies on the other, so none of tg's ON
// exceptions apply).  Where tg's visit order matters (the segment test
// without edges keeps state) the segments are visited in tg's order.
#pragma once
#include "predicates.cuh"
#include "relate_flags.cuh"

namespace spj {
namespace pred {
namespace {

__device__ __forceinline__ uint8_t ring_flags_of(const GeomsView& G, uint32_t r) {
  if (G.ring_flags) return G.ring_flags[r];
  const uint32_t V = G.ring_vtx[r];
  return tg_ring_flags(G.xy + V, G.ring_vtx[r + 1] - V - 1);
}

struct Seg {
  double2 a, b;
  float2 a32, b32;
};

__device__ __forceinline__ Seg ring_segment(const GeomsView& G, uint32_t r, int i) {
  const uint32_t V = G.ring_vtx[r];
  return Seg{G.xy[V + i], G.xy[V + i + 1], G.xy32[V + i], G.xy32[V + i + 1]};
}

// FP32 classification of tg_segment_intersects_segment((a, b), (c, d)) on
// RN32 copies: 0 proven false, 1 proven true (a proper crossing), -1 open.
__device__ __forceinline__ int seg_x32(float2 a, float2 b, float2 c, float2 d) {
  if (fmin0f(c.x, d.x) > fmax0f(a.x, b.x) || fmax0f(c.x, d.x) < fmin0f(a.x, b.x) ||
      fmin0f(c.y, d.y) > fmax0f(a.y, b.y) || fmax0f(c.y, d.y) < fmin0f(a.y, b.y))
    return 0;
  const int o1 = orient32(a, b, c), o2 = orient32(a, b, d);
  if (o1 != 0 && o1 == o2) return 0;
  const int o3 = orient32(c, d, a), o4 = orient32(c, d, b);
  if (o3 != 0 && o3 == o4) return 0;
  if (o1 != 0 && o2 != 0 && o3 != 0 && o4 != 0) return 1;
  return -1;
}

// Calls f(i) for the segments i of ring r whose rect may meet the closed rect
// [qx0, qx1] x [qy0, qy1] (RN32 bounds of a query), each at most once; the
// FP32 form leaves out segments whose RN32 rect is strictly separated (tg's
// rect test fails for them).  f returns true to stop; returns whether it
// stopped.  With a band index (both forms) only the query's bands are read,
// up to the entries whose key (RN32 xmax) is strictly left of the query.
template <bool kFast, class F>
__device__ __forceinline__ bool any_segment_near(const GeomsView& G, uint32_t r, float qx0,
                                                 float qy0, float qx1, float qy1, F&& f) {
  if (G.ring_bands != nullptr && G.band_param[r].y >= 0.0f) {
    const uint32_t B = G.ring_bands[r];
    const int nb = (int)(G.ring_bands[r + 1] - B) - 1;
    const float2 prm = G.band_param[r];
    const int b0 = band_of(qy0, prm.x, prm.y, nb), b1 = band_of(qy1, prm.x, prm.y, nb);
    for (int bb = b0; bb <= b1; bb++) {
      const uint32_t e0 = G.band_off[B + bb], e1 = G.band_off[B + bb + 1];
      for (uint32_t k = e0; k < e1; k++) {
        const float4 sg = G.band_seg[k];
        // xmax descending: the rest of the band is strictly left of the query
        if (fmax0f(sg.x, sg.z) < qx0) break;
        // each segment once: in the first band of the query that it spans
        if (bb > b0 && band_of(fmin0f(sg.y, sg.w), prm.x, prm.y, nb) < bb) continue;
        if (kFast && (fmin0f(sg.x, sg.z) > qx1 || fmax0f(sg.y, sg.w) < qy0 ||
                      fmin0f(sg.y, sg.w) > qy1))
          continue;
        if (f((int)G.band_edges[k])) return true;
      }
    }
    return false;
  }
  const uint32_t V = G.ring_vtx[r];
  const int ns = G.ring_nsegs[r];
  for (int i = 0; i < ns; i++) {
    if (kFast) {
      const float2 c = G.xy32[V + i], d = G.xy32[V + i + 1];
      if (fmin0f(c.x, d.x) > qx1 || fmax0f(c.x, d.x) < qx0 || fmin0f(c.y, d.y) > qy1 ||
          fmax0f(c.y, d.y) < qy0)
        continue;
    }
    if (f(i)) return true;
  }
  return false;
}

// tg.c:2910-3039 tg_ring_contains_segment.  tg's searches (tg_ring_search)
// ask whether any segment meets a condition that starts with
// tg_segment_intersects_segment(query, segment), so neither their visit
// order nor their rect filter changes the answer.  ring_pip reports tg's ON
// edge index (the last ON segment in index order).  carry: on entry the
// point-in-ring result of q.a when known (idx != kNoCarry), the previous
// segment's end point; on return q.b's result when it was computed (the next
// segment's start point), else kNoCarry.
constexpr int kNoCarry = -0x7fffffff;
template <bool kFast>
__device__ __noinline__ bool ring_contains_segment(const GeomsView& G, uint32_t r, const Seg q,
                                                   bool aoe, uint32_t& esc, RingHit* carry) {
  const RingHit known = *carry;
  carry->idx = kNoCarry;
  const Rect64 R = G.ring_rect[r];
  if (fmin0(q.a.x, q.b.x) < R.x || fmax0(q.a.x, q.b.x) > R.z || fmin0(q.a.y, q.b.y) < R.y ||
      fmax0(q.a.y, q.b.y) > R.w)
    return false;
  const RingHit ha = known.idx != kNoCarry ? known : ring_pip<kFast>(G, r, q.a, q.a32, aoe, esc);
  if (!ha.hit) return false;
  if (pteq(q.b, q.a)) return true;
  const RingHit hb = ring_pip<kFast>(G, r, q.b, q.b32, aoe, esc);
  *carry = hb;
  if (!hb.hit) return false;
  const uint8_t fl = ring_flags_of(G, r);
  if (fl & kRingConvex) return true;
  // which of tg's segment visitors decides (contsegiter1..5)
  int mode = 3;
  if (aoe) {
    if (ha.idx != -1 && hb.idx != -1) {
      if (ha.idx == hb.idx) return true;
      Seg sa = ring_segment(G, r, ha.idx), sb = ring_segment(G, r, hb.idx);
      if (pteq(sa.a, q.a) || pteq(sa.b, q.a) || pteq(sb.a, q.a) || pteq(sb.b, q.a) ||
          pteq(sa.a, q.b) || pteq(sa.b, q.b) || pteq(sb.a, q.b) || pteq(sb.b, q.b))
        return true;
      if (hb.idx < ha.idx) {
        const Seg t = sa;
        sa = sb;
        sb = t;
      }
      // winding of the ring made of the two edges (tg.c:2977-2990)
      const double2 w[5] = {sa.a, sa.b, sb.a, sb.b, sa.a};
      double cwc = 0.0;
      for (int i = 0; i < 4; i++)
        cwc = __dadd_rn(cwc, __dmul_rn(__dsub_rn(w[i + 1].x, w[i].x), __dadd_rn(w[i + 1].y, w[i].y)));
      if ((cwc > 0) != ((fl & kRingClockwise) != 0)) return false;
      mode = 1;
    } else if (ha.idx != -1) {
      mode = 4;
    } else if (hb.idx != -1) {
      mode = 2;
    } else {
      mode = 5;
    }
  }
  const bool hit = any_segment_near<kFast>(
      G, r, fmin0f(q.a32.x, q.b32.x), fmin0f(q.a32.y, q.b32.y), fmax0f(q.a32.x, q.b32.x),
      fmax0f(q.a32.y, q.b32.y), [&](int i) {
        const Seg s = ring_segment(G, r, i);
        if (kFast) {
          const int c = seg_x32(q.a32, q.b32, s.a32, s.b32);
          if (c == 0) return false;
          if (c == 1) return true;  // a proper crossing meets every visitor's condition
          esc++;
        }
        if (!seg_intersects_seg(q.a, q.b, s.a, s.b)) return false;
        switch (mode) {
          case 1:
            return raycast(s.a, s.b, q.a) != kOn && raycast(s.a, s.b, q.b) != kOn;
          case 4:
            return raycast(s.a, s.b, q.a) != kOn;
          case 2:
            return raycast(s.a, s.b, q.b) != kOn;
          case 5:
            return raycast(q.a, q.b, s.a) != kOn && raycast(q.a, q.b, s.b) != kOn;
          default:
            return true;
        }
      });
  return !hit;
}

// tg.c:3046-3113 tg_ring_intersects_segment.  With allow_on_edge the visitor
// counts intersecting segments up to two (any order).  Without it the
// visitor keeps state (a collinear overlap resets the count; the first
// shared endpoint of each query end is passed over once), so segments are
// visited in tg_ring_search's order: ascending index.  Segments that do not
// intersect the query leave the state alone, so skipping them is exact.
template <bool kFast>
__device__ __noinline__ bool ring_intersects_segment(const GeomsView& G, uint32_t r, const Seg q,
                                                     bool aoe, uint32_t& esc) {
  const Rect64 R = G.ring_rect[r];
  if (fmin0(q.a.x, q.b.x) > R.z || fmax0(q.a.x, q.b.x) < R.x || fmin0(q.a.y, q.b.y) > R.w ||
      fmax0(q.a.y, q.b.y) < R.y)
    return false;
  if (ring_pip<kFast>(G, r, q.a, q.a32, aoe, esc).hit ||
      ring_pip<kFast>(G, r, q.b, q.b32, aoe, esc).hit)
    return true;
  if (aoe) return ring_seg_hits<kFast>(G, r, q.a, q.b, q.a32, q.b32, esc) >= 2;
  const uint32_t V = G.ring_vtx[r];
  const int ns = G.ring_nsegs[r];
  int count = 0;
  bool a_on = false, b_on = false;
  for (int i = 0; i < ns && count < 2; i++) {
    const Seg s{G.xy[V + i], G.xy[V + i + 1], G.xy32[V + i], G.xy32[V + i + 1]};
    if (kFast) {
      const int c = seg_x32(q.a32, q.b32, s.a32, s.b32);
      if (c == 0) continue;
      if (c == 1) {  // proper crossing: not collinear, no shared endpoint
        count++;
        continue;
      }
      esc++;
    }
    if (!seg_intersects_seg(q.a, q.b, s.a, s.b)) continue;
    const bool ccol = collinear(q.a.x, q.a.y, q.b.x, q.b.y, s.a.x, s.a.y);
    const bool dcol = collinear(q.a.x, q.a.y, q.b.x, q.b.y, s.b.x, s.b.y);
    if (ccol && dcol) {
      count = 0;  // parallel
      continue;
    }
    if (!a_on && (pteq(q.a, s.a) || pteq(q.a, s.b))) {
      a_on = true;
      continue;
    }
    if (!b_on && (pteq(q.b, s.a) || pteq(q.b, s.b))) {
      b_on = true;
      continue;
    }
    count++;
  }
  return count >= 2;
}

// tg.c:3120-3156 tg_ring_contains_ring
template <bool kFast>
__device__ __noinline__ bool ring_contains_ring(const GeomsView& GA, uint32_t ra,
                                                const GeomsView& GB, uint32_t rb, bool aoe,
                                                uint32_t& esc) {
  if (ring_npts(GA, ra) < 3 || ring_npts(GB, rb) < 3) return false;
  const Rect64 A = GA.ring_rect[ra], Bq = GB.ring_rect[rb];
  if (Bq.x < A.x || Bq.z > A.z || Bq.y < A.y || Bq.w > A.w) return false;
  if (kFast) {
    // b's box in clean cells of a: every point of b strictly inside (1) or
    // outside (2) a, and no edge of a meets b, whatever allow_on_edge says
    const int st = grid_rect_status(GA, ra, Bq, GB.ring_rect32[rb]);
    if (st != 0) return st == 1;
    // no edge of a near b's box (ring_isolation): b lies strictly inside or
    // strictly outside a.  Inside, every point of b is inside a and no
    // segment of b meets an edge of a, so tg's point tests (convex a) and
    // segment tests (tg_ring_contains_segment: both ends in, no edge met)
    // all pass; outside, the first vertex's test fails.  allow_on_edge
    // changes neither.
    const int iso = ring_isolation<kFast>(GA, ra, GB, rb, esc);
    if (iso >= 0) return iso == 1;
  }
  const uint32_t Vb = GB.ring_vtx[rb];
  if (ring_flags_of(GA, ra) & kRingConvex) {
    const uint32_t n = ring_npts(GB, rb);
    for (uint32_t i = 0; i < n; i++)
      if (!ring_pip<kFast>(GA, ra, GB.xy[Vb + i], GB.xy32[Vb + i], aoe, esc).hit) return false;
    return true;
  }
  const int ns = GB.ring_nsegs[rb];
  // consecutive segments share a vertex: its point-in-ring result carries over
  RingHit carry{false, kNoCarry};
  for (int i = 0; i < ns; i++)
    if (!ring_contains_segment<kFast>(GA, ra, ring_segment(GB, rb, i), aoe, esc, &carry))
      return false;
  return true;
}

// tg.c:3166-3192 tg_ring_intersects_ring.  With allow_on_edge it is
// ring_intersects_ring of predicates.cuh (its isolation exit included).
template <bool kFast>
__device__ __noinline__ bool ring_intersects_ring_aoe(const GeomsView& GA, uint32_t ra,
                                                      const GeomsView& GB, uint32_t rb, bool aoe,
                                                      uint32_t& esc) {
  if (aoe) return ring_intersects_ring<kFast>(GA, ra, GB, rb, esc) == 1;
  if (ring_npts(GA, ra) < 3 || ring_npts(GB, rb) < 3) return false;
  if (!ring_rects_intersect<kFast>(GA, ra, GB, rb)) return false;
  const GeomsView* Gr = &GA;
  const GeomsView* Go = &GB;
  uint32_t rr = ra, ro = rb;
  if (swap_rings<kFast>(GA, ra, GB, rb)) {
    Gr = &GB;
    Go = &GA;
    rr = rb;
    ro = ra;
  }
  const int nso = Go->ring_nsegs[ro];
  for (int i = 0; i < nso; i++)
    if (ring_intersects_segment<kFast>(*Gr, rr, ring_segment(*Go, ro, i), false, esc)) return true;
  return false;
}

// tg_line_covers_point over a ring's segments (tg.c:3436-3443)
template <bool kFast>
__device__ __forceinline__ bool ring_covers_point_as_line(const GeomsView& G, uint32_t r,
                                                          double2 p, float2 p32, uint32_t& esc) {
  const uint32_t V = G.ring_vtx[r];
  const int ns = G.ring_nsegs[r];
  for (int i = 0; i < ns; i++) {
    if (kFast) {
      const float2 a = G.xy32[V + i], b = G.xy32[V + i + 1];
      if (p32.x < fmin0f(a.x, b.x) || p32.x > fmax0f(a.x, b.x) || p32.y < fmin0f(a.y, b.y) ||
          p32.y > fmax0f(a.y, b.y))
        continue;
      esc++;
    }
    if (point_on_segment(p, G.xy[V + i], G.xy[V + i + 1])) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// polygons (parts): ring 0 of a part is its shell, the rest its holes; a part
// with one ring is a tg ring (tg.c:3785-3789) and takes the ring fast paths

// tg.c:4040-4092 tg_poly_covers_poly (= tg_poly_contains_poly, tg.c:4094)
template <bool kFast>
__device__ __noinline__ bool poly_covers_poly(const GeomsView& GA, uint32_t qa,
                                              const GeomsView& GB, uint32_t qb, uint32_t& esc) {
  const uint32_t a0 = GA.part_ring[qa], a1 = GA.part_ring[qa + 1];
  const uint32_t b0 = GB.part_ring[qb], b1 = GB.part_ring[qb + 1];
  if (a1 - a0 == 1 && b1 - b0 == 1) return ring_contains_ring<kFast>(GA, a0, GB, b0, true, esc);
  if (ring_npts(GA, a0) < 3 || ring_npts(GB, b0) < 3) return false;
  if (!ring_contains_ring<kFast>(GA, a0, GB, b0, true, esc)) return false;
  for (uint32_t h = a0 + 1; h < a1; h++) {
    if (ring_contains_ring<kFast>(GA, h, GB, b0, true, esc) ||
        ring_intersects_ring_aoe<kFast>(GA, h, GB, b0, false, esc)) {
      // unless the hole lies inside one of b's holes
      bool covered = false;
      for (uint32_t g = b0 + 1; g < b1 && !covered; g++)
        covered = ring_contains_ring<kFast>(GB, g, GA, h, true, esc);
      if (!covered) return false;
    }
  }
  return true;
}

// tg.c:4100-4136 tg_poly_intersects_poly
template <bool kFast>
__device__ __noinline__ bool poly_intersects_poly(const GeomsView& GA, uint32_t qa,
                                                  const GeomsView& GB, uint32_t qb,
                                                  uint32_t& esc) {
  const uint32_t a0 = GA.part_ring[qa], a1 = GA.part_ring[qa + 1];
  const uint32_t b0 = GB.part_ring[qb], b1 = GB.part_ring[qb + 1];
  if (a1 - a0 == 1 && b1 - b0 == 1) return ring_intersects_ring<kFast>(GA, a0, GB, b0, esc) == 1;
  if (ring_npts(GA, a0) < 3 || ring_npts(GB, b0) < 3) return false;
  if (!ring_intersects_ring_aoe<kFast>(GB, b0, GA, a0, true, esc)) return false;
  for (uint32_t h = a0 + 1; h < a1; h++)
    if (ring_contains_ring<kFast>(GA, h, GB, b0, false, esc)) return false;
  for (uint32_t h = b0 + 1; h < b1; h++)
    if (ring_contains_ring<kFast>(GB, h, GA, a0, false, esc)) return false;
  return true;
}

// tg.c:4184-4262 tg_poly_touches_poly
template <bool kFast>
__device__ __noinline__ bool poly_touches_poly(const GeomsView& GA, uint32_t qa,
                                               const GeomsView& GB, uint32_t qb, uint32_t& esc) {
  const uint32_t a0 = GA.part_ring[qa], a1 = GA.part_ring[qa + 1];
  const uint32_t b0 = GB.part_ring[qb], b1 = GB.part_ring[qb + 1];
  if (!ring_rects_intersect<kFast>(GA, a0, GB, b0)) return false;
  if (kFast && a1 - a0 == 1 && b1 - b0 == 1) {
    // two single rings, no edge of one near the other's box (ring_isolation):
    // the other lies strictly inside or strictly outside, so the boundaries
    // do not meet.  Inside, its segments' ends are in the ring with and
    // without allow_on_edge (the loop below returns false); outside, no
    // segment of either ring meets the other ring (no touches counted).
    if (ring_isolation<kFast>(GA, a0, GB, b0, esc) >= 0) return false;
    if (ring_isolation<kFast>(GB, b0, GA, a0, esc) >= 0) return false;
  }
  // one polygon inside a hole of the other, touching the hole's boundary
  for (int ii = 0; ii < 2; ii++) {
    const GeomsView& GP = ii == 0 ? GA : GB;
    const GeomsView& GR = ii == 0 ? GB : GA;
    const uint32_t h0 = (ii == 0 ? a0 : b0) + 1, h1 = ii == 0 ? a1 : b1;
    const uint32_t ring = ii == 0 ? b0 : a0;
    for (uint32_t h = h0; h < h1; h++) {
      if (ring_contains_ring<kFast>(GP, h, GR, ring, true, esc)) {
        const uint32_t V = GR.ring_vtx[ring], n = ring_npts(GR, ring);
        for (uint32_t j = 0; j < n; j++)
          if (ring_covers_point_as_line<kFast>(GP, h, GR.xy[V + j], GR.xy32[V + j], esc))
            return true;
        return false;
      }
    }
  }
  const int ansegs = GA.ring_nsegs[a0], bnsegs = GB.ring_nsegs[b0];
  int atouches = 0, btouches = 0;
  for (int ii = 0; ii < 2; ii++) {
    const GeomsView& Ga = ii == 0 ? GA : GB;
    const GeomsView& Gb = ii == 0 ? GB : GA;
    const uint32_t ra = ii == 0 ? a0 : b0, rb = ii == 0 ? b0 : a0;
    const int nsegs = ii == 0 ? bnsegs : ansegs;
    int touches = 0;
    for (int i = 0; i < nsegs; i++) {
      const Seg seg = ring_segment(Gb, rb, i);
      const bool i0 = ring_intersects_segment<kFast>(Ga, ra, seg, true, esc);
      const bool i1 = ring_intersects_segment<kFast>(Ga, ra, seg, false, esc);
      if (i0 && !i1) touches++;
      else if (i0 || i1) return false;
    }
    if (ii == 0) btouches = touches;
    else atouches = touches;
  }
  if (atouches > 0 || btouches > 0) return !(atouches == ansegs && btouches == bnsegs);
  return false;
}

// ---------------------------------------------------------------------------
// rows: dispatch over polygon / multipolygon parts (and point rows where a
// multipolygon meets a point), as tg's geometry-level predicates do

__device__ __forceinline__ bool is_polygonal(uint8_t k) {
  return k == kPolygon || k == kMultiPolygon;
}
__device__ __forceinline__ bool has_empty_parts(const GeomsView& G, uint32_t i) {
  return G.row_flags != nullptr && (G.row_flags[i] & 1);
}

// intersects between two polygonal rows: any pair of parts, a's part first
// (poly_intersects_geom / multiiter, tg.c:5648-5738)
template <bool kFast>
__device__ __noinline__ bool row_intersects_rows(const GeomsView& GA, uint32_t ia,
                                                 const GeomsView& GB, uint32_t ib,
                                                 uint32_t& esc) {
  for (uint32_t qa = GA.row_part[ia]; qa < GA.row_part[ia + 1]; qa++)
    for (uint32_t qb = GB.row_part[ib]; qb < GB.row_part[ib + 1]; qb++)
      if (poly_intersects_poly<kFast>(GA, qa, GB, qb, esc)) return true;
  return false;
}

// covers between two polygonal rows (tg.c:5869-6026): a polygon must cover
// every part of b (an empty part of b fails it); a multipolygon must cover
// each part of b with one of its parts
template <bool kFast>
__device__ __noinline__ bool row_covers_rows(const GeomsView& GA, uint32_t ia,
                                             const GeomsView& GB, uint32_t ib, uint32_t& esc) {
  const uint32_t pa0 = GA.row_part[ia], pa1 = GA.row_part[ia + 1];
  const uint32_t pb0 = GB.row_part[ib], pb1 = GB.row_part[ib + 1];
  if (GA.kind[ia] == kPolygon) {
    if (has_empty_parts(GB, ib)) return false;
    for (uint32_t qb = pb0; qb < pb1; qb++)
      if (!poly_covers_poly<kFast>(GA, pa0, GB, qb, esc)) return false;
    return true;
  }
  for (uint32_t qb = pb0; qb < pb1; qb++) {
    bool found = false;
    for (uint32_t qa = pa0; qa < pa1 && !found; qa++)
      found = poly_covers_poly<kFast>(GA, qa, GB, qb, esc);
    if (!found) return false;
  }
  return true;
}

// contains between two polygonal rows (tg.c:6053-6106, 6477-6487): for a
// polygon a it is covers (tg_poly_contains_poly is tg_poly_covers_poly); for
// a multipolygon a, covers plus some part of b meeting the interior of some
// part of a (intersects and does not touch)
template <bool kFast>
__device__ __noinline__ bool row_contains_rows(const GeomsView& GA, uint32_t ia,
                                               const GeomsView& GB, uint32_t ib, uint32_t& esc) {
  if (!row_covers_rows<kFast>(GA, ia, GB, ib, esc)) return false;
  if (GA.kind[ia] == kPolygon) return true;
  for (uint32_t qb = GB.row_part[ib]; qb < GB.row_part[ib + 1]; qb++)
    for (uint32_t qa = GA.row_part[ia]; qa < GA.row_part[ia + 1]; qa++)
      if (poly_intersects_poly<kFast>(GA, qa, GB, qb, esc) &&
          !poly_touches_poly<kFast>(GA, qa, GB, qb, esc))
        return true;
  return false;
}

// touches(part qa of a, row ib of b), b a point or polygonal row
// (poly_touches_geom, tg.c:6679-6733)
template <bool kFast>
__device__ __forceinline__ bool part_touches_row(const GeomsView& GA, uint32_t qa,
                                                 const GeomsView& GB, uint32_t ib,
                                                 uint32_t& esc) {
  if (GB.kind[ib] == kPoint) {
    const float4 pb = GB.box[ib];
    return poly_touches_point<kFast>(GA, qa, GB.pt[ib], make_float2(pb.x, pb.y), esc);
  }
  const uint32_t pb0 = GB.row_part[ib], pb1 = GB.row_part[ib + 1];
  if (GB.kind[ib] == kPolygon) return poly_touches_poly<kFast>(GA, qa, GB, pb0, esc);
  bool touches = false;
  for (uint32_t qb = pb0; qb < pb1; qb++) {
    if (poly_touches_poly<kFast>(GA, qa, GB, qb, esc)) touches = true;
    else if (poly_intersects_poly<kFast>(GA, qa, GB, qb, esc)) return false;
  }
  return touches;
}

template <bool kFast>
__device__ __forceinline__ bool part_intersects_row(const GeomsView& GA, uint32_t qa,
                                                    const GeomsView& GB, uint32_t ib,
                                                    uint32_t& esc) {
  if (GB.kind[ib] == kPoint) {
    const float4 pb = GB.box[ib];
    return poly_contains_point<kFast>(GA, qa, GB.pt[ib], make_float2(pb.x, pb.y), true, esc);
  }
  for (uint32_t qb = GB.row_part[ib]; qb < GB.row_part[ib + 1]; qb++)
    if (poly_intersects_poly<kFast>(GA, qa, GB, qb, esc)) return true;
  return false;
}

// touches of a polygonal row a with a point or polygonal row b
// (tg.c:6735-6768 for a multipolygon: some part touches and no part meets
// b's interior)
template <bool kFast>
__device__ __noinline__ bool row_touches_row(const GeomsView& GA, uint32_t ia,
                                             const GeomsView& GB, uint32_t ib, uint32_t& esc) {
  const uint32_t pa0 = GA.row_part[ia], pa1 = GA.row_part[ia + 1];
  if (GA.kind[ia] == kPolygon) return part_touches_row<kFast>(GA, pa0, GB, ib, esc);
  bool touches = false;
  for (uint32_t qa = pa0; qa < pa1; qa++) {
    if (part_touches_row<kFast>(GA, qa, GB, ib, esc)) touches = true;
    else if (part_intersects_row<kFast>(GA, qa, GB, ib, esc)) return false;
  }
  return touches;
}

}  // namespace
}  // namespace pred
}  // namespace spj
