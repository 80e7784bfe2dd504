/*
 * spj_oracle.c — CPU oracle for the spatial-join hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs load
 * it.  The product library never links or calls it.
 *
 * Every predicate below restates the arithmetic of the tg library that the
 * reference CPU join uses as its default refiner (c/sedona-tg/src/tg/tg.c,
 * vendored at TG_REF e136401, c/sedona-tg/vendor-tg.sh:20).  The operation
 * order matters: the reference result is defined by tg's FP64 operation
 * sequence (including its division-based slope test), so the same sequence is
 * used here.  Build with -ffp-contract=off so no multiply-add is fused.
 */
#include "spj_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double x, y; } opt_t;
typedef struct { double minx, miny, maxx, maxy; } orect_t;
typedef struct { opt_t a, b; } oseg_t;

typedef struct {
  int32_t npts;   /* number of points as stored */
  int32_t nsegs;  /* tg num_segments (tg.c:2124-2134) */
  int64_t first;  /* index of first point in spj_geoms.pts; pts[first+npts] = pts[first] */
  orect_t rect;
  int convex, clockwise; /* tg's ring flags (tg.c:1910-2113 process_points) */
} oring_t;

typedef struct { int64_t first_ring; int32_t nrings; } opoly_t;

typedef struct {
  int8_t kind;
  opt_t pt;
  int64_t first_poly;
  int32_t npolys;
  int32_t empty_parts; /* a multipolygon that had parts without rings */
  orect_t rect;
} ogeom_t;

struct spj_geoms {
  int64_t n;
  ogeom_t* g;
  opoly_t* polys;
  int64_t npolys, cap_polys;
  oring_t* rings;
  int64_t nrings, cap_rings;
  opt_t* pts;
  int64_t npts, cap_pts;
  int64_t nvert;
};

/* ------------------------------------------------------------------------ */
/* tg numeric primitives                                                     */
/* ------------------------------------------------------------------------ */

/* tg.c:853-859 */
static inline int feq(double x, double y) { return !((x < y) | (x > y)); }
static inline int eq_zero(double x) { return feq(x, 0); }
/* tg.c:831-840 fmin0/fmax0 */
static inline double fmin0(double x, double y) { return x < y ? x : y; }
static inline double fmax0(double x, double y) { return x > y ? x : y; }

/* tg.c:861-900 */
static int collinear(double x1, double y1, double x2, double y2, double x3, double y3) {
  int x1x2 = feq(x1, x2), x1x3 = feq(x1, x3), x2x3 = feq(x2, x3);
  int y1y2 = feq(y1, y2), y1y3 = feq(y1, y3), y2y3 = feq(y2, y3);
  if (x1x2) return x1x3;
  if (y1y2) return y1y3;
  if ((x1x2 & y1y2) | (x1x3 & y1y3) | (x2x3 & y2y3)) return 1;
  double cx1 = x3 - x1, cy1 = y3 - y1;
  double cx2 = x2 - x1, cy2 = y2 - y1;
  double s1 = cx1 * cy2;
  double s2 = cy1 * cx2;
  double s3 = (s1 / cy2) - cx1;
  double s4 = (s2 / cx2) - cy1;
  if (s3 < 0) s1 = nextafter(s1, -INFINITY);
  else if (s3 > 0) s1 = nextafter(s1, INFINITY);
  if (s4 < 0) s2 = nextafter(s2, -INFINITY);
  else if (s4 > 0) s2 = nextafter(s2, INFINITY);
  return eq_zero(s1 - s2);
}

/* tg.c:1076-1078 */
static inline int pteq(opt_t a, opt_t b) { return feq(a.x, b.x) && feq(a.y, b.y); }

/* tg.c:1776-1785 */
static inline int rect_covers_point(orect_t r, opt_t p) {
  return !(p.x < r.minx || p.y < r.miny || p.x > r.maxx || p.y > r.maxy);
}
/* tg.c:1327-1330 (rect_intersects_rect(a, b)) */
static inline int rect_intersects_rect(orect_t a, orect_t b) {
  return !(b.minx > a.maxx || b.maxx < a.minx || b.miny > a.maxy || b.maxy < a.miny);
}
/* tg.c:1339-1342 */
static inline int rect_covers_rect(orect_t a, orect_t b) {
  return !(b.minx < a.minx || b.maxx > a.maxx || b.miny < a.miny || b.maxy > a.maxy);
}
/* tg.c:1311-1325 segment_fill_rect */
static inline orect_t seg_rect(oseg_t s) {
  orect_t r = {fmin0(s.a.x, s.b.x), fmin0(s.a.y, s.b.y), fmax0(s.a.x, s.b.x),
               fmax0(s.a.y, s.b.y)};
  return r;
}

/* tg.c:1192-1197 */
static int point_on_segment(opt_t p, oseg_t s) {
  if (!rect_covers_point(seg_rect(s), p)) return 0;
  return collinear(s.a.x, s.a.y, s.b.x, s.b.y, p.x, p.y);
}

enum { RC_OUT = 0, RC_IN = 1, RC_ON = 2 };

/* tg.c:1199-1276 raycast: +x ray from p against segment seg. */
static int raycast(oseg_t seg, opt_t p) {
  orect_t r = seg_rect(seg);
  if (p.y < r.miny || p.y > r.maxy) return RC_OUT;
  if (p.x < r.minx) {
    if (p.y != r.miny && p.y != r.maxy) return RC_IN;
  } else if (p.x > r.maxx) {
    if (r.miny != r.maxy && r.minx != r.maxx) return RC_OUT;
  }
  opt_t a = seg.a, b = seg.b;
  if (b.y < a.y) {
    opt_t t = a;
    a = b;
    b = t;
  }
  if (pteq(p, a) || pteq(p, b)) return RC_ON;
  if (a.y == b.y) {
    if (a.x == b.x) return RC_OUT;
    if (p.y == b.y) {
      if (!(p.x < r.minx || p.x > r.maxx)) return RC_ON;
    }
  }
  if (a.x == b.x && p.x == b.x) {
    if (p.y >= a.y && p.y <= b.y) return RC_ON;
  }
  if (collinear(a.x, a.y, b.x, b.y, p.x, p.y)) {
    if (p.x < r.minx) {
      if (r.miny == r.maxy) return RC_OUT;
    } else if (p.x > r.maxx) {
      return RC_OUT;
    }
    return RC_ON;
  }
  if (p.y == a.y || p.y == b.y) p.y = nextafter(p.y, INFINITY);
  if (p.y < a.y || p.y > b.y) return RC_OUT;
  if (a.x > b.x) {
    if (p.x >= a.x) return RC_OUT;
    if (p.x <= b.x) return RC_IN;
  } else {
    if (p.x >= b.x) return RC_OUT;
    if (p.x <= a.x) return RC_IN;
  }
  if ((p.y - a.y) / (p.x - a.x) >= (b.y - a.y) / (b.x - a.x)) return RC_IN;
  return RC_OUT;
}

/* tg.c:1392-1440 */
static int segment_intersects_segment(oseg_t sa, oseg_t sb) {
  opt_t a = sa.a, b = sa.b, c = sb.a, d = sb.b;
  if (!rect_intersects_rect(seg_rect(sa), seg_rect(sb))) return 0;
  if (pteq(sa.a, sb.a) || pteq(sa.a, sb.b) || pteq(sa.b, sb.a) || pteq(sa.b, sb.b)) return 1;
  double cmpx = c.x - a.x, cmpy = c.y - a.y;
  double rx = b.x - a.x, ry = b.y - a.y;
  double cmpxr = cmpx * ry - cmpy * rx;
  if (eq_zero(cmpxr)) {
    if (!(((c.x - a.x <= 0) != (c.x - b.x <= 0))) || ((c.y - a.y <= 0) != (c.y - b.y <= 0))) {
      return point_on_segment(sb.a, sa) || point_on_segment(sb.b, sa) ||
             point_on_segment(sa.a, sb) || point_on_segment(sa.b, sb);
    }
    return 1;
  }
  double sx = d.x - c.x, sy = d.y - c.y;
  double rxs = rx * sy - ry * sx;
  if (eq_zero(rxs)) return 0;
  double cmpxs = cmpx * sy - cmpy * sx;
  double rxsr = 1 / rxs;
  double t = cmpxs * rxsr;
  double u = cmpxr * rxsr;
  if (!((t >= 0) && (t <= 1) && (u >= 0) && (u <= 1))) return 0;
  return 1;
}

/* ------------------------------------------------------------------------ */
/* rings and polygons                                                        */
/* ------------------------------------------------------------------------ */

static inline oseg_t ring_seg(const spj_geoms* G, const oring_t* r, int i) {
  oseg_t s = {G->pts[r->first + i], G->pts[r->first + i + 1]};
  return s;
}

/* tg.c:3115-3118 (closed rings) */
static inline int ring_empty(const oring_t* r) { return r->npts < 3; }

typedef struct { int hit, idx; } ring_result;

/* tg.c:2809-2822 with the per-segment evaluation of tg.c:2668-2720.
 * Any iteration order gives the same hit: once a segment reports ON the
 * result is allow_on_edge and IN toggles stop; otherwise it is the parity of
 * IN segments.  idx is the last ON segment in increasing order. */
static ring_result ring_contains_point(const spj_geoms* G, const oring_t* r, opt_t p,
                                       int allow_on_edge) {
  ring_result res = {0, -1};
  if (!rect_covers_point(r->rect, p)) return res;
  int in = 0, idx = -1;
  for (int i = 0; i < r->nsegs; i++) {
    oseg_t s = ring_seg(G, r, i);
    double ymin = fmin0(s.a.y, s.b.y), ymax = fmax0(s.a.y, s.b.y);
    if (p.y < ymin || p.y > ymax) continue;
    switch (raycast(s, p)) {
      case RC_OUT:
        break;
      case RC_IN:
        if (idx == -1) in = !in;
        break;
      case RC_ON:
        in = allow_on_edge;
        idx = i;
        break;
    }
  }
  res.hit = in;
  res.idx = idx;
  return res;
}

/* tg.c:3909-3934 (a polygon without holes is a tg ring, tg.c:3785-3789) */
static int poly_contains_point(const spj_geoms* G, const opoly_t* P, opt_t p, int allow_on_edge) {
  const oring_t* ext = &G->rings[P->first_ring];
  if (P->nrings == 1) return ring_contains_point(G, ext, p, allow_on_edge).hit;
  if (ring_empty(ext)) return 0;
  if (!ring_contains_point(G, ext, p, allow_on_edge).hit) return 0;
  for (int h = 1; h < P->nrings; h++) {
    if (ring_contains_point(G, &G->rings[P->first_ring + h], p, !allow_on_edge).hit) return 0;
  }
  return 1;
}

/* tg.c:3436-3443 tg_line_covers_point over a ring's segments */
static int ring_covers_point_as_line(const spj_geoms* G, const oring_t* r, opt_t p) {
  for (int i = 0; i < r->nsegs; i++)
    if (point_on_segment(p, ring_seg(G, r, i))) return 1;
  return 0;
}

/* tg.c:1171-1190 tg_point_touches_poly */
static int poly_touches_point(const spj_geoms* G, const opoly_t* P, opt_t p) {
  for (int h = 0; h < P->nrings; h++)
    if (ring_covers_point_as_line(G, &G->rings[P->first_ring + h], p)) return 1;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* ring relations (tg.c:2910-3192)                                          */
/* ------------------------------------------------------------------------ */

/* tg_segment_rect(seg) intersects tg_segment_rect(other) (tg.c:1311-1330) */
static inline int seg_rects_intersect(oseg_t a, oseg_t b) {
  return rect_intersects_rect(seg_rect(a), seg_rect(b));
}

/* tg.c:2910-3039 tg_ring_contains_segment.  tg_ring_search (tg.c:2468-2485)
 * visits the segments whose rect meets the query's; every visitor below asks
 * "does any segment ..." and each test starts with the same rect test, so a
 * plain loop over all segments gives the same answer. */
static int ring_contains_segment(const spj_geoms* G, const oring_t* ring, oseg_t seg,
                                 int allow_on_edge) {
  if (!rect_covers_rect(ring->rect, seg_rect(seg))) return 0;
  ring_result ra = ring_contains_point(G, ring, seg.a, allow_on_edge);
  if (!ra.hit) return 0;
  if (pteq(seg.b, seg.a)) return 1;
  ring_result rb = ring_contains_point(G, ring, seg.b, allow_on_edge);
  if (!rb.hit) return 0;
  if (ring->convex) return 1;
  if (allow_on_edge) {
    if (ra.idx != -1) {
      if (rb.idx != -1) {
        if (rb.idx == ra.idx) return 1;
        oseg_t sa = ring_seg(G, ring, ra.idx), sb = ring_seg(G, ring, rb.idx);
        if (pteq(sa.a, seg.a) || pteq(sa.b, seg.a) || pteq(sb.a, seg.a) || pteq(sb.b, seg.a) ||
            pteq(sa.a, seg.b) || pteq(sa.b, seg.b) || pteq(sb.a, seg.b) || pteq(sb.b, seg.b))
          return 1;
        if (rb.idx < ra.idx) {
          oseg_t t = sa;
          sa = sb;
          sb = t;
        }
        /* winding of the ring made of the two edges (tg.c:2977-2990) */
        opt_t q[5] = {sa.a, sa.b, sb.a, sb.b, sa.a};
        double cwc = 0.0;
        for (int i = 0; i < 4; i++) cwc += (q[i + 1].x - q[i].x) * (q[i + 1].y + q[i].y);
        int clockwise = cwc > 0;
        if (clockwise != ring->clockwise) return 0;
        for (int i = 0; i < ring->nsegs; i++) { /* contsegiter1 */
          oseg_t s = ring_seg(G, ring, i);
          if (segment_intersects_segment(seg, s) && raycast(s, seg.a) != RC_ON &&
              raycast(s, seg.b) != RC_ON)
            return 0;
        }
        return 1;
      }
      for (int i = 0; i < ring->nsegs; i++) { /* contsegiter4 */
        oseg_t s = ring_seg(G, ring, i);
        if (segment_intersects_segment(seg, s) && raycast(s, seg.a) != RC_ON) return 0;
      }
      return 1;
    } else if (rb.idx != -1) {
      for (int i = 0; i < ring->nsegs; i++) { /* contsegiter2 */
        oseg_t s = ring_seg(G, ring, i);
        if (segment_intersects_segment(seg, s) && raycast(s, seg.b) != RC_ON) return 0;
      }
      return 1;
    }
    for (int i = 0; i < ring->nsegs; i++) { /* contsegiter5 */
      oseg_t s = ring_seg(G, ring, i);
      if (segment_intersects_segment(seg, s) && raycast(seg, s.a) != RC_ON &&
          raycast(seg, s.b) != RC_ON)
        return 0;
    }
    return 1;
  }
  for (int i = 0; i < ring->nsegs; i++) { /* contsegiter3 */
    if (segment_intersects_segment(seg, ring_seg(G, ring, i))) return 0;
  }
  return 1;
}

/* tg.c:3046-3113 tg_ring_intersects_segment.  With allow_on_edge the visitor
 * counts intersecting segments up to two (order does not matter).  Without
 * it the visitor keeps state (a collinear overlap resets the count, the first
 * shared endpoint of each query end is skipped once), so the segments are
 * visited as tg_ring_search does: ascending index, those whose rect meets
 * the query's rect. */
static int ring_intersects_segment(const spj_geoms* G, const oring_t* ring, oseg_t seg,
                                   int allow_on_edge) {
  if (!rect_intersects_rect(seg_rect(seg), ring->rect)) return 0;
  if (ring_contains_point(G, ring, seg.a, allow_on_edge).hit ||
      ring_contains_point(G, ring, seg.b, allow_on_edge).hit)
    return 1;
  int count = 0, a_on = 0, b_on = 0;
  opt_t a = seg.a, b = seg.b;
  for (int i = 0; i < ring->nsegs && count < 2; i++) {
    oseg_t s = ring_seg(G, ring, i);
    if (!seg_rects_intersect(s, seg)) continue;
    if (!segment_intersects_segment(seg, s)) continue;
    if (allow_on_edge) {
      count++;
      continue;
    }
    opt_t c = s.a, d = s.b;
    int ccol = collinear(a.x, a.y, b.x, b.y, c.x, c.y);
    int dcol = collinear(a.x, a.y, b.x, b.y, d.x, d.y);
    if (ccol && dcol) {
      count = 0; /* parallel */
    } else {
      if (!a_on && (pteq(a, c) || pteq(a, d))) {
        a_on = 1;
        continue;
      }
      if (!b_on && (pteq(b, c) || pteq(b, d))) {
        b_on = 1;
        continue;
      }
      count++;
    }
  }
  return count >= 2;
}

static inline double rect_area(orect_t r) { return (r.maxx - r.minx) * (r.maxy - r.miny); }

/* tg.c:3120-3156 tg_ring_contains_ring */
static int ring_contains_ring(const spj_geoms* GA, const oring_t* a, const spj_geoms* GB,
                              const oring_t* b, int allow_on_edge) {
  if (ring_empty(a) || ring_empty(b)) return 0;
  if (!rect_covers_rect(a->rect, b->rect)) return 0;
  if (a->convex) {
    for (int i = 0; i < b->npts; i++)
      if (!ring_contains_point(GA, a, GB->pts[b->first + i], allow_on_edge).hit) return 0;
  } else {
    for (int i = 0; i < b->nsegs; i++)
      if (!ring_contains_segment(GA, a, ring_seg(GB, b, i), allow_on_edge)) return 0;
  }
  return 1;
}

/* tg.c:3166-3192 tg_ring_intersects_ring */
static int ring_intersects_ring(const spj_geoms* GA, const oring_t* ring, const spj_geoms* GB,
                                const oring_t* other, int allow_on_edge) {
  if (ring_empty(ring) || ring_empty(other)) return 0;
  if (!rect_intersects_rect(ring->rect, other->rect)) return 0;
  double a1 = rect_area(ring->rect), a2 = rect_area(other->rect);
  if (a2 > a1) {
    const oring_t* t = ring;
    ring = other;
    other = t;
    const spj_geoms* tg = GA;
    GA = GB;
    GB = tg;
  }
  for (int i = 0; i < other->nsegs; i++) {
    if (ring_intersects_segment(GA, ring, ring_seg(GB, other, i), allow_on_edge)) return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* polygon relations (tg.c:4040-4262); a polygon without holes is its ring  */
/* (tg.c:3785-3789), which takes the ring fast paths                        */
/* ------------------------------------------------------------------------ */

static inline const oring_t* poly_ext(const spj_geoms* G, const opoly_t* P) {
  return &G->rings[P->first_ring];
}
static inline const oring_t* poly_hole(const spj_geoms* G, const opoly_t* P, int h) {
  return &G->rings[P->first_ring + 1 + h];
}

/* tg.c:4040-4092 tg_poly_covers_poly (= tg_poly_contains_poly, tg.c:4094-4096) */
static int poly_covers_poly(const spj_geoms* GA, const opoly_t* A, const spj_geoms* GB,
                            const opoly_t* B) {
  if (A->nrings == 1 && B->nrings == 1)
    return ring_contains_ring(GA, poly_ext(GA, A), GB, poly_ext(GB, B), 1);
  if (ring_empty(poly_ext(GA, A)) || ring_empty(poly_ext(GB, B))) return 0;
  const oring_t* bext = poly_ext(GB, B);
  if (!ring_contains_ring(GA, poly_ext(GA, A), GB, bext, 1)) return 0;
  int covers = 1;
  for (int i = 0; i < A->nrings - 1; i++) {
    const oring_t* h = poly_hole(GA, A, i);
    if (ring_contains_ring(GA, h, GB, bext, 1) || ring_intersects_ring(GA, h, GB, bext, 0)) {
      covers = 0;
      for (int j = 0; j < B->nrings - 1; j++) {
        if (ring_contains_ring(GB, poly_hole(GB, B, j), GA, h, 1)) {
          covers = 1;
          break;
        }
      }
      if (!covers) break;
    }
  }
  return covers;
}

/* tg.c:4100-4136 tg_poly_intersects_poly */
static int poly_intersects_poly(const spj_geoms* GA, const opoly_t* A, const spj_geoms* GB,
                                const opoly_t* B) {
  if (A->nrings == 1 && B->nrings == 1)
    return ring_intersects_ring(GA, poly_ext(GA, A), GB, poly_ext(GB, B), 1);
  if (ring_empty(poly_ext(GA, A)) || ring_empty(poly_ext(GB, B))) return 0;
  if (!ring_intersects_ring(GB, poly_ext(GB, B), GA, poly_ext(GA, A), 1)) return 0;
  for (int i = 0; i < A->nrings - 1; i++)
    if (ring_contains_ring(GA, poly_hole(GA, A, i), GB, poly_ext(GB, B), 0)) return 0;
  for (int i = 0; i < B->nrings - 1; i++)
    if (ring_contains_ring(GB, poly_hole(GB, B, i), GA, poly_ext(GA, A), 0)) return 0;
  return 1;
}

/* tg.c:4184-4262 tg_poly_touches_poly */
static int poly_touches_poly(const spj_geoms* GA, const opoly_t* A, const spj_geoms* GB,
                             const opoly_t* B) {
  const oring_t* aext = poly_ext(GA, A);
  const oring_t* bext = poly_ext(GB, B);
  if (!rect_intersects_rect(aext->rect, bext->rect)) return 0;
  /* one polygon inside a hole of the other, touching the hole's boundary */
  for (int ii = 0; ii < 2; ii++) {
    const spj_geoms* GP = ii == 0 ? GA : GB;
    const opoly_t* P = ii == 0 ? A : B;
    const spj_geoms* GR = ii == 0 ? GB : GA;
    const oring_t* ring = ii == 0 ? bext : aext;
    for (int i = 0; i < P->nrings - 1; i++) {
      const oring_t* hole = poly_hole(GP, P, i);
      if (ring_contains_ring(GP, hole, GR, ring, 1)) {
        for (int j = 0; j < ring->npts; j++)
          if (ring_covers_point_as_line(GP, hole, GR->pts[ring->first + j])) return 1;
        return 0;
      }
    }
  }
  int ansegs = aext->nsegs, bnsegs = bext->nsegs;
  int atouches = 0, btouches = 0;
  for (int ii = 0; ii < 2; ii++) {
    const spj_geoms* Ga = ii == 0 ? GA : GB;
    const oring_t* a = ii == 0 ? aext : bext;
    const spj_geoms* Gb = ii == 0 ? GB : GA;
    const oring_t* b = ii == 0 ? bext : aext;
    int nsegs = ii == 0 ? bnsegs : ansegs;
    int touches = 0;
    for (int i = 0; i < nsegs; i++) {
      oseg_t seg = ring_seg(Gb, b, i);
      int i0 = ring_intersects_segment(Ga, a, seg, 1);
      int i1 = ring_intersects_segment(Ga, a, seg, 0);
      if (i0 && !i1) touches++;
      else if (i0 || i1) return 0;
    }
    if (ii == 0) btouches = touches;
    else atouches = touches;
  }
  if (atouches > 0 || btouches > 0) return !(atouches == ansegs && btouches == bnsegs);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* predicate dispatch over geometry kinds (tg.c:5544-5760 intersects,       */
/* 5767-6046 covers, 6053-6556 contains, 6575-6789 touches,                 */
/* 15299-15330 equals / within / coveredby / disjoint)                       */
/* ------------------------------------------------------------------------ */

#define UNSUPPORTED (-1)

static inline const opoly_t* part_of(const spj_geoms* G, const ogeom_t* g, int i) {
  return &G->polys[g->first_poly + i];
}
static inline int is_polygonal(const ogeom_t* g) {
  return g->kind == SPJO_POLYGON || g->kind == SPJO_MULTIPOLYGON;
}

/* a (multi)polygon covers / contains / touches a point */
static int any_part_contains_point(const spj_geoms* G, const ogeom_t* g, opt_t p, int aoe) {
  for (int i = 0; i < g->npolys; i++)
    if (poly_contains_point(G, part_of(G, g, i), p, aoe)) return 1;
  return 0;
}

static int geom_intersects(const spj_geoms* GA, int64_t ia, const spj_geoms* GB, int64_t ib) {
  const ogeom_t* a = &GA->g[ia];
  const ogeom_t* b = &GB->g[ib];
  if (a->kind == SPJO_EMPTY || b->kind == SPJO_EMPTY) return 0;
  if (a->kind == SPJO_POINT && b->kind == SPJO_POINT) return pteq(a->pt, b->pt);
  if (a->kind == SPJO_POINT) return any_part_contains_point(GB, b, a->pt, 1);
  if (b->kind == SPJO_POINT) return any_part_contains_point(GA, a, b->pt, 1);
  /* any pair of parts, a's part first (poly_intersects_geom, multiiter) */
  for (int i = 0; i < a->npolys; i++)
    for (int j = 0; j < b->npolys; j++)
      if (poly_intersects_poly(GA, part_of(GA, a, i), GB, part_of(GB, b, j))) return 1;
  return 0;
}

static int geom_covers(const spj_geoms* GA, int64_t ia, const spj_geoms* GB, int64_t ib) {
  const ogeom_t* a = &GA->g[ia];
  const ogeom_t* b = &GB->g[ib];
  if (a->kind == SPJO_EMPTY || b->kind == SPJO_EMPTY) return 0;
  if (a->kind == SPJO_POINT && b->kind == SPJO_POINT) return pteq(a->pt, b->pt);
  if (a->kind == SPJO_POINT) {
    /* tg.c:1152-1155 per part (point_covers_base_geom: every part, and an
     * empty part fails) */
    if (b->empty_parts) return 0;
    for (int j = 0; j < b->npolys; j++) {
      const oring_t* e = poly_ext(GB, part_of(GB, b, j));
      if (ring_empty(e)) return 0;
      if (!(pteq(a->pt, (opt_t){e->rect.minx, e->rect.miny}) &&
            pteq(a->pt, (opt_t){e->rect.maxx, e->rect.maxy})))
        return 0;
    }
    return 1;
  }
  if (b->kind == SPJO_POINT) return any_part_contains_point(GA, a, b->pt, 1);
  if (a->kind == SPJO_POLYGON) {
    /* poly_covers_base_geom: every part of b, an empty part fails */
    if (b->empty_parts) return 0;
    for (int j = 0; j < b->npolys; j++)
      if (!poly_covers_poly(GA, part_of(GA, a, 0), GB, part_of(GB, b, j))) return 0;
    return 1;
  }
  /* a multipolygon: every non-empty part of b is covered by some part of a */
  for (int j = 0; j < b->npolys; j++) {
    int found = 0;
    for (int i = 0; i < a->npolys && !found; i++)
      found = poly_covers_poly(GA, part_of(GA, a, i), GB, part_of(GB, b, j));
    if (!found) return 0;
  }
  return 1;
}

static int geom_contains(const spj_geoms* GA, int64_t ia, const spj_geoms* GB, int64_t ib) {
  const ogeom_t* a = &GA->g[ia];
  const ogeom_t* b = &GB->g[ib];
  if (a->kind == SPJO_EMPTY || b->kind == SPJO_EMPTY) return 0;
  if (a->kind == SPJO_POINT && b->kind == SPJO_POINT) return pteq(a->pt, b->pt);
  if (a->kind == SPJO_POINT) return 0; /* tg.c:1157-1162 */
  if (b->kind == SPJO_POINT) {
    /* polygon: tg.c:3940-3943; multipolygon: tg.c:6288-6307, an interior
     * hit in any part wins */
    return any_part_contains_point(GA, a, b->pt, 0);
  }
  if (a->kind == SPJO_POLYGON) {
    /* poly_contains_base_geom: every part of b (tg_poly_contains_poly is
     * tg_poly_covers_poly), an empty part fails */
    if (b->empty_parts) return 0;
    for (int j = 0; j < b->npolys; j++)
      if (!poly_covers_poly(GA, part_of(GA, a, 0), GB, part_of(GB, b, j))) return 0;
    return 1;
  }
  /* a multipolygon (tg.c:6477-6487): a covers b, and some part of b meets
   * the interior of some part of a (intersects and does not touch) */
  if (!geom_covers(GA, ia, GB, ib)) return 0;
  for (int j = 0; j < b->npolys; j++)
    for (int i = 0; i < a->npolys; i++) {
      const opoly_t* pa = part_of(GA, a, i);
      const opoly_t* pb = part_of(GB, b, j);
      if (poly_intersects_poly(GA, pa, GB, pb) && !poly_touches_poly(GA, pa, GB, pb)) return 1;
    }
  return 0;
}

/* touches(one part of a, b) for a polygon part pa and b a point or
 * (multi)polygon (poly_touches_geom, tg.c:6679-6733) */
static int part_touches_geom(const spj_geoms* GA, const opoly_t* pa, const spj_geoms* GB,
                             const ogeom_t* b) {
  if (b->kind == SPJO_POINT) return poly_touches_point(GA, pa, b->pt);
  if (b->kind == SPJO_POLYGON) return poly_touches_poly(GA, pa, GB, part_of(GB, b, 0));
  int touches = 0;
  for (int j = 0; j < b->npolys; j++) {
    const opoly_t* pb = part_of(GB, b, j);
    if (poly_touches_poly(GA, pa, GB, pb)) touches = 1;
    else if (poly_intersects_poly(GA, pa, GB, pb)) return 0;
  }
  return touches;
}

static int part_intersects_geom(const spj_geoms* GA, const opoly_t* pa, const spj_geoms* GB,
                                const ogeom_t* b) {
  if (b->kind == SPJO_POINT) return poly_contains_point(GA, pa, b->pt, 1);
  for (int j = 0; j < b->npolys; j++)
    if (poly_intersects_poly(GA, pa, GB, part_of(GB, b, j))) return 1;
  return 0;
}

static int geom_touches(const spj_geoms* GA, int64_t ia, const spj_geoms* GB, int64_t ib) {
  const ogeom_t* a = &GA->g[ia];
  const ogeom_t* b = &GB->g[ib];
  if (a->kind == SPJO_EMPTY || b->kind == SPJO_EMPTY) return 0;
  if (a->kind == SPJO_POINT && b->kind == SPJO_POINT) return 0; /* tg.c:1102-1106 */
  if (a->kind == SPJO_POINT) {
    /* tg_point_touches_poly per part, any part (tg.c:6575-6625) */
    for (int j = 0; j < b->npolys; j++)
      if (poly_touches_point(GB, part_of(GB, b, j), a->pt)) return 1;
    return 0;
  }
  if (a->kind == SPJO_POLYGON) return part_touches_geom(GA, part_of(GA, a, 0), GB, b);
  /* a multipolygon (tg.c:6735-6768) */
  int touches = 0;
  for (int i = 0; i < a->npolys; i++) {
    const opoly_t* pa = part_of(GA, a, i);
    if (part_touches_geom(GA, pa, GB, b)) touches = 1;
    else if (part_intersects_geom(GA, pa, GB, b)) return 0;
  }
  return touches;
}


/* ------------------------------------------------------------------------ */
/* Euclidean distance of the reference's ST_DWithin refine,                  */
/* build.distance_ext(probe) <= d (rust/sedona-spatial-join/src/refine/      */
/* geo.rs:312-321), as sedona-geo-generic-alg computes it                    */
/* (rust/sedona-geo-generic-alg/src/algorithm/line_measures/metric_spaces/   */
/* euclidean/utils.rs, distance.rs).  The reference's intersects tests are   */
/* geo's; tg's stand in for them (they differ only where a distance is       */
/* within FP64 rounding of zero).                                            */
/* ------------------------------------------------------------------------ */

/* utils.rs:127-165 distance_coord_to_line_generic */
static double coord_line_dist(opt_t p, opt_t a, opt_t b) {
  if (a.x == b.x && a.y == b.y) return hypot(p.x - a.x, p.y - a.y);
  double dx = b.x - a.x, dy = b.y - a.y;
  double d2 = dx * dx + dy * dy;
  double r = ((p.x - a.x) * dx + (p.y - a.y) * dy) / d2;
  if (r <= 0) return hypot(p.x - a.x, p.y - a.y);
  if (r >= 1) return hypot(p.x - b.x, p.y - b.y);
  double s = ((a.y - p.y) * dx - (a.x - p.x) * dy) / d2;
  return fabs(s) * hypot(dx, dy);
}

/* utils.rs:291-314 distance_line_to_line_generic */
static double line_line_dist(oseg_t s1, oseg_t s2) {
  if (segment_intersects_segment(s1, s2)) return 0;
  double d1 = coord_line_dist(s1.a, s2.a, s2.b), d2 = coord_line_dist(s1.b, s2.a, s2.b);
  double d3 = coord_line_dist(s2.a, s1.a, s1.b), d4 = coord_line_dist(s2.b, s1.a, s1.b);
  return fmin(fmin(fmin(d1, d2), d3), d4);
}

/* distance.rs:486-505 LineString to LineString (and utils.rs:36-73
 * nearest_neighbour_distance, whose vertex passes cannot go below the
 * segment pairs' minimum): min over segment pairs, 0 at the first pair
 * that meets */
static double ring_ring_dist(const spj_geoms* G1, const oring_t* r1, const spj_geoms* G2,
                             const oring_t* r2) {
  double m = DBL_MAX;
  for (int i = 0; i < r1->nsegs; i++)
    for (int j = 0; j < r2->nsegs; j++) {
      double d = line_line_dist(ring_seg(G1, r1, i), ring_seg(G2, r2, j));
      if (d == 0) return 0;
      m = fmin(m, d);
    }
  return m == DBL_MAX ? 0 : m;
}

/* utils.rs:231-289 distance_point_to_polygon_generic */
static double point_poly_dist(const spj_geoms* G, const opoly_t* P, opt_t p) {
  if (poly_contains_point(G, P, p, 1)) return 0;
  double m = DBL_MAX;
  for (int h = 0; h < P->nrings; h++) {
    const oring_t* r = &G->rings[P->first_ring + h];
    for (int i = 0; i < r->nsegs; i++) {
      oseg_t s = ring_seg(G, r, i);
      m = fmin(m, coord_line_dist(p, s.a, s.b));
    }
  }
  return m;
}

/* utils.rs:567-657 distance_polygon_to_polygon_generic */
static double poly_poly_dist(const spj_geoms* GA, const opoly_t* A, const spj_geoms* GB,
                             const opoly_t* B) {
  if (poly_intersects_poly(GA, A, GB, B)) return 0;
  const oring_t* ea = poly_ext(GA, A);
  const oring_t* eb = poly_ext(GB, B);
  if (A->nrings == 1 && B->nrings == 1) return ring_ring_dist(GA, ea, GB, eb);
  /* b inside a (strictly inside a's shell at b's first point): the nearest
   * of a's holes; the same the other way round */
  if (A->nrings > 1 && ring_contains_point(GA, ea, GB->pts[eb->first], 0).hit) {
    double m = DBL_MAX;
    for (int h = 0; h < A->nrings - 1; h++)
      m = fmin(m, ring_ring_dist(GB, eb, GA, poly_hole(GA, A, h)));
    return m;
  }
  if (B->nrings > 1 && ring_contains_point(GB, eb, GA->pts[ea->first], 0).hit) {
    double m = DBL_MAX;
    for (int h = 0; h < B->nrings - 1; h++)
      m = fmin(m, ring_ring_dist(GA, ea, GB, poly_hole(GB, B, h)));
    return m;
  }
  return ring_ring_dist(GA, ea, GB, eb);
}

/* build.distance_ext(probe) over points, polygons and multipolygons: a
 * multipolygon is the minimum over its parts (distance.rs:224-246; an empty
 * part has distance 0, utils.rs:236-238) */
double spjo_geo_distance(const spj_geoms* GA, int64_t ia, const spj_geoms* GB, int64_t ib) {
  const ogeom_t* a = &GA->g[ia];
  const ogeom_t* b = &GB->g[ib];
  if (a->kind == SPJO_EMPTY || b->kind == SPJO_EMPTY) return 0;
  if (a->kind == SPJO_POINT && b->kind == SPJO_POINT)
    return hypot(a->pt.x - b->pt.x, a->pt.y - b->pt.y);
  if (a->empty_parts || b->empty_parts) return 0;
  double m = DBL_MAX;
  if (a->kind == SPJO_POINT || b->kind == SPJO_POINT) {
    const spj_geoms* GY = a->kind == SPJO_POINT ? GB : GA;
    const ogeom_t* y = a->kind == SPJO_POINT ? b : a;
    opt_t p = a->kind == SPJO_POINT ? a->pt : b->pt;
    for (int i = 0; i < y->npolys; i++) m = fmin(m, point_poly_dist(GY, part_of(GY, y, i), p));
    return m;
  }
  for (int i = 0; i < a->npolys; i++)
    for (int j = 0; j < b->npolys; j++)
      m = fmin(m, poly_poly_dist(GA, part_of(GA, a, i), GB, part_of(GB, b, j)));
  return m;
}

int spjo_predicate(const spj_geoms* B, int64_t bi, const spj_geoms* P, int64_t pi, int pred) {
  switch (pred) {
    case SPJO_INTERSECTS:
      return geom_intersects(B, bi, P, pi);
    case SPJO_DISJOINT:
      return !geom_intersects(B, bi, P, pi);
    case SPJO_CONTAINS:
      return geom_contains(B, bi, P, pi);
    case SPJO_WITHIN:
      return geom_contains(P, pi, B, bi);
    case SPJO_COVERS:
      return geom_covers(B, bi, P, pi);
    case SPJO_COVEREDBY:
      return geom_covers(P, pi, B, bi);
    case SPJO_TOUCHES:
      return geom_touches(B, bi, P, pi);
    case SPJO_EQUALS:
      return geom_contains(P, pi, B, bi) && geom_contains(B, bi, P, pi);
  }
  return UNSUPPORTED;
}

int spjo_raycast(double ax, double ay, double bx, double by, double px, double py) {
  oseg_t s = {{ax, ay}, {bx, by}};
  return raycast(s, (opt_t){px, py});
}
int spjo_segment_intersects(double ax, double ay, double bx, double by, double cx, double cy,
                            double dx, double dy) {
  oseg_t s1 = {{ax, ay}, {bx, by}}, s2 = {{cx, cy}, {dx, dy}};
  return segment_intersects_segment(s1, s2);
}
int spjo_collinear(double x1, double y1, double x2, double y2, double x3, double y3) {
  return collinear(x1, y1, x2, y2, x3, y3);
}

/* ------------------------------------------------------------------------ */
/* WKB parsing                                                               */
/* ------------------------------------------------------------------------ */

typedef struct {
  const uint8_t* p;
  int64_t len, pos;
  char* err;
  int errlen;
  int64_t row;
} wkb_reader;

static int rd_fail(wkb_reader* r, const char* what) {
  if (r->err) snprintf(r->err, r->errlen, "row %lld: invalid WKB (%s)", (long long)r->row, what);
  return -1;
}

static int rd_u8(wkb_reader* r, uint8_t* v) {
  if (r->pos + 1 > r->len) return rd_fail(r, "truncated");
  *v = r->p[r->pos++];
  return 0;
}
static int rd_u32(wkb_reader* r, int le, uint32_t* v) {
  if (r->pos + 4 > r->len) return rd_fail(r, "truncated");
  const uint8_t* b = r->p + r->pos;
  *v = le ? ((uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) |
             ((uint32_t)b[3] << 24))
          : ((uint32_t)b[3] | ((uint32_t)b[2] << 8) | ((uint32_t)b[1] << 16) |
             ((uint32_t)b[0] << 24));
  r->pos += 4;
  return 0;
}
static int rd_f64(wkb_reader* r, int le, double* v) {
  if (r->pos + 8 > r->len) return rd_fail(r, "truncated");
  uint64_t u = 0;
  const uint8_t* b = r->p + r->pos;
  for (int i = 0; i < 8; i++) u |= (uint64_t)b[le ? i : 7 - i] << (8 * i);
  memcpy(v, &u, 8);
  r->pos += 8;
  return 0;
}

static int grow(void** p, int64_t* cap, int64_t need, size_t elt) {
  if (need <= *cap) return 0;
  int64_t nc = *cap ? *cap : 1024;
  while (nc < need) nc *= 2;
  void* q = realloc(*p, (size_t)nc * elt);
  if (!q) return -1;
  *p = q;
  *cap = nc;
  return 0;
}

static void rect_extend(orect_t* r, opt_t p) {
  if (p.x < r->minx) r->minx = p.x;
  if (p.y < r->miny) r->miny = p.y;
  if (p.x > r->maxx) r->maxx = p.x;
  if (p.y > r->maxy) r->maxy = p.y;
}
static orect_t rect_empty(void) {
  orect_t r = {INFINITY, INFINITY, -INFINITY, -INFINITY};
  return r;
}

/* header: byte order + geometry type; only 2D geometries are accepted. */
static int rd_header(wkb_reader* r, int* le, uint32_t* type) {
  uint8_t bo;
  if (rd_u8(r, &bo)) return -1;
  if (bo > 1) return rd_fail(r, "byte order");
  *le = bo;
  uint32_t t;
  if (rd_u32(r, *le, &t)) return -1;
  if (t & 0xE0000000u) return rd_fail(r, "EWKB flags are not supported");
  if (t >= 1000) return rd_fail(r, "only 2D geometries are supported");
  *type = t;
  return 0;
}

/* tg.c:1910-2113 process_points: a ring is concave when some vertex turn has
 * the sign opposite to the first turn's (a first turn of exactly zero counts
 * as positive), clockwise when the shoelace sum of (b.x - a.x) * (b.y + a.y)
 * is positive.  The turns and the sum run over the points as stored (the
 * closing point included), wrapping to the first points at the end. */
static void ring_flags(const opt_t* p, int n, int* convex, int* clockwise) {
  if (n < 2) {
    *convex = 0;
    *clockwise = 0;
    return;
  }
  int concave = 0, dir = 0;
  double cwc = 0;
  for (int i = 0; i < n; i++) {
    opt_t a = p[i], b, c;
    if (i < n - 2) {
      b = p[i + 1];
      c = p[i + 2];
    } else if (i == n - 1) {
      b = p[0];
      c = p[1];
    } else {
      b = p[i + 1];
      c = p[0];
    }
    cwc += (b.x - a.x) * (b.y + a.y);
    if (!concave) {
      double z = (b.x - a.x) * (c.y - b.y) - (b.y - a.y) * (c.x - b.x);
      if (dir == 0) {
        dir = z < 0 ? -1 : 1;
      } else if (z < 0) {
        if (dir == 1) concave = 1;
      } else if (z > 0) {
        if (dir == -1) concave = 1;
      }
    }
  }
  *convex = !concave;
  *clockwise = cwc > 0;
}

static int rd_polygon_body(spj_geoms* G, wkb_reader* r, int le, orect_t* grect) {
  uint32_t nrings;
  if (rd_u32(r, le, &nrings)) return -1;
  if ((int64_t)nrings * 4 > r->len - r->pos) return rd_fail(r, "ring count");
  if (grow((void**)&G->polys, &G->cap_polys, G->npolys + 1, sizeof(opoly_t))) return -1;
  opoly_t* P = &G->polys[G->npolys++];
  P->first_ring = G->nrings;
  P->nrings = (int32_t)nrings;
  if (grow((void**)&G->rings, &G->cap_rings, G->nrings + nrings, sizeof(oring_t))) return -1;
  for (uint32_t k = 0; k < nrings; k++) {
    uint32_t npts;
    if (rd_u32(r, le, &npts)) return -1;
    if ((int64_t)npts * 16 > r->len - r->pos) return rd_fail(r, "point count");
    if (grow((void**)&G->pts, &G->cap_pts, G->npts + npts + 1, sizeof(opt_t))) return -1;
    oring_t* R = &G->rings[G->nrings++];
    R->npts = (int32_t)npts;
    R->first = G->npts;
    R->rect = rect_empty();
    for (uint32_t i = 0; i < npts; i++) {
      opt_t q;
      if (rd_f64(r, le, &q.x) || rd_f64(r, le, &q.y)) return -1;
      G->pts[G->npts + i] = q;
      rect_extend(&R->rect, q);
      rect_extend(grect, q);
    }
    G->nvert += npts;
    /* tg.c:2124-2134 num_segments for closed series */
    if (npts < 3) R->nsegs = 0;
    else if (pteq(G->pts[G->npts + npts - 1], G->pts[G->npts])) R->nsegs = (int32_t)npts - 1;
    else R->nsegs = (int32_t)npts;
    ring_flags(&G->pts[G->npts], (int)npts, &R->convex, &R->clockwise);
    /* tg.c:2220 the extra closing point */
    G->pts[G->npts + npts] = npts ? G->pts[G->npts] : (opt_t){0, 0};
    G->npts += npts + 1;
  }
  return 0;
}

static int parse_one(spj_geoms* G, int64_t row, const uint8_t* p, int64_t len, char* err,
                     int errlen) {
  wkb_reader r = {p, len, 0, err, errlen, row};
  ogeom_t* g = &G->g[row];
  g->kind = SPJO_EMPTY;
  g->rect = rect_empty();
  int le;
  uint32_t type;
  if (rd_header(&r, &le, &type)) return -1;
  if (type == 1) {
    opt_t q;
    if (rd_f64(&r, le, &q.x) || rd_f64(&r, le, &q.y)) return -1;
    if (isnan(q.x) && isnan(q.y)) return 0; /* POINT EMPTY */
    g->kind = SPJO_POINT;
    g->pt = q;
    rect_extend(&g->rect, q);
    G->nvert += 1;
    return 0;
  }
  if (type == 3) {
    int64_t before = G->npolys;
    if (rd_polygon_body(G, &r, le, &g->rect)) return -1;
    if (G->polys[before].nrings == 0) {
      G->npolys = before; /* POLYGON EMPTY */
      return 0;
    }
    g->kind = SPJO_POLYGON;
    g->first_poly = before;
    g->npolys = 1;
    return 0;
  }
  if (type == 6) {
    uint32_t n;
    if (rd_u32(&r, le, &n)) return -1;
    int64_t before = G->npolys;
    int32_t kept = 0;
    for (uint32_t i = 0; i < n; i++) {
      int le2;
      uint32_t t2;
      if (rd_header(&r, &le2, &t2)) return -1;
      if (t2 != 3) return rd_fail(&r, "multipolygon part is not a polygon");
      int64_t pb = G->npolys;
      if (rd_polygon_body(G, &r, le2, &g->rect)) return -1;
      if (G->polys[pb].nrings == 0) {
        G->npolys = pb; /* empty part */
        g->empty_parts = 1;
        continue;
      }
      kept++;
    }
    if (kept == 0) {
      g->empty_parts = 0;
      return 0;
    }
    g->kind = SPJO_MULTIPOLYGON;
    g->first_poly = before;
    g->npolys = kept;
    return 0;
  }
  return rd_fail(&r, "unsupported geometry type");
}

spj_geoms* spjo_parse(const int64_t* offsets, const uint8_t* data, const uint8_t* validity,
                      int64_t n, char* err, int errlen) {
  spj_geoms* G = (spj_geoms*)calloc(1, sizeof(spj_geoms));
  if (!G) return NULL;
  G->n = n;
  G->g = (ogeom_t*)calloc((size_t)(n > 0 ? n : 1), sizeof(ogeom_t));
  if (!G->g) {
    free(G);
    return NULL;
  }
  for (int64_t i = 0; i < n; i++) {
    int valid = validity ? (validity[i >> 3] >> (i & 7)) & 1 : 1;
    G->g[i].kind = SPJO_EMPTY;
    G->g[i].rect = rect_empty();
    if (!valid) continue;
    int64_t len = offsets[i + 1] - offsets[i];
    if (parse_one(G, i, data + offsets[i], len, err, errlen)) {
      spjo_free_geoms(G);
      return NULL;
    }
  }
  return G;
}

void spjo_free_geoms(spj_geoms* G) {
  if (!G) return;
  free(G->g);
  free(G->polys);
  free(G->rings);
  free(G->pts);
  free(G);
}
int64_t spjo_count(const spj_geoms* G) { return G->n; }
int spjo_kind(const spj_geoms* G, int64_t i) { return G->g[i].kind; }
int64_t spjo_num_vertices(const spj_geoms* G) { return G->nvert; }
int spjo_point(const spj_geoms* G, int64_t i, double* x, double* y) {
  if (G->g[i].kind != SPJO_POINT) return 0;
  *x = G->g[i].pt.x;
  *y = G->g[i].pt.y;
  return 1;
}

/* ------------------------------------------------------------------------ */
/* f32 boxes                                                                 */
/* ------------------------------------------------------------------------ */

/* rust/sedona-spatial-join/src/utils/bounds.rs:147-162 */
static void f64_interval_to_f32(double lo, double hi, float* flo, float* fhi) {
  float a = (float)lo, b = (float)hi;
  if ((double)a > lo) a = nextafterf(a, -INFINITY);
  if ((double)b < hi) b = nextafterf(b, INFINITY);
  *flo = a;
  *fhi = b;
}

static void box_of(const ogeom_t* g, int mode, double expand, float* o) {
  if (g->kind == SPJO_EMPTY) {
    o[0] = o[1] = o[2] = o[3] = NAN;
    return;
  }
  if (mode == 1 && g->kind == SPJO_POINT && expand == 0) {
    /* join_provider.rs:128-132: round to nearest, degenerate box */
    o[0] = o[2] = (float)g->pt.x;
    o[1] = o[3] = (float)g->pt.y;
    return;
  }
  /* operand_evaluator.rs:605-607 expand in f64, then outward */
  f64_interval_to_f32(g->rect.minx - expand, g->rect.maxx + expand, &o[0], &o[2]);
  f64_interval_to_f32(g->rect.miny - expand, g->rect.maxy + expand, &o[1], &o[3]);
}

void spjo_boxes(const spj_geoms* G, int mode, float* out) {
  for (int64_t i = 0; i < G->n; i++) box_of(&G->g[i], mode, 0, out + 4 * i);
}

/* ------------------------------------------------------------------------ */
/* uniform grid over f32 build boxes                                         */
/* ------------------------------------------------------------------------ */

typedef struct {
  double x0, y0, inv;
  int gx, gy;
  int64_t* cell_off; /* gx*gy + 1 */
  uint32_t* ids;
} ogrid_t;

static inline int box_is_empty(const float* b) {
  return isnan(b[0]) || isnan(b[1]) || isnan(b[2]) || isnan(b[3]) || b[0] > b[2] ||
         b[1] > b[3];
}

static inline int cell_x(const ogrid_t* g, double x) {
  double c = floor((x - g->x0) * g->inv);
  if (!(c >= 0)) return 0;
  if (c >= g->gx) return g->gx - 1;
  return (int)c;
}
static inline int cell_y(const ogrid_t* g, double y) {
  double c = floor((y - g->y0) * g->inv);
  if (!(c >= 0)) return 0;
  if (c >= g->gy) return g->gy - 1;
  return (int)c;
}

static int grid_build(ogrid_t* g, const float* boxes, int64_t n) {
  memset(g, 0, sizeof(*g));
  double minx = INFINITY, miny = INFINITY, maxx = -INFINITY, maxy = -INFINITY, wsum = 0;
  int64_t cnt = 0;
  for (int64_t i = 0; i < n; i++) {
    const float* b = boxes + 4 * i;
    if (box_is_empty(b)) continue;
    if (b[0] < minx) minx = b[0];
    if (b[1] < miny) miny = b[1];
    if (b[2] > maxx) maxx = b[2];
    if (b[3] > maxy) maxy = b[3];
    wsum += (double)(b[2] - b[0]) + (double)(b[3] - b[1]);
    cnt++;
  }
  if (cnt == 0) {
    g->gx = g->gy = 1;
    g->x0 = g->y0 = 0;
    g->inv = 1;
  } else {
    double w = maxx - minx, h = maxy - miny;
    double ext = w > h ? w : h;
    if (!(ext > 0)) ext = 1;
    double cs = ext / sqrt((double)cnt) * 1.5;
    double avg = wsum / (2.0 * cnt);
    if (avg > cs) cs = avg;
    if (cs < ext / 4096) cs = ext / 4096;
    g->x0 = minx;
    g->y0 = miny;
    g->inv = 1.0 / cs;
    g->gx = (int)(w / cs) + 1;
    g->gy = (int)(h / cs) + 1;
  }
  int64_t nc = (int64_t)g->gx * g->gy;
  g->cell_off = (int64_t*)calloc((size_t)nc + 1, sizeof(int64_t));
  if (!g->cell_off) return -1;
  for (int64_t i = 0; i < n; i++) {
    const float* b = boxes + 4 * i;
    if (box_is_empty(b)) continue;
    int x0 = cell_x(g, b[0]), x1 = cell_x(g, b[2]), y0 = cell_y(g, b[1]), y1 = cell_y(g, b[3]);
    for (int y = y0; y <= y1; y++)
      for (int x = x0; x <= x1; x++) g->cell_off[(int64_t)y * g->gx + x + 1]++;
  }
  for (int64_t c = 0; c < nc; c++) g->cell_off[c + 1] += g->cell_off[c];
  g->ids = (uint32_t*)malloc((size_t)(g->cell_off[nc] > 0 ? g->cell_off[nc] : 1) * 4);
  int64_t* fill = (int64_t*)malloc((size_t)nc * sizeof(int64_t));
  if (!g->ids || !fill) return -1;
  memcpy(fill, g->cell_off, (size_t)nc * sizeof(int64_t));
  for (int64_t i = 0; i < n; i++) {
    const float* b = boxes + 4 * i;
    if (box_is_empty(b)) continue;
    int x0 = cell_x(g, b[0]), x1 = cell_x(g, b[2]), y0 = cell_y(g, b[1]), y1 = cell_y(g, b[3]);
    for (int y = y0; y <= y1; y++)
      for (int x = x0; x <= x1; x++) g->ids[fill[(int64_t)y * g->gx + x]++] = (uint32_t)i;
  }
  free(fill);
  return 0;
}

static void grid_free(ogrid_t* g) {
  free(g->cell_off);
  free(g->ids);
}

/* visit every build id whose box intersects pb (closed), exactly once */
typedef int (*visit_fn)(void* ctx, uint32_t build);
static int grid_query(const ogrid_t* g, const float* boxes, const float* pb, visit_fn fn,
                      void* ctx) {
  if (box_is_empty(pb)) return 0;
  int x0 = cell_x(g, pb[0]), x1 = cell_x(g, pb[2]), y0 = cell_y(g, pb[1]), y1 = cell_y(g, pb[3]);
  for (int y = y0; y <= y1; y++) {
    for (int x = x0; x <= x1; x++) {
      int64_t c = (int64_t)y * g->gx + x;
      for (int64_t k = g->cell_off[c]; k < g->cell_off[c + 1]; k++) {
        uint32_t id = g->ids[k];
        const float* b = boxes + 4 * (int64_t)id;
        if (b[0] > pb[2] || b[2] < pb[0] || b[1] > pb[3] || b[3] < pb[1]) continue;
        /* report in the cell holding the intersection's lower-left corner */
        float lx = b[0] > pb[0] ? b[0] : pb[0];
        float ly = b[1] > pb[1] ? b[1] : pb[1];
        if (cell_x(g, lx) != x || cell_y(g, ly) != y) continue;
        if (fn(ctx, id)) return -1;
      }
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* threaded join driver                                                      */
/* ------------------------------------------------------------------------ */

typedef struct {
  uint32_t* b;
  uint32_t* p;
  int64_t n, cap;
} pairvec;

static int pv_push(pairvec* v, uint32_t b, uint32_t p) {
  if (v->n == v->cap) {
    int64_t nc = v->cap ? v->cap * 2 : 4096;
    uint32_t* nb = (uint32_t*)realloc(v->b, (size_t)nc * 4);
    if (!nb) return -1;
    v->b = nb;
    uint32_t* np = (uint32_t*)realloc(v->p, (size_t)nc * 4);
    if (!np) return -1;
    v->p = np;
    v->cap = nc;
  }
  v->b[v->n] = b;
  v->p[v->n] = p;
  v->n++;
  return 0;
}

static int cmp_u32(const void* a, const void* b) {
  uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? -1 : x > y;
}

typedef struct {
  /* inputs */
  const spj_geoms *B, *P;
  const float* bboxes;
  const float* pboxes; /* may be NULL: computed per probe */
  const ogrid_t* grid;
  int pred;
  double distance;
  const double* dists; /* per probe row (NULL: distance for every row) */
  int64_t p0, p1;
  /* per-probe scratch */
  uint32_t* cand;
  int64_t ncand, capcand;
  uint32_t cur_probe;
  /* outputs */
  pairvec out;
  int status;
  char err[256];
} jobctx;

static int collect(void* vctx, uint32_t build) {
  jobctx* c = (jobctx*)vctx;
  if (c->ncand == c->capcand) {
    int64_t nc = c->capcand ? c->capcand * 2 : 256;
    uint32_t* q = (uint32_t*)realloc(c->cand, (size_t)nc * 4);
    if (!q) return -1;
    c->cand = q;
    c->capcand = nc;
  }
  c->cand[c->ncand++] = build;
  return 0;
}

static void* join_worker(void* arg) {
  jobctx* c = (jobctx*)arg;
  for (int64_t pi = c->p0; pi < c->p1; pi++) {
    float pb[4];
    if (c->pboxes) memcpy(pb, c->pboxes + 4 * pi, sizeof pb);
    else box_of(&c->P->g[pi], 0,
                c->pred == SPJO_DWITHIN ? (c->dists ? c->dists[pi] : c->distance) : 0, pb);
    c->ncand = 0;
    if (grid_query(c->grid, c->bboxes, pb, collect, c)) {
      c->status = -1;
      snprintf(c->err, sizeof c->err, "out of memory");
      return NULL;
    }
    if (c->ncand > 1) qsort(c->cand, (size_t)c->ncand, 4, cmp_u32);
    for (int64_t k = 0; k < c->ncand; k++) {
      uint32_t bi = c->cand[k];
      int keep;
      if (!c->B) {
        keep = 1; /* rect join */
      } else if (c->pred == SPJO_DWITHIN) {
        /* geo.rs:312-321 build.distance_ext(probe) <= d */
        const double dd = c->dists ? c->dists[pi] : c->distance;
        keep = spjo_geo_distance(c->B, bi, c->P, pi) <= dd;
      } else {
        keep = spjo_predicate(c->B, bi, c->P, pi, c->pred);
        if (keep < 0) {
          c->status = -1;
          snprintf(c->err, sizeof c->err,
                   "predicate %d is not supported for geometry kinds %d/%d", c->pred,
                   c->B->g[bi].kind, c->P->g[pi].kind);
          return NULL;
        }
      }
      if (keep && pv_push(&c->out, bi, (uint32_t)pi)) {
        c->status = -1;
        snprintf(c->err, sizeof c->err, "out of memory");
        return NULL;
      }
    }
  }
  return NULL;
}

static int64_t run_join(const spj_geoms* B, const spj_geoms* P, const float* bboxes, int64_t nb,
                        const float* pboxes, int64_t np, int pred, double distance,
                        const double* dists, int nthreads, uint32_t** ob, uint32_t** op,
                        char* err, int errlen) {
  ogrid_t grid;
  if (grid_build(&grid, bboxes, nb)) {
    grid_free(&grid);
    if (err) snprintf(err, errlen, "out of memory");
    return -1;
  }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if (np < (int64_t)nthreads * 16) nthreads = np > 16 ? (int)(np / 16) : 1;
  jobctx* jobs = (jobctx*)calloc((size_t)nthreads, sizeof(jobctx));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  int64_t chunk = (np + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    jobs[t].B = B;
    jobs[t].P = P;
    jobs[t].bboxes = bboxes;
    jobs[t].pboxes = pboxes;
    jobs[t].grid = &grid;
    jobs[t].pred = pred;
    jobs[t].distance = distance;
    jobs[t].dists = dists;
    jobs[t].p0 = t * chunk < np ? t * chunk : np;
    jobs[t].p1 = (t + 1) * chunk < np ? (t + 1) * chunk : np;
  }
  if (nthreads == 1) {
    join_worker(&jobs[0]);
  } else {
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, join_worker, &jobs[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  }
  int64_t total = 0;
  int status = 0;
  for (int t = 0; t < nthreads; t++) {
    total += jobs[t].out.n;
    if (jobs[t].status && !status) {
      status = -1;
      if (err) snprintf(err, errlen, "%s", jobs[t].err);
    }
  }
  uint32_t* rb = NULL;
  uint32_t* rp = NULL;
  if (!status) {
    rb = (uint32_t*)malloc((size_t)(total > 0 ? total : 1) * 4);
    rp = (uint32_t*)malloc((size_t)(total > 0 ? total : 1) * 4);
    int64_t pos = 0;
    for (int t = 0; t < nthreads; t++) {
      memcpy(rb + pos, jobs[t].out.b, (size_t)jobs[t].out.n * 4);
      memcpy(rp + pos, jobs[t].out.p, (size_t)jobs[t].out.n * 4);
      pos += jobs[t].out.n;
    }
  }
  for (int t = 0; t < nthreads; t++) {
    free(jobs[t].out.b);
    free(jobs[t].out.p);
    free(jobs[t].cand);
  }
  free(jobs);
  free(th);
  grid_free(&grid);
  if (status) return -1;
  *ob = rb;
  *op = rp;
  return total;
}

int64_t spjo_rect_join(const float* build_rects, int64_t nb, const float* probe_rects,
                       int64_t np, int nthreads, uint32_t** out_build, uint32_t** out_probe) {
  return run_join(NULL, NULL, build_rects, nb, probe_rects, np, SPJO_INTERSECTS, 0, NULL, nthreads,
                  out_build, out_probe, NULL, 0);
}

int64_t spjo_join(const spj_geoms* B, const spj_geoms* P, int pred, double distance,
                  int nthreads, uint32_t** out_build, uint32_t** out_probe, char* err,
                  int errlen) {
  float* bb = (float*)malloc((size_t)(B->n > 0 ? B->n : 1) * 16);
  if (!bb) return -1;
  spjo_boxes(B, 0, bb);
  int64_t r = run_join(B, P, bb, B->n, NULL, P->n, pred, distance, NULL, nthreads, out_build,
                       out_probe, err, errlen);
  free(bb);
  return r;
}

int64_t spjo_join_dists(const spj_geoms* B, const spj_geoms* P, const double* dists,
                        int nthreads, uint32_t** out_build, uint32_t** out_probe, char* err,
                        int errlen) {
  float* bb = (float*)malloc((size_t)(B->n > 0 ? B->n : 1) * 16);
  if (!bb) return -1;
  spjo_boxes(B, 0, bb);
  int64_t r = run_join(B, P, bb, B->n, NULL, P->n, SPJO_DWITHIN, 0, dists, nthreads, out_build,
                       out_probe, err, errlen);
  free(bb);
  return r;
}

/* ------------------------------------------------------------------------ */
/* KNN                                                                       */
/* ------------------------------------------------------------------------ */

typedef struct {
  const spj_geoms *B, *P;
  const float* bboxes;
  const ogrid_t* grid;
  int k;
  int64_t p0, p1;
  uint32_t* ob;
  double* od;
} knnctx;

/* (dist, id) strictly better: total order on distances, then build id */
static inline int knn_better(double d1, uint32_t i1, double d2, uint32_t i2) {
  return d1 < d2 || (d1 == d2 && i1 < i2);
}

static void* knn_worker(void* arg) {
  knnctx* c = (knnctx*)arg;
  const ogrid_t* g = c->grid;
  int k = c->k;
  double* bd = (double*)malloc((size_t)k * sizeof(double));
  uint32_t* bi = (uint32_t*)malloc((size_t)k * 4);
  for (int64_t pi = c->p0; pi < c->p1; pi++) {
    uint32_t* ob = c->ob + pi * k;
    double* od = c->od + pi * k;
    for (int j = 0; j < k; j++) {
      ob[j] = 0xFFFFFFFFu;
      od[j] = INFINITY;
    }
    const ogeom_t* gp = &c->P->g[pi];
    if (gp->kind != SPJO_POINT) continue;
    double px = gp->pt.x, py = gp->pt.y;
    int have = 0;
    int cx = cell_x(g, px), cy = cell_y(g, py);
    for (int ring = 0;; ring++) {
      int x0 = cx - ring, x1 = cx + ring, y0 = cy - ring, y1 = cy + ring;
      for (int y = y0; y <= y1; y++) {
        if (y < 0 || y >= g->gy) continue;
        for (int x = x0; x <= x1; x++) {
          if (x < 0 || x >= g->gx) continue;
          if (y != y0 && y != y1 && x != x0 && x != x1) continue; /* ring cells only */
          int64_t cc = (int64_t)y * g->gx + x;
          for (int64_t q = g->cell_off[cc]; q < g->cell_off[cc + 1]; q++) {
            uint32_t id = g->ids[q];
            const ogeom_t* gb = &c->B->g[id];
            double d = hypot(px - gb->pt.x, py - gb->pt.y);
            if (have == k && !knn_better(d, id, bd[k - 1], bi[k - 1])) continue;
            /* a point whose outward box straddles a cell edge is listed in
               every cell it touches: keep one entry per build row */
            int dup = 0;
            for (int t = 0; t < have && !dup; t++) dup = bi[t] == id;
            if (dup) continue;
            int j = have < k ? have++ : k - 1;
            while (j > 0 && knn_better(d, id, bd[j - 1], bi[j - 1])) {
              bd[j] = bd[j - 1];
              bi[j] = bi[j - 1];
              j--;
            }
            bd[j] = d;
            bi[j] = id;
          }
        }
      }
      int covers_all = x0 <= 0 && y0 <= 0 && x1 >= g->gx - 1 && y1 >= g->gy - 1;
      if (covers_all) break;
      if (have == k) {
        /* distance from p to the outside of the visited square */
        double lx = g->x0 + (double)x0 / g->inv, hx = g->x0 + (double)(x1 + 1) / g->inv;
        double ly = g->y0 + (double)y0 / g->inv, hy = g->y0 + (double)(y1 + 1) / g->inv;
        double m = px - lx;
        if (hx - px < m) m = hx - px;
        if (py - ly < m) m = py - ly;
        if (hy - py < m) m = hy - py;
        /* margin absorbs rounding in the cell-edge arithmetic */
        if (bd[k - 1] < m * (1 - 1e-9) - 1e-9 * fabs(px) - 1e-9 * fabs(py)) break;
      }
    }
    for (int j = 0; j < have; j++) {
      ob[j] = bi[j];
      od[j] = bd[j];
    }
  }
  free(bd);
  free(bi);
  return NULL;
}

int spjo_knn(const spj_geoms* B, const spj_geoms* P, int k, int nthreads, uint32_t* out_build,
             double* out_dist, char* err, int errlen) {
  if (k <= 0) {
    if (err) snprintf(err, errlen, "k must be positive");
    return -1;
  }
  for (int64_t i = 0; i < B->n; i++) {
    if (B->g[i].kind != SPJO_POINT && B->g[i].kind != SPJO_EMPTY) {
      if (err) snprintf(err, errlen, "KNN build side must be points");
      return -1;
    }
  }
  float* bb = (float*)malloc((size_t)(B->n > 0 ? B->n : 1) * 16);
  spjo_boxes(B, 0, bb);
  ogrid_t grid;
  if (grid_build(&grid, bb, B->n)) {
    free(bb);
    if (err) snprintf(err, errlen, "out of memory");
    return -1;
  }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  int64_t np = P->n;
  if (np < (int64_t)nthreads * 16) nthreads = np > 16 ? (int)(np / 16) : 1;
  knnctx* jobs = (knnctx*)calloc((size_t)nthreads, sizeof(knnctx));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  int64_t chunk = (np + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    jobs[t] = (knnctx){B, P, bb, &grid, k, 0, 0, out_build, out_dist};
    jobs[t].p0 = t * chunk < np ? t * chunk : np;
    jobs[t].p1 = (t + 1) * chunk < np ? (t + 1) * chunk : np;
  }
  if (nthreads == 1) knn_worker(&jobs[0]);
  else {
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, knn_worker, &jobs[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  }
  free(jobs);
  free(th);
  grid_free(&grid);
  free(bb);
  return 0;
}

/* ------------------------------------------------------------------------ */

static inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

uint64_t spjo_digest(const uint32_t* b, const uint32_t* p, int64_t n) {
  uint64_t s = 0;
  for (int64_t i = 0; i < n; i++) s += splitmix64(((uint64_t)p[i] << 32) | b[i]);
  return s;
}

void spjo_free(void* p) { free(p); }
