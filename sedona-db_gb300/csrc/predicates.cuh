// predicates.cuh — device restatement of the reference refiner's predicate
// arithmetic (the tg library, c/sedona-tg/src/tg/tg.c, which the reference
// CPU join calls as tg_geom_<pred>(build, probe),
// rust/sedona-spatial-join/src/refine/tg.rs:322-357).
//
// Two tiers per segment test:
//   * an FP32 classifier on round-to-nearest copies of the coordinates that
//     only decides a segment when a strict FP32 comparison proves the FP64
//     comparison tg makes (round-to-nearest is monotone, so RN(a) < RN(b)
//     implies a < b); everything else escalates;
//   * the FP64 path, which repeats tg's operation sequence exactly (including
//     its division-based slope test and nextafter nudges), so escalated
//     decisions are the reference's decisions bit for bit.
// The library is compiled with --fmad=false so no multiply-add is fused.
#pragma once
#include "geoms.cuh"

namespace spj {
namespace pred {
namespace {  // internal linkage: included by several translation units

enum { kOut = 0, kIn = 1, kOn = 2 };

__device__ __forceinline__ bool feq(double x, double y) { return !((x < y) | (x > y)); }
__device__ __forceinline__ bool eq_zero(double x) { return feq(x, 0.0); }
__device__ __forceinline__ double fmin0(double x, double y) { return x < y ? x : y; }
__device__ __forceinline__ double fmax0(double x, double y) { return x > y ? x : y; }
__device__ __forceinline__ float fmin0f(float x, float y) { return x < y ? x : y; }
__device__ __forceinline__ float fmax0f(float x, float y) { return x > y ? x : y; }
__device__ __forceinline__ bool pteq(double2 a, double2 b) { return feq(a.x, b.x) && feq(a.y, b.y); }

// tg.c:861-900
__device__ __noinline__ bool collinear(double x1, double y1, double x2, double y2, double x3,
                                       double y3) {
  const bool x1x2 = feq(x1, x2), x1x3 = feq(x1, x3), x2x3 = feq(x2, x3);
  const bool y1y2 = feq(y1, y2), y1y3 = feq(y1, y3), y2y3 = feq(y2, y3);
  if (x1x2) return x1x3;
  if (y1y2) return y1y3;
  if ((x1x2 & y1y2) | (x1x3 & y1y3) | (x2x3 & y2y3)) return true;
  const double cx1 = __dsub_rn(x3, x1), cy1 = __dsub_rn(y3, y1);
  const double cx2 = __dsub_rn(x2, x1), cy2 = __dsub_rn(y2, y1);
  double s1 = __dmul_rn(cx1, cy2);
  double s2 = __dmul_rn(cy1, cx2);
  const double s3 = __dsub_rn(__ddiv_rn(s1, cy2), cx1);
  const double s4 = __dsub_rn(__ddiv_rn(s2, cx2), cy1);
  if (s3 < 0) s1 = next_down(s1);
  else if (s3 > 0) s1 = next_up(s1);
  if (s4 < 0) s2 = next_down(s2);
  else if (s4 > 0) s2 = next_up(s2);
  return eq_zero(__dsub_rn(s1, s2));
}

// tg.c:1192-1197 with tg_rect_covers_point (tg.c:1776-1785)
__device__ __forceinline__ bool point_on_segment(double2 p, double2 a, double2 b) {
  const double mnx = fmin0(a.x, b.x), mny = fmin0(a.y, b.y);
  const double mxx = fmax0(a.x, b.x), mxy = fmax0(a.y, b.y);
  if (p.x < mnx || p.y < mny || p.x > mxx || p.y > mxy) return false;
  return collinear(a.x, a.y, b.x, b.y, p.x, p.y);
}

// tg.c:1199-1276: +x ray from p against segment (sa, sb)
__device__ __noinline__ int raycast(double2 sa, double2 sb, double2 p) {
  const double rminx = fmin0(sa.x, sb.x), rminy = fmin0(sa.y, sb.y);
  const double rmaxx = fmax0(sa.x, sb.x), rmaxy = fmax0(sa.y, sb.y);
  if (p.y < rminy || p.y > rmaxy) return kOut;
  if (p.x < rminx) {
    if (p.y != rminy && p.y != rmaxy) return kIn;
  } else if (p.x > rmaxx) {
    if (rminy != rmaxy && rminx != rmaxx) return kOut;
  }
  double2 a = sa, b = sb;
  if (b.y < a.y) {
    double2 t = a;
    a = b;
    b = t;
  }
  if (pteq(p, a) || pteq(p, b)) return kOn;
  if (a.y == b.y) {
    if (a.x == b.x) return kOut;
    if (p.y == b.y) {
      if (!(p.x < rminx || p.x > rmaxx)) return kOn;
    }
  }
  if (a.x == b.x && p.x == b.x) {
    if (p.y >= a.y && p.y <= b.y) return kOn;
  }
  if (collinear(a.x, a.y, b.x, b.y, p.x, p.y)) {
    if (p.x < rminx) {
      if (rminy == rmaxy) return kOut;
    } else if (p.x > rmaxx) {
      return kOut;
    }
    return kOn;
  }
  double py = p.y;
  if (py == a.y || py == b.y) py = next_up(py);
  if (py < a.y || py > b.y) return kOut;
  if (a.x > b.x) {
    if (p.x >= a.x) return kOut;
    if (p.x <= b.x) return kIn;
  } else {
    if (p.x >= b.x) return kOut;
    if (p.x <= a.x) return kIn;
  }
  const double lhs = __ddiv_rn(__dsub_rn(py, a.y), __dsub_rn(p.x, a.x));
  const double rhs = __ddiv_rn(__dsub_rn(b.y, a.y), __dsub_rn(b.x, a.x));
  return lhs >= rhs ? kIn : kOut;
}

// tg.c:1392-1440
__device__ __noinline__ bool seg_intersects_seg(double2 a, double2 b, double2 c, double2 d) {
  {
    const double aminx = fmin0(a.x, b.x), aminy = fmin0(a.y, b.y);
    const double amaxx = fmax0(a.x, b.x), amaxy = fmax0(a.y, b.y);
    const double bminx = fmin0(c.x, d.x), bminy = fmin0(c.y, d.y);
    const double bmaxx = fmax0(c.x, d.x), bmaxy = fmax0(c.y, d.y);
    if (bminx > amaxx || bmaxx < aminx || bminy > amaxy || bmaxy < aminy) return false;
  }
  if (pteq(a, c) || pteq(a, d) || pteq(b, c) || pteq(b, d)) return true;
  const double cmpx = __dsub_rn(c.x, a.x), cmpy = __dsub_rn(c.y, a.y);
  const double rx = __dsub_rn(b.x, a.x), ry = __dsub_rn(b.y, a.y);
  const double cmpxr = __dsub_rn(__dmul_rn(cmpx, ry), __dmul_rn(cmpy, rx));
  if (eq_zero(cmpxr)) {
    if (!(((__dsub_rn(c.x, a.x) <= 0) != (__dsub_rn(c.x, b.x) <= 0))) ||
        ((__dsub_rn(c.y, a.y) <= 0) != (__dsub_rn(c.y, b.y) <= 0))) {
      return point_on_segment(c, a, b) || point_on_segment(d, a, b) ||
             point_on_segment(a, c, d) || point_on_segment(b, c, d);
    }
    return true;
  }
  const double sx = __dsub_rn(d.x, c.x), sy = __dsub_rn(d.y, c.y);
  const double rxs = __dsub_rn(__dmul_rn(rx, sy), __dmul_rn(ry, sx));
  if (eq_zero(rxs)) return false;
  const double cmpxs = __dsub_rn(__dmul_rn(cmpx, sy), __dmul_rn(cmpy, sx));
  const double rxsr = __ddiv_rn(1.0, rxs);
  const double t = __dmul_rn(cmpxs, rxsr);
  const double u = __dmul_rn(cmpxr, rxsr);
  if (!((t >= 0) && (t <= 1) && (u >= 0) && (u <= 1))) return false;
  return true;
}

// ---------------------------------------------------------------------------
// per-ring point evaluation (tg.c:2668-2735, 2809-2822)

struct RingHit {
  bool hit;
  int idx;
};

// One segment's contribution, FP64 (tg pip_eval_seg + pip_eval_seg_slow).
__device__ __forceinline__ void pip_seg_f64(double2 a, double2 b, double2 p, int i, bool aoe,
                                            bool& in, int& idx) {
  const double ymin = fmin0(a.y, b.y), ymax = fmax0(a.y, b.y);
  if (p.y < ymin || p.y > ymax) return;
  switch (raycast(a, b, p)) {
    case kIn:
      if (idx == -1) in = !in;
      break;
    case kOn:
      // tg keeps the last ON segment of its visit in index order; the
      // largest index is that segment whatever order the caller visits in
      in = aoe;
      if (i > idx) idx = i;
      break;
    default:
      break;
  }
}

// Sign of the exact orientation (b - a) x (p - a) of three FP64 points known
// through their round-to-nearest f32 copies a, b, p: +1 / -1 when the f32
// evaluation clears twice a static bound E on its error, else 0.
// E covers the coordinate rounding (|c - RN32(c)| <= 2^-24 |RN32(c)|, doubled,
// plus 2^-150 absolute for the subnormal range), the rounding of the two
// differences, the two products and the final difference.  A decided sign
// therefore leaves |exact| >= E, some 2^28 times the FP64 rounding of tg's
// own orientation / slope / intersection arithmetic on the same points, so
// tg's FP64 decisions follow the exact sign.
__device__ __forceinline__ int orient32(float2 a, float2 b, float2 p) {
  const float dx = __fsub_rn(b.x, a.x), dy = __fsub_rn(b.y, a.y);
  const float ex = __fsub_rn(p.x, a.x), ey = __fsub_rn(p.y, a.y);
  const float t1 = __fmul_rn(dx, ey), t2 = __fmul_rn(dy, ex);
  const float o = __fsub_rn(t1, t2);
  const float u = 5.9604645e-08f;   // 2^-24
  const float c2 = 1.1920929e-07f;  // 2^-23
  const float tiny = 1.4012985e-45f;
  const float Edx = __fadd_ru(__fmul_ru(c2, __fadd_ru(fabsf(b.x), fabsf(a.x))),
                              __fadd_ru(__fmul_ru(u, fabsf(dx)), tiny));
  const float Edy = __fadd_ru(__fmul_ru(c2, __fadd_ru(fabsf(b.y), fabsf(a.y))),
                              __fadd_ru(__fmul_ru(u, fabsf(dy)), tiny));
  const float Eex = __fadd_ru(__fmul_ru(c2, __fadd_ru(fabsf(p.x), fabsf(a.x))),
                              __fadd_ru(__fmul_ru(u, fabsf(ex)), tiny));
  const float Eey = __fadd_ru(__fmul_ru(c2, __fadd_ru(fabsf(p.y), fabsf(a.y))),
                              __fadd_ru(__fmul_ru(u, fabsf(ey)), tiny));
  const float E1 = __fadd_ru(__fadd_ru(__fmul_ru(fabsf(dx), Eey), __fmul_ru(fabsf(ey), Edx)),
                             __fadd_ru(__fmul_ru(Edx, Eey), __fmul_ru(u, fabsf(t1))));
  const float E2 = __fadd_ru(__fadd_ru(__fmul_ru(fabsf(dy), Eex), __fmul_ru(fabsf(ex), Edy)),
                             __fadd_ru(__fmul_ru(Edy, Eex), __fmul_ru(u, fabsf(t2))));
  const float E = __fmul_ru(__fadd_ru(__fadd_ru(E1, E2), __fadd_ru(__fmul_ru(u, fabsf(o)), tiny)),
                            2.0000019f);  // x2 margin, x(1 + 2^-20) slack
  if (o > E) return 1;
  if (o < -E) return -1;
  return 0;  // undecided (also for NaN / inf)
}

// FP32 classification of one segment: returns kOut / kIn when it provably
// equals tg's FP64 ray-cast result, or -1.  Strict comparisons of
// round-to-nearest values prove tg's early exits; a point strictly inside
// the segment's y-range gets tg's slope-test answer, which for such a point
// is the side of p relative to the upward segment (IN when p is left of it),
// from orient32 when that sign is decided.
__device__ __forceinline__ int pip_seg_f32(float2 a, float2 b, float2 p) {
  const float ymin = fmin0f(a.y, b.y), ymax = fmax0f(a.y, b.y);
  if (p.y < ymin || p.y > ymax) return kOut;
  const float xmin = fmin0f(a.x, b.x), xmax = fmax0f(a.x, b.x);
  const bool inner_y = p.y > ymin && p.y < ymax;
  if (p.x < xmin && inner_y) return kIn;
  if (p.x > xmax && ymin < ymax && xmin < xmax) return kOut;
  if (inner_y) {
    const bool up = a.y < b.y;
    const int o = orient32(up ? a : b, up ? b : a, p);
    if (o > 0) return kIn;
    if (o < 0) return kOut;
  }
  return -1;
}

__device__ __forceinline__ bool rect_covers_point(Rect64 r, double2 p) {
  return !(p.x < r.x || p.y < r.y || p.x > r.z || p.y > r.w);
}

// tg_rect_covers_point(ring rect, p), decided on the RN32 copies when a strict
// comparison settles it (strictly outside, or strictly inside), else in FP64.
__device__ __forceinline__ bool ring_rect_covers(const GeomsView& G, uint32_t r, double2 p,
                                                 float2 p32) {
  const float4 q = G.ring_rect32[r];
  if (p32.x < q.x || p32.y < q.y || p32.x > q.z || p32.y > q.w) return false;
  if (p32.x > q.x && p32.y > q.y && p32.x < q.z && p32.y < q.w) return true;
  return rect_covers_point(G.ring_rect[r], p);
}

__device__ __forceinline__ int band_of(float y32, float y0, float inv_h, int nb) {
  float t = __fmul_rn(__fsub_rn(y32, y0), inv_h);
  if (!(t >= 0.0f)) return 0;
  float f = floorf(t);
  if (f >= (float)(nb - 1)) return nb - 1;
  return (int)f;
}

// --- cell grid lookups -------------------------------------------------------
// Boundary k of a grid axis: origin + k * step in f32 arithmetic (the same
// expression the grid builder used, so cells tile the axis exactly).
__device__ __forceinline__ float grid_edge(float o, float step, int k) {
  return __fadd_rn(o, __fmul_rn((float)k, step));
}

// v32 strictly inside (a, b).
__device__ __forceinline__ bool p_inside_open(float v32, float a, float b) {
  return v32 > a && v32 < b;
}

// Index of a closed cell [edge(i), edge(i+1)] containing the FP64 coordinate
// v, or -1 when v lies outside the grid.  The f32 estimate is corrected
// against the exact boundary values.
__device__ __forceinline__ int grid_index(float o, float step, int n, double v) {
  if (!(v >= (double)grid_edge(o, step, 0)) || !(v <= (double)grid_edge(o, step, n))) return -1;
  int i = (int)floorf(__fdiv_rn(__fsub_rn(__double2float_rn(v), o), step));
  i = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
  while (i > 0 && v < (double)grid_edge(o, step, i)) i--;
  while (i < n - 1 && v > (double)grid_edge(o, step, i + 1)) i++;
  return i;
}

// The same index from v's round-to-nearest copy v32, in FP32 alone when that
// settles it.  A strict f32 comparison of RN values proves the exact one
// (RN is monotone), so v32 strictly between two edges puts v strictly inside
// that cell, and v32 strictly outside the first / last edge puts v outside
// the grid.  Only a v32 equal to an edge (v within half an f32 ulp of it)
// takes the FP64 lookup.
__device__ __forceinline__ int grid_index32(float o, float step, int n, float v32, double v) {
  const float e0 = grid_edge(o, step, 0), en = grid_edge(o, step, n);
  if (p_inside_open(v32, e0, en)) {
    int i = (int)floorf(__fdiv_rn(__fsub_rn(v32, o), step));
    i = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
    while (i > 0 && v32 < grid_edge(o, step, i)) i--;
    while (i < n - 1 && v32 > grid_edge(o, step, i + 1)) i++;
    if (v32 > grid_edge(o, step, i) && v32 < grid_edge(o, step, i + 1)) return i;
  } else if (v32 < e0 || v32 > en || v32 != v32) {
    return -1;
  }
  return grid_index(o, step, n, v);
}

// Status of the grid cell holding p (0 mixed / no grid, 1 inside, 2 outside).
// A clean cell is touched by no edge, so every point of it has the ring's
// status there, on tg's arithmetic as well (the argument of the isolation
// exit in ring_intersects_ring).  p32 is p rounded to nearest.
__device__ __forceinline__ int grid_point_status(const GeomsView& G, uint32_t r, double2 p,
                                                 float2 p32) {
  if (G.grid_meta == nullptr) return 0;
  const uint2 m = G.grid_meta[r];
  if (m.y == 0) return 0;
  const float4 q = G.grid_rect[r];
  const int i = grid_index32(q.x, q.z, (int)m.y, p32.x, p.x);
  if (i < 0) return 0;
  const int j = grid_index32(q.y, q.w, (int)m.y, p32.y, p.y);
  if (j < 0) return 0;
  return G.grid_status[m.x + (uint32_t)j * m.y + (uint32_t)i];
}

// Status shared by every grid cell that holds the closed box of another ring
// (its exact rect R, RN32 rect q): 1 inside / 2 outside when those cells (at
// most 2 x 2) are all clean with that status, else 0.  Clean cells are free
// of the ring's edges (each edge strictly bbox-separated from the cell, or
// the cell strictly on one side of its line), so no edge of this ring meets
// the box (their union is a rectangle that holds it), tg's segment tests
// against anything inside fail, and every point of the box has that status
// in tg's arithmetic (the argument of the isolation exit below).
__device__ __forceinline__ int grid_rect_status(const GeomsView& G, uint32_t r, Rect64 R,
                                                float4 q) {
  if (!G.grid_rings || G.grid_meta == nullptr) return 0;
  const uint2 m = G.grid_meta[r];
  if (m.y == 0) return 0;
  const float4 g = G.grid_rect[r];
  const int i0 = grid_index32(g.x, g.z, (int)m.y, q.x, R.x);
  const int i1 = grid_index32(g.x, g.z, (int)m.y, q.z, R.z);
  if (i0 < 0 || i1 < 0 || i1 - i0 > 1) return 0;
  const int j0 = grid_index32(g.y, g.w, (int)m.y, q.y, R.y);
  const int j1 = grid_index32(g.y, g.w, (int)m.y, q.w, R.w);
  if (j0 < 0 || j1 < 0 || j1 - j0 > 1) return 0;
  const uint8_t* st = G.grid_status + m.x;
  const int s = st[(uint32_t)j0 * m.y + (uint32_t)i0];
  if (s == 0) return 0;
  for (int j = j0; j <= j1; j++)
    for (int i = i0; i <= i1; i++)
      if (st[(uint32_t)j * m.y + (uint32_t)i] != s) return 0;
  return s;
}

// Plain FP64 form: tg's FP64 sequence for every segment it visits, with the
// same index as the chosen form and no FP32 arithmetic tier.  With a band
// index the visited segments are the point's band (every segment whose
// y-range holds p.y is listed there), in the band's order, up to the first
// entry whose key (its RN32 xmax) is strictly left of the point's RN32 x:
// every later entry is strictly left of p, where tg's ray cast gives OUT.
// Without one, all segments in index order.
__device__ __forceinline__ RingHit ring_pip_plain(const GeomsView& G, uint32_t r, double2 p,
                                                  float2 p32, bool aoe) {
  RingHit h{false, -1};
  if (!rect_covers_point(G.ring_rect[r], p)) return h;
  const uint32_t V = G.ring_vtx[r];
  const int ns = G.ring_nsegs[r];
  bool in = false;
  int idx = -1;
  if (G.ring_bands != nullptr && G.band_param[r].y >= 0.0f) {
    const uint32_t B = G.ring_bands[r];
    const int nb = (int)(G.ring_bands[r + 1] - B) - 1;
    const float2 prm = G.band_param[r];
    const int b = band_of(p32.y, prm.x, prm.y, nb);
    const uint32_t e0 = G.band_off[B + b], e1 = G.band_off[B + b + 1];
    for (uint32_t k = e0; k < e1; k++) {
      const float4 sg = G.band_seg[k];
      if (fmax0f(sg.x, sg.z) < p32.x) break;
      const int i = G.band_edges[k];
      pip_seg_f64(G.xy[V + i], G.xy[V + i + 1], p, i, aoe, in, idx);
    }
    h.hit = in;
    h.idx = idx;
    return h;
  }
  double2 a = G.xy[V];
  for (int i = 0; i < ns; i++) {
    const double2 b = G.xy[V + i + 1];
    pip_seg_f64(a, b, p, i, aoe, in, idx);
    a = b;
  }
  h.hit = in;
  h.idx = idx;
  return h;
}

// Chosen form: y-band edge index + FP32 classification + FP64 escalation.
// Without a band index on this column the ring's segments are all scanned
// (still with the FP32 classifier).  The answer does not depend on the
// order of the visits: any ON segment makes it allow_on_edge, else it is the
// parity of the IN segments (tg.c:2668-2735).  idx is tg's: the largest ON
// segment index (tg visits in index order and keeps the last).
__device__ __forceinline__ RingHit ring_pip_fast(const GeomsView& G, uint32_t r, double2 p,
                                                 float2 p32, bool aoe, uint32_t& esc,
                                                 bool use_grid = true) {
  RingHit h{false, -1};
  if (!ring_rect_covers(G, r, p, p32)) return h;
  if (use_grid) {
    const int st = grid_point_status(G, r, p, p32);
    if (st != 0) {  // clean cell: not on any edge, status known
      h.hit = st == 1;
      return h;
    }
  }
  const uint32_t V = G.ring_vtx[r];
  bool in = false;
  int idx = -1;
  bool banded = G.ring_bands != nullptr && G.band_param[r].y >= 0.0f;
  if (banded) {
    const uint32_t B = G.ring_bands[r];
    const int nb = (int)(G.ring_bands[r + 1] - B) - 1;
    const float2 prm = G.band_param[r];
    const int b = band_of(p32.y, prm.x, prm.y, nb);
    const uint32_t e0 = G.band_off[B + b], e1 = G.band_off[B + b + 1];
    for (uint32_t k = e0; k < e1; k++) {
      const float4 sg = G.band_seg[k];
      // entries run by xmax descending: from here on every segment lies
      // strictly left of p, and tg's +x ray cast gives OUT for each
      if (fmax0f(sg.x, sg.z) < p32.x) break;
      const int c = pip_seg_f32(make_float2(sg.x, sg.y), make_float2(sg.z, sg.w), p32);
      if (c == kOut) continue;
      if (c == kIn) {
        if (idx == -1) in = !in;
        continue;
      }
      esc++;
      const int i = G.band_edges[k];
      pip_seg_f64(G.xy[V + i], G.xy[V + i + 1], p, i, aoe, in, idx);
    }
  } else {
    const int ns = G.ring_nsegs[r];
    float2 a32 = G.xy32[V];
    for (int i = 0; i < ns; i++) {
      const float2 b32 = G.xy32[V + i + 1];
      const int c = pip_seg_f32(a32, b32, p32);
      a32 = b32;
      if (c == kOut) continue;
      if (c == kIn) {
        if (idx == -1) in = !in;
        continue;
      }
      esc++;
      pip_seg_f64(G.xy[V + i], G.xy[V + i + 1], p, i, aoe, in, idx);
    }
  }
  h.hit = in;
  h.idx = idx;
  return h;
}

// use_grid = false skips the cell-grid lookup (for points known to lie near
// the ring's edges, where the cell is mixed)
template <bool kFast>
__device__ __forceinline__ RingHit ring_pip(const GeomsView& G, uint32_t r, double2 p, float2 p32,
                                            bool aoe, uint32_t& esc, bool use_grid = true) {
  if (kFast) return ring_pip_fast(G, r, p, p32, aoe, esc, use_grid);
  return ring_pip_plain(G, r, p, p32, aoe);
}

__device__ __forceinline__ uint32_t ring_npts(const GeomsView& G, uint32_t r) {
  return G.ring_vtx[r + 1] - G.ring_vtx[r] - 1;
}

// tg.c:3909-3934 (a polygon without holes is a tg ring, tg.c:3785-3789)
template <bool kFast>
__device__ __forceinline__ bool poly_contains_point(const GeomsView& G, uint32_t part, double2 p,
                                                    float2 p32, bool aoe, uint32_t& esc) {
  const uint32_t r0 = G.part_ring[part], r1 = G.part_ring[part + 1];
  if (r1 - r0 == 1) return ring_pip<kFast>(G, r0, p, p32, aoe, esc).hit;
  if (ring_npts(G, r0) < 3) return false;  // tg_poly_empty
  if (!ring_pip<kFast>(G, r0, p, p32, aoe, esc).hit) return false;
  for (uint32_t h = r0 + 1; h < r1; h++)
    if (ring_pip<kFast>(G, h, p, p32, !aoe, esc).hit) return false;
  return true;
}

// tg.c:1171-1190 + tg.c:3436-3443: p lies on a segment of any ring
template <bool kFast>
__device__ __forceinline__ bool poly_touches_point(const GeomsView& G, uint32_t part, double2 p,
                                                   float2 p32, uint32_t& esc) {
  const uint32_t r0 = G.part_ring[part], r1 = G.part_ring[part + 1];
  for (uint32_t r = r0; r < r1; r++) {
    const uint32_t V = G.ring_vtx[r];
    const int ns = G.ring_nsegs[r];
    for (int i = 0; i < ns; i++) {
      if (kFast) {
        // point_on_segment starts with a rect cover test; strict FP32
        // separation proves it fails
        const float2 a = G.xy32[V + i], b = G.xy32[V + i + 1];
        if (p32.x < fmin0f(a.x, b.x) || p32.x > fmax0f(a.x, b.x) || p32.y < fmin0f(a.y, b.y) ||
            p32.y > fmax0f(a.y, b.y))
          continue;
        esc++;
      }
      if (point_on_segment(p, G.xy[V + i], G.xy[V + i + 1])) return true;
    }
  }
  return false;
}

// Number of segments of ring r intersecting segment (a, b), stopping at 2
// (tg.c:3046-3087 with allow_on_edge; tg_ring_search filter tg.c:2468-2485).
template <bool kFast>
__device__ __forceinline__ int ring_seg_hits(const GeomsView& G, uint32_t r, double2 a, double2 b,
                                             float2 a32, float2 b32, uint32_t& esc) {
  const uint32_t V = G.ring_vtx[r];
  int count = 0;
  const float qx0 = fmin0f(a32.x, b32.x), qx1 = fmax0f(a32.x, b32.x);
  const float qy0 = fmin0f(a32.y, b32.y), qy1 = fmax0f(a32.y, b32.y);
  if (!kFast) {
    // plain form: the same band index, every visited segment in FP64
    if (G.ring_bands != nullptr && G.band_param[r].y >= 0.0f) {
      const uint32_t B = G.ring_bands[r];
      const int nb = (int)(G.ring_bands[r + 1] - B) - 1;
      const float2 prm = G.band_param[r];
      const int b0 = band_of(qy0, prm.x, prm.y, nb), b1 = band_of(qy1, prm.x, prm.y, nb);
      for (int bb = b0; bb <= b1 && count < 2; bb++) {
        const uint32_t e0 = G.band_off[B + bb], e1 = G.band_off[B + bb + 1];
        for (uint32_t k = e0; k < e1 && count < 2; k++) {
          const float4 sg = G.band_seg[k];
          if (fmax0f(sg.x, sg.z) < qx0) break;  // index key: the rest is left
          if (bb > b0 && band_of(fmin0f(sg.y, sg.w), prm.x, prm.y, nb) < bb) continue;
          const int i = G.band_edges[k];
          if (seg_intersects_seg(a, b, G.xy[V + i], G.xy[V + i + 1])) count++;
        }
      }
      return count;
    }
    const int ns = G.ring_nsegs[r];
    for (int i = 0; i < ns && count < 2; i++)
      if (seg_intersects_seg(a, b, G.xy[V + i], G.xy[V + i + 1])) count++;
    return count;
  }
  // segment (c, d) of the ring; its index (needed only by the FP64 tier)
  // is band entry k's edge when banded, else k itself
  auto test = [&](const float2 c, const float2 d, const uint32_t k, const bool banded_k) {
    if (fmin0f(c.x, d.x) > qx1 || fmax0f(c.x, d.x) < qx0 || fmin0f(c.y, d.y) > qy1 ||
        fmax0f(c.y, d.y) < qy0)
      return;  // strictly separated rects: tg's first test fails
    // Decided orientations: c, d strictly on one side of line ab (or a, b of
    // line cd) means tg's parameter u (or t) = o1 / (o1 - o2) lies outside
    // [0, 1] by far more than its FP64 rounding -> no intersection; strictly
    // opposite sides on both lines means t, u are inside (0, 1) -> crossing.
    const int o1 = orient32(a32, b32, c), o2 = orient32(a32, b32, d);
    if (o1 != 0 && o1 == o2) return;
    const int o3 = orient32(c, d, a32), o4 = orient32(c, d, b32);
    if (o3 != 0 && o3 == o4) return;
    if (o1 != 0 && o2 != 0 && o3 != 0 && o4 != 0) {
      count++;
      return;
    }
    esc++;
    const int i = banded_k ? (int)G.band_edges[k] : (int)k;
    if (seg_intersects_seg(a, b, G.xy[V + i], G.xy[V + i + 1])) count++;
  };
  const bool banded = G.ring_bands != nullptr && G.band_param[r].y >= 0.0f;
  if (banded) {
    const uint32_t B = G.ring_bands[r];
    const int nb = (int)(G.ring_bands[r + 1] - B) - 1;
    const float2 prm = G.band_param[r];
    const int b0 = band_of(qy0, prm.x, prm.y, nb), b1 = band_of(qy1, prm.x, prm.y, nb);
    for (int bb = b0; bb <= b1 && count < 2; bb++) {
      const uint32_t e0 = G.band_off[B + bb], e1 = G.band_off[B + bb + 1];
      for (uint32_t k = e0; k < e1 && count < 2; k++) {
        const float4 sg = G.band_seg[k];
        const float2 c = make_float2(sg.x, sg.y), d = make_float2(sg.z, sg.w);
        // xmax descending: the rest of the band is strictly left of the query
        if (fmax0f(c.x, d.x) < qx0) break;
        // visit each segment once: only in the first band of the query it spans
        if (bb > b0 && band_of(fmin0f(c.y, d.y), prm.x, prm.y, nb) < bb) continue;
        test(c, d, k, true);
      }
    }
  } else {
    const int ns = G.ring_nsegs[r];
    for (int i = 0; i < ns && count < 2; i++)
      test(G.xy32[V + i], G.xy32[V + i + 1], (uint32_t)i, false);
  }
  return count;
}

__device__ __forceinline__ double rect_area(Rect64 r) {
  return __dmul_rn(__dsub_rn(r.z, r.x), __dsub_rn(r.w, r.y));
}

// Interval [lo, hi] containing the exact area of a rect known only through
// its RN32 corners (each exact coordinate is within one f32 ulp of its RN).
__device__ __forceinline__ void rect_area_bounds(float4 q, float& lo, float& hi) {
  const float wl = fmaxf(__fsub_rd(next_downf(q.z), next_upf(q.x)), 0.0f);
  const float wh = __fsub_ru(next_upf(q.z), next_downf(q.x));
  const float hl = fmaxf(__fsub_rd(next_downf(q.w), next_upf(q.y)), 0.0f);
  const float hh = __fsub_ru(next_upf(q.w), next_downf(q.y));
  lo = __fmul_rd(wl, hl);
  hi = __fmul_ru(wh, hh);
}

// tg swaps the rings when rect_area(other) > rect_area(ring) in FP64
// (tg.c:3176-3183).  Decided from f32 area bounds when they are separated by
// far more than FP64 rounding can move the two products; else in FP64.
template <bool kFast>
__device__ __forceinline__ bool swap_rings(const GeomsView& GA, uint32_t ra, const GeomsView& GB,
                                           uint32_t rb) {
  if (kFast) {
    float a_lo, a_hi, b_lo, b_hi;
    rect_area_bounds(GA.ring_rect32[ra], a_lo, a_hi);
    rect_area_bounds(GB.ring_rect32[rb], b_lo, b_hi);
    if (b_lo > __fmul_ru(a_hi, 1.0000010f)) return true;
    if (__fmul_ru(b_hi, 1.0000010f) < a_lo) return false;
  }
  return rect_area(GB.ring_rect[rb]) > rect_area(GA.ring_rect[ra]);
}

// tg_rect_intersects_rect of two ring rects, f32 first when strict.
template <bool kFast>
__device__ __forceinline__ bool ring_rects_intersect(const GeomsView& GA, uint32_t ra,
                                                     const GeomsView& GB, uint32_t rb) {
  if (kFast) {
    const float4 a = GA.ring_rect32[ra], b = GB.ring_rect32[rb];
    if (b.x > a.z || b.z < a.x || b.y > a.w || b.w < a.y) return false;
    if (b.x < a.z && b.z > a.x && b.y < a.w && b.w > a.y) return true;
  }
  const Rect64 A = GA.ring_rect[ra], Bq = GB.ring_rect[rb];
  return !(Bq.x > A.z || Bq.z < A.x || Bq.y > A.w || Bq.w < A.y);
}

// Isolation test of ring ro of Go against ring rr of Gr, in the FP32 form,
// with rr's y-band index.  If every segment of rr has a bbox strictly
// separated from ro's bbox (a strict f32 comparison of round-to-nearest
// values proves the f64 one), or has that whole box strictly on one side of
// its line (all four corners, decided orientations), then
//  - no segment test between rr and ro can succeed (tg's first test is the
//    bbox test, and a segment that misses the box misses every segment in
//    it), and
//  - for every point v of ro's box, each ray-cast decision is one of tg's
//    comparison-only exits or the exact side test, i.e. the exact half-open
//    crossing rule; no segment crosses the box, so that parity is the same
//    for every point of ro: ro lies strictly inside rr or strictly outside.
// Returns 1 / 0 in that case (the point-in-ring answer of ro's first vertex,
// which every point of ro shares), kIsoNear when a segment of rr comes near
// the box, kIsoNoIndex when rr has no band index (or ro no segments).
constexpr int kIsoNear = -4, kIsoNoIndex = -5;
template <bool kFast>
__device__ __forceinline__ int ring_isolation(const GeomsView& Gr, uint32_t rr,
                                              const GeomsView& Go, uint32_t ro, uint32_t& esc) {
  if (!kFast || Go.ring_nsegs[ro] <= 0 || Gr.ring_bands == nullptr ||
      !(Gr.band_param[rr].y >= 0.0f))
    return kIsoNoIndex;
  const float4 ob = Go.ring_rect32[ro];
  const float bx0 = ob.x, by0 = ob.y, bx1 = ob.z, by1 = ob.w;
  const uint32_t B = Gr.ring_bands[rr];
  const int nb = (int)(Gr.ring_bands[rr + 1] - B) - 1;
  const float2 prm = Gr.band_param[rr];
  const int b0 = band_of(by0, prm.x, prm.y, nb), b1 = band_of(by1, prm.x, prm.y, nb);
  // The first vertex's point-in-ring test rides along: its band is one of
  // b0..b1, so the same scan classifies that band's edges for it (the FP32
  // tier of ring_pip_fast).  When the box is isolated and every one of those
  // edges was decided, the parity is ring_pip's answer; otherwise ring_pip
  // runs as before.
  const uint32_t Vo = Go.ring_vtx[ro];
  const double2 v0 = Go.xy[Vo];
  const float2 v032 = Go.xy32[Vo];
  const bool v_in_rect = ring_rect_covers(Gr, rr, v0, v032);
  const int bv = band_of(v032.y, prm.x, prm.y, nb);
  bool v_decided = true;
  unsigned v_par = 0;
  bool near = false;
  for (int bb = b0; bb <= b1 && !near; bb++) {
    const uint32_t e0 = Gr.band_off[B + bb], e1 = Gr.band_off[B + bb + 1];
    const bool vband = v_in_rect && bb == bv;
    for (uint32_t k = e0; k < e1; k++) {
      const float4 sg = Gr.band_seg[k];
      const float2 c = make_float2(sg.x, sg.y), d = make_float2(sg.z, sg.w);
      // xmax descending: the rest of the band is strictly left of the box
      // (bbox-separated) and of its first vertex (tg's ray cast: OUT)
      if (fmax0f(c.x, d.x) < bx0) break;
      if (vband) {
        const int pc = pip_seg_f32(c, d, v032);
        if (pc == kIn) v_par ^= 1u;
        else if (pc != kOut) v_decided = false;
      }
      if (fmax0f(c.x, d.x) < bx0 || fmin0f(c.x, d.x) > bx1 || fmax0f(c.y, d.y) < by0 ||
          fmin0f(c.y, d.y) > by1)
        continue;  // bboxes strictly separated
      const int s0 = orient32(c, d, make_float2(bx0, by0));
      if (s0 != 0 && orient32(c, d, make_float2(bx1, by0)) == s0 &&
          orient32(c, d, make_float2(bx1, by1)) == s0 &&
          orient32(c, d, make_float2(bx0, by1)) == s0)
        continue;
      near = true;
      break;
    }
  }
  if (near) return kIsoNear;
  if (!v_in_rect) return 0;  // ring_pip's first test
  if (v_decided) return v_par != 0;
  return ring_pip<kFast>(Gr, rr, v0, v032, true, esc).hit ? 1 : 0;
}

// tg.c:3166-3192 + tg.c:3089-3113 with allow_on_edge = true, for two rings.
// The result is the OR over the smaller ring's vertices of "vertex in or on
// the larger ring" and over its segments of "crosses >= 2 of the larger
// ring's segments"; tg's per-segment rect test only skips terms that are
// false, so the vertex tests run first and the result is the same.
//
// kCheap (FP32 form with a band index) stops early: a pair that the
// isolation exit does not decide, and whose first vertex is not in the larger
// ring, returns kDeferred instead of running the vertex and segment loops.
// Returns 1 / 0 (or kDeferred).
constexpr int kDeferred = -2;

template <bool kFast, bool kCheap = false>
__device__ __forceinline__ int ring_intersects_ring(const GeomsView& GA, uint32_t ra,
                                                    const GeomsView& GB, uint32_t rb,
                                                    uint32_t& esc) {
  if (ring_npts(GA, ra) < 3 || ring_npts(GB, rb) < 3) return 0;
  if (!ring_rects_intersect<kFast>(GA, ra, GB, rb)) return 0;
  const GeomsView* Gr = &GA;
  const GeomsView* Go = &GB;
  uint32_t rr = ra, ro = rb;
  if (swap_rings<kFast>(GA, ra, GB, rb)) {
    Gr = &GB;
    Go = &GA;
    rr = rb;
    ro = ra;
  }
  const uint32_t Vo = Go->ring_vtx[ro];
  const int nso = Go->ring_nsegs[ro];
  if (kFast && nso > 0) {
    // the smaller ring's box inside clean cells of the larger ring: no edge
    // of the larger ring comes near, so the answer is the cells' status
    const int st = grid_rect_status(*Gr, rr, Go->ring_rect[ro], Go->ring_rect32[ro]);
    if (st != 0) return st == 1 ? 1 : 0;
  }
  {
    const int iso = ring_isolation<kFast>(*Gr, rr, *Go, ro, esc);
    if (iso >= 0) return iso;
    if (kCheap && iso == kIsoNear) {
      // the vertex loop below starts with this test
      if (ring_pip<kFast>(*Gr, rr, Go->xy[Vo], Go->xy32[Vo], true, esc, false).hit) return 1;
      return kDeferred;
    }
  }
  // (the vertices of a ring that came near the larger ring's edges: the grid
  // cells around them are mostly mixed, so they skip the lookup)
  for (int i = 0; i <= nso; i++) {
    const double2 v = Go->xy[Vo + i];
    const float2 v32 = Go->xy32[Vo + i];
    if (ring_pip<kFast>(*Gr, rr, v, v32, true, esc, false).hit) return 1;
  }
  const float4 R32 = Gr->ring_rect32[rr];
  for (int i = 0; i < nso; i++) {
    const double2 a = Go->xy[Vo + i], b = Go->xy[Vo + i + 1];
    const float2 a32 = Go->xy32[Vo + i], b32 = Go->xy32[Vo + i + 1];
    // tg.c:3092-3094 segment rect vs ring rect: a separated segment has no
    // hits anyway, so only the strict f32 separation is used to skip it
    if (kFast && (fmin0f(a32.x, b32.x) > R32.z || fmax0f(a32.x, b32.x) < R32.x ||
                  fmin0f(a32.y, b32.y) > R32.w || fmax0f(a32.y, b32.y) < R32.y))
      continue;
    if (!kFast) {
      const Rect64 R = Gr->ring_rect[rr];
      if (fmin0(a.x, b.x) > R.z || fmax0(a.x, b.x) < R.x || fmin0(a.y, b.y) > R.w ||
          fmax0(a.y, b.y) < R.y)
        continue;
    }
    if (ring_seg_hits<kFast>(*Gr, rr, a, b, a32, b32, esc) >= 2) return 1;
  }
  return 0;
}

}  // namespace
}  // namespace pred
}  // namespace spj
