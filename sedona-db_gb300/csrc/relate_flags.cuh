// relate_flags.cuh — tg's per-ring convex / clockwise flags, which select the
// algorithm of tg's ring-in-ring and segment-in-ring tests
// (c/sedona-tg/src/tg/tg.c:2910-3039, 3120-3156).
#pragma once
#include "common.cuh"

namespace spj {

enum RingFlag : uint8_t { kRingConvex = 1, kRingClockwise = 2, kRingFlagsSet = 0x80 };

// tg.c:1910-2113 process_points over the ring's points as stored (npts of
// them, the closing point included): the ring is concave when some vertex
// turn (b - a) x (c - b) has the sign opposite to the first turn's (a first
// turn of exactly zero counts as positive), and clockwise when the running
// sum of (b.x - a.x) * (b.y + a.y), taken in point order, is positive.  The
// last two steps wrap to the first points.  Every product and sum is a
// separately rounded FP64 operation, as in tg (the library is built without
// multiply-add contraction).
__host__ __device__ inline uint8_t tg_ring_flags(const double2* p, uint32_t n) {
  if (n < 2) return kRingFlagsSet;
  bool concave = false;
  int dir = 0;
  double cwc = 0.0;
  for (uint32_t i = 0; i < n; i++) {
    const double2 a = p[i];
    double2 b, c;
    if (i + 2 < n) {
      b = p[i + 1];
      c = p[i + 2];
    } else if (i == n - 1) {
      b = p[0];
      c = p[1];
    } else {
      b = p[i + 1];
      c = p[0];
    }
    cwc = cwc + (b.x - a.x) * (b.y + a.y);
    if (!concave) {
      const double z = (b.x - a.x) * (c.y - b.y) - (b.y - a.y) * (c.x - b.x);
      if (dir == 0) {
        dir = z < 0 ? -1 : 1;
      } else if (z < 0) {
        if (dir == 1) concave = true;
      } else if (z > 0) {
        if (dir == -1) concave = true;
      }
    }
  }
  uint8_t f = kRingFlagsSet;
  if (!concave) f |= kRingConvex;
  if (cwc > 0) f |= kRingClockwise;
  return f;
}

}  // namespace spj
