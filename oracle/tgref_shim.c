/*
 * tgref_shim.c — thin C entry points over the reference's vendored tg library
 * (c/sedona-tg/src/tg/tg.c, compiled from the reference tree by
 * oracle/Makefile into oracle/_ref/).  TEST INFRASTRUCTURE ONLY: it pins the
 * oracle's restatement (spj_oracle.c) against the reference's own predicate
 * code in this container; the fixtures it produces are committed under
 * tests/golden/.  Argument order follows the reference refiner:
 * tg_geom_<pred>(build, probe) (rust/sedona-spatial-join/src/refine/tg.rs:322-357).
 */
#include <stddef.h>
#include <stdint.h>
#include "tg.h"

/* index: 0 none, 1 natural, 2 ystripes, 3 default (tg.rs:39-47) */
static enum tg_index ix_of(int index) {
  switch (index) {
    case 0: return TG_NONE;
    case 1: return TG_NATURAL;
    case 2: return TG_YSTRIPES;
    default: return TG_DEFAULT;
  }
}

/* pred codes: gpuspatial_c.h:142-151 order */
int tgref_pred(const uint8_t* wb, size_t lb, const uint8_t* wp, size_t lp, int pred, int index) {
  struct tg_geom* b = tg_parse_wkb_ix(wb, lb, ix_of(index));
  struct tg_geom* p = tg_parse_wkb_ix(wp, lp, ix_of(index));
  int r = -1;
  if (b && p && !tg_geom_error(b) && !tg_geom_error(p)) {
    switch (pred) {
      case 0: r = tg_geom_equals(b, p); break;
      case 1: r = tg_geom_disjoint(b, p); break;
      case 2: r = tg_geom_touches(b, p); break;
      case 3: r = tg_geom_contains(b, p); break;
      case 4: r = tg_geom_covers(b, p); break;
      case 5: r = tg_geom_intersects(b, p); break;
      case 6: r = tg_geom_within(b, p); break;
      case 7: r = tg_geom_coveredby(b, p); break;
    }
  }
  if (b) tg_geom_free(b);
  if (p) tg_geom_free(p);
  return r;
}

int tgref_raycast(double ax, double ay, double bx, double by, double px, double py) {
  struct tg_segment s = {{ax, ay}, {bx, by}};
  struct tg_point p = {px, py};
  return (int)tg_raycast(s, p);
}

int tgref_segment_intersects(double ax, double ay, double bx, double by, double cx, double cy,
                             double dx, double dy) {
  struct tg_segment s1 = {{ax, ay}, {bx, by}}, s2 = {{cx, cy}, {dx, dy}};
  return tg_segment_intersects_segment(s1, s2);
}
