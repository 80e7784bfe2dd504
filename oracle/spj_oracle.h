/*
 * spj_oracle.h — CPU oracle for the spatial-join hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against (tests/, __graft_entry__.smoke() and the cpu_baseline
 * leg of bench.py).  The product never links, loads or calls it.
 *
 * It restates, in plain C, the semantics of the reference CPU spatial join:
 *   - WKB parsing and xy bounds  (rust/sedona-geometry/src/bounds.rs:240)
 *   - f64 -> f32 outward box rounding
 *       (rust/sedona-spatial-join/src/utils/bounds.rs:49-63,147-162)
 *   - the GPU factory's round-to-nearest point boxes
 *       (rust/sedona-spatial-join-gpu/src/join_provider.rs:109-141)
 *   - closed-interval f32 box filter
 *       (rust/sedona-spatial-join/src/index/default_spatial_index.rs:529-569)
 *   - the default tg refiner: tg_geom_<pred>(build, probe)
 *       (rust/sedona-spatial-join/src/refine/tg.rs:322-357,
 *        c/sedona-tg/src/tg/tg.c — cited per function in spj_oracle.c)
 *   - ST_DWithin: rect expansion + hypot(dx,dy) <= d
 *       (rust/sedona-spatial-join/src/operand_evaluator.rs:605-607,
 *        rust/sedona-spatial-join/src/refine/geo.rs:312-321)
 *   - KNN: top-k by (distance total order, build row id)
 *       (rust/sedona-spatial-join/tests/spatial_join_integration.rs:1373-1414)
 */
#ifndef SPJ_ORACLE_H
#define SPJ_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Predicate codes: same order as enum SedonaSpatialRelationPredicate
 * (c/sedona-libgpuspatial/libgpuspatial/include/gpuspatial/gpuspatial_c.h:142-151). */
enum {
  SPJO_EQUALS = 0,
  SPJO_DISJOINT = 1,
  SPJO_TOUCHES = 2,
  SPJO_CONTAINS = 3,
  SPJO_COVERS = 4,
  SPJO_INTERSECTS = 5,
  SPJO_WITHIN = 6,
  SPJO_COVEREDBY = 7,
  SPJO_DWITHIN = 100
};

/* Geometry kinds after parsing. */
enum { SPJO_EMPTY = 0, SPJO_POINT = 1, SPJO_POLYGON = 3, SPJO_MULTIPOLYGON = 6 };

typedef struct spj_geoms spj_geoms;

/* Parse an Arrow binary WKB column.  offsets has n+1 entries (int64, already
 * widened from int32 by the caller when needed); validity is an Arrow LSB
 * bitmap or NULL.  Returns NULL on error and writes a message into err. */
spj_geoms* spjo_parse(const int64_t* offsets, const uint8_t* data, const uint8_t* validity,
                      int64_t n, char* err, int errlen);
void spjo_free_geoms(spj_geoms* g);
int64_t spjo_count(const spj_geoms* g);
int spjo_kind(const spj_geoms* g, int64_t i);
int64_t spjo_num_vertices(const spj_geoms* g);

/* f32 boxes, 4 floats per row [xmin,ymin,xmax,ymax]; empty rows get NaN.
 * mode 0: Bounds2D::new (outward) for every geometry (CPU provider);
 * mode 1: GPU factory — points get a round-to-nearest degenerate box. */
void spjo_boxes(const spj_geoms* g, int mode, float* out);

/* Point coordinates of a point geometry (row i); returns 0 if not a point. */
int spjo_point(const spj_geoms* g, int64_t i, double* x, double* y);

/* One predicate, argument order pred(build, probe). */
int spjo_predicate(const spj_geoms* build, int64_t bi, const spj_geoms* probe, int64_t pi,
                   int pred);

/* tg primitives exposed for known-answer tests.
 * raycast result: 0 OUT, 1 IN, 2 ON (tg.c:95 enum order). */
int spjo_raycast(double ax, double ay, double bx, double by, double px, double py);
int spjo_segment_intersects(double ax, double ay, double bx, double by, double cx, double cy,
                            double dx, double dy);
int spjo_collinear(double x1, double y1, double x2, double y2, double x3, double y3);

/* Closed-interval intersection join of two f32 rect arrays (candidate set,
 * the SedonaFloatIndex2D::probe contract).  NaN rects are empty.  Output is
 * malloc'd, sorted by (probe, build).  Returns the pair count or -1. */
int64_t spjo_rect_join(const float* build_rects, int64_t nb, const float* probe_rects,
                       int64_t np, int nthreads, uint32_t** out_build, uint32_t** out_probe);

/* Full join: box filter + tg refine (pred) or DWithin (pred = SPJO_DWITHIN
 * with distance).  Output malloc'd, sorted by (probe, build).
 * Returns the pair count, or -1 with a message in err. */
int64_t spjo_join(const spj_geoms* build, const spj_geoms* probe, int pred, double distance,
                  int nthreads, uint32_t** out_build, uint32_t** out_probe, char* err,
                  int errlen);

/* KNN join over point geometries: for every probe row, the k build rows with
 * the smallest hypot distance, ties broken by build row id.  Output rows are
 * (probe, rank) ordered; out arrays hold n_probe*k entries, unused slots have
 * build = 0xFFFFFFFF and dist = +inf.  Returns 0 or -1. */
/* ST_DWithin with one distance per probe row (the reference's distance
 * column, rust/sedona-spatial-join/src/operand_evaluator.rs:556-627). */
int64_t spjo_join_dists(const spj_geoms* build, const spj_geoms* probe, const double* dists,
                        int nthreads, uint32_t** out_build, uint32_t** out_probe, char* err,
                        int errlen);
/* build.distance_ext(probe): the Euclidean distance the DWithin refine uses. */
double spjo_geo_distance(const spj_geoms* build, int64_t bi, const spj_geoms* probe, int64_t pi);

int spjo_knn(const spj_geoms* build, const spj_geoms* probe, int k, int nthreads,
             uint32_t* out_build, double* out_dist, char* err, int errlen);

/* Order-independent digest of a pair set: sum of splitmix64(probe<<32|build). */
uint64_t spjo_digest(const uint32_t* build, const uint32_t* probe, int64_t n);

void spjo_free(void* p);

/* GeoParquet (spj_parquet.c): a flat BYTE_ARRAY column (NULL: the "geo"
 * metadata's primary column) of every row group.  On success returns 0 and
 * malloc'd arrays: offsets (n + 1, nulls are empty), data, valid (one byte
 * per row); free them with spjo_free.  On failure returns -1 with a message
 * in err. */
int spjo_parquet_read(const char* path, const char* column, int64_t* n_rows, int64_t** offsets,
                      uint8_t** data, uint8_t** valid, char* err, int errcap);

#ifdef __cplusplus
}
#endif
#endif
