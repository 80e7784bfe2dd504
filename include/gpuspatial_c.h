/*
 * gpuspatial_c.h — the C ABI of the GB300 spatial-join library.
 *
 * Drop-in replacement for the reference's libgpuspatial C interface
 * (c/sedona-libgpuspatial/libgpuspatial/include/gpuspatial/gpuspatial_c.h).
 * Struct layouts, member order, function-pointer signatures, enum values and
 * error conventions are kept identical so the reference's Rust bindings
 * (c/sedona-libgpuspatial/src/libgpuspatial.rs, generated by bindgen from
 * that header) link against this library unchanged:
 *   - functions return 0 on success and EINVAL on failure; the message is
 *     available from get_last_error (per object) or, for probe, from
 *     context_get_last_error (per context, so concurrent probes do not race);
 *   - the caller owns rect buffers, index arrays and Arrow arrays (borrowed
 *     for the duration of the call); callback buffers are valid only inside
 *     the callback;
 *   - every call selects the runtime's device first.
 * Entry points beyond the reference interface are declared in spj_gb300.h.
 */
#ifndef SPJ_GPUSPATIAL_C_H
#define SPJ_GPUSPATIAL_C_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

struct ArrowSchema;
struct ArrowArray;

/* gpuspatial_c.h:28-38 in the reference.  ptx_root is accepted and ignored
 * (there is no OptiX pipeline to load). */
struct GpuSpatialRuntimeConfig {
  const char* ptx_root;
  int device_id;
  bool use_cuda_memory_pool;
  int cuda_memory_pool_init_precent;
};

/* gpuspatial_c.h:40-53.  One per process. */
struct GpuSpatialRuntime {
  int (*init)(struct GpuSpatialRuntime* self, struct GpuSpatialRuntimeConfig* config);
  void (*release)(struct GpuSpatialRuntime* self);
  const char* (*get_last_error)(struct GpuSpatialRuntime* self);
  void* private_data;
};

/* gpuspatial_c.h:54-55 */
void GpuSpatialRuntimeCreate(struct GpuSpatialRuntime* runtime);

/* gpuspatial_c.h:57-62 */
struct GpuSpatialIndexConfig {
  const struct GpuSpatialRuntime* runtime;
  uint32_t concurrency;
};

/* gpuspatial_c.h:64-67 */
struct SedonaSpatialIndexContext {
  void* private_data;
};

/* gpuspatial_c.h:69-128.  Rects are [min_x, min_y, max_x, max_y] float32; a
 * rect with NaN is empty; a degenerate rect is a point.  probe reports every
 * (build, probe) pair of intersecting rects (closed intervals). */
struct SedonaFloatIndex2D {
  int (*clear)(struct SedonaFloatIndex2D* self);
  void (*create_context)(struct SedonaSpatialIndexContext* context);
  void (*destroy_context)(struct SedonaSpatialIndexContext* context);
  int (*push_build)(struct SedonaFloatIndex2D* self, const float* buf, uint32_t n_rects);
  int (*finish_building)(struct SedonaFloatIndex2D* self);
  int (*probe)(struct SedonaFloatIndex2D* self, struct SedonaSpatialIndexContext* context,
               const float* buf, uint32_t n_rects,
               int (*callback)(const uint32_t* build_indices, const uint32_t* probe_indices,
                               uint32_t length, void* user_data),
               void* user_data);
  const char* (*get_last_error)(struct SedonaFloatIndex2D* self);
  const char* (*context_get_last_error)(struct SedonaSpatialIndexContext* context);
  void (*release)(struct SedonaFloatIndex2D* self);
  void* private_data;
};

/* gpuspatial_c.h:130-134 */
int GpuSpatialIndexFloat2DCreate(struct SedonaFloatIndex2D* index,
                                 const struct GpuSpatialIndexConfig* config);

/* gpuspatial_c.h:136-145.  compress_bvh and pipeline_batches are accepted;
 * the build side is decoded once into HBM, so neither changes results. */
struct GpuSpatialRefinerConfig {
  const struct GpuSpatialRuntime* runtime;
  uint32_t concurrency;
  bool compress_bvh;
  uint32_t pipeline_batches;
};

/* gpuspatial_c.h:142-151: same values. */
enum SedonaSpatialRelationPredicate {
  SedonaSpatialPredicateEquals = 0,
  SedonaSpatialPredicateDisjoint,
  SedonaSpatialPredicateTouches,
  SedonaSpatialPredicateContains,
  SedonaSpatialPredicateCovers,
  SedonaSpatialPredicateIntersects,
  SedonaSpatialPredicateWithin,
  SedonaSpatialPredicateCoveredBy
};

/* gpuspatial_c.h:153-210.  Geometries are Arrow binary / large_binary WKB
 * (Point, Polygon, MultiPolygon; 2D).  refine evaluates
 * predicate(build[build_indices[i]], probe[probe_indices[i]]) with the
 * semantics of the reference CPU join's default refiner and compacts both
 * arrays in place, ordered by probe index; *new_indices_size receives the
 * number kept. */
struct SedonaSpatialRefiner {
  int (*clear)(struct SedonaSpatialRefiner* self);
  int (*init_build_schema)(struct SedonaSpatialRefiner* self,
                           const struct ArrowSchema* build_schema);
  int (*push_build)(struct SedonaSpatialRefiner* self, const struct ArrowArray* build_array);
  int (*finish_building)(struct SedonaSpatialRefiner* self);
  int (*refine)(struct SedonaSpatialRefiner* self, const struct ArrowSchema* probe_schema,
                const struct ArrowArray* probe_array,
                enum SedonaSpatialRelationPredicate predicate, uint32_t* build_indices,
                uint32_t* probe_indices, uint32_t indices_size, uint32_t* new_indices_size);
  const char* (*get_last_error)(struct SedonaSpatialRefiner* self);
  void (*release)(struct SedonaSpatialRefiner* self);
  void* private_data;
};

/* gpuspatial_c.h:212-216 */
int GpuSpatialRefinerCreate(struct SedonaSpatialRefiner* refiner,
                            const struct GpuSpatialRefinerConfig* config);

#ifdef __cplusplus
}
#endif
#endif
