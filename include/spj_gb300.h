/*
 * spj_gb300.h — entry points of the GB300 spatial-join library beyond the
 * reference's gpuspatial_c.h.  None of these have a counterpart in the
 * reference's C interface; each line says which reference caller it serves.
 *
 *  - SpjJoin*: the fused build/probe join that GPUSpatialIndex::query_batch
 *    (rust/sedona-spatial-join-gpu/src/index/gpu_spatial_index.rs:163-229)
 *    performs as two FFI calls (index probe, then refine) with host round
 *    trips in between.  Here probe WKB goes in and the refined (build, probe)
 *    pairs come out, with no host work in between.  It also carries ST_DWithin
 *    (rejected on the reference GPU path,
 *    rust/sedona-spatial-join-gpu/src/physical_planner.rs:155).
 *  - SpjJoinProbeDevice: device-resident variant (the batched mode: WKB
 *    columns already in HBM, pairs left in HBM).
 *  - SpjKnn*: the KNN join (query_knn is NotImplemented on the reference GPU
 *    path, rust/sedona-spatial-join-gpu/src/index/gpu_spatial_index.rs:252-264;
 *    the CPU semantics followed are
 *    rust/sedona-spatial-join/src/index/default_spatial_index.rs:306-502).
 *  - SpjHostRegister / SpjHostUnregister: page-lock caller buffers so the
 *    host<->device copies of probe columns and results run at full speed.
 *
 * All functions return 0 on success and EINVAL (or another errno value) on
 * failure; SpjJoinLastError / SpjKnnLastError give the message.  An SpjJoin
 * or SpjKnn object is used by one thread at a time.
 */
#ifndef SPJ_GB300_H
#define SPJ_GB300_H

#include <stdint.h>

#include "gpuspatial_c.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Predicate code for ST_DWithin(build, probe, distance); relation predicates
 * use enum SedonaSpatialRelationPredicate. */
#define SPJ_PREDICATE_DWITHIN 100

/* refine_form values */
#define SPJ_REFINE_PLAIN_F64 0 /* every test in FP64, full segment scans */
#define SPJ_REFINE_FAST_F32 1  /* y-band index + FP32 filter + FP64 escalation */

struct SpjJoinConfig {
  const struct GpuSpatialRuntime* runtime; /* initialized runtime (device) */
  uint32_t leaf_size;                      /* LBVH leaf size, 0 = by build side (16 for
                                              points, 4 otherwise) */
  int32_t refine_form;                     /* SPJ_REFINE_* (default FAST_F32) */
  int32_t profile;                         /* 1: time phases with CUDA events */
  int32_t probe_order; /* traversal order of probe rows: 0 = Morton order of the
                          box centres from 65536 rows up, 1 = always, -1 = row
                          order; the pairs and their order do not depend on it */
};

/* An Arrow binary (int32 offsets) or large_binary (int64 offsets) WKB column
 * whose buffers live in device memory.  offsets index data; validity is an
 * LSB bitmap or NULL, its bits start at validity_offset. */
struct SpjDeviceWkb {
  int64_t length;
  const void* offsets;
  int32_t offsets_are_64bit;
  const uint8_t* data;
  uint64_t data_length;
  const uint8_t* validity;
  int64_t validity_offset;
};

/* Per-phase device time (ms, CUDA events on the join's stream; zero unless
 * profile = 1) and counters since the last reset. */
struct SpjJoinStats {
  double ms_decode, ms_filter, ms_refine, ms_compact;
  uint64_t calls, probe_rows, candidates, results;
  uint64_t escalations;     /* segment / distance tests decided in FP64 */
  uint64_t pairs_evaluated; /* candidate pairs refined */
  uint64_t kernel_launches;
  uint64_t probe_bytes;
  uint64_t build_rows, build_vertices, build_device_bytes;
};

typedef struct SpjJoin SpjJoin;

int SpjJoinCreate(const struct SpjJoinConfig* config, SpjJoin** out);
void SpjJoinRelease(SpjJoin* join);
const char* SpjJoinLastError(SpjJoin* join);

/* Build side from a host Arrow array (binary / large_binary WKB); may be
 * called repeatedly to append batches, then SpjJoinFinishBuild. */
int SpjJoinPushBuildArrow(SpjJoin* join, const struct ArrowSchema* schema,
                          const struct ArrowArray* array);
int SpjJoinFinishBuild(SpjJoin* join);
/* Execution options (they change speed, never the pairs or their order):
 *   "probe_order"       -1 row order, 0 Morton order from 65536 rows up, 1 always
 *   "candidate_order"   3 (default) auto: 2 for relation predicates with 4M+
 *                       candidates over a build side that is not all points,
 *                       else 0; 2 by build row then probe Morton rank, 0 as
 *                       listed
 *   "order_tiles"       -1 (default: auto, tiles of 524,288 candidates),
 *                       0-16: build-major order within 2^n equal tiles of
 *                       the probes' Morton-ordered candidate list
 *   "refine_min_blocks" 0 (default: auto, 6 for ST_Intersects / ST_Disjoint
 *                       in build-major candidate order, else 4), 4 or 6:
 *                       FP32 refine built for that many resident 256-thread
 *                       blocks per SM (fewer registers)
 *   "refine_split"      2 (default: auto, on unless the candidates are in
 *                       build-major order), 1 on, 0 off: FP32 refine of
 *                       relation predicates in two passes (a cheap pass over
 *                       all pairs queues the pairs it leaves open for a full
 *                       pass); 3 on, with the queue sorted back into the
 *                       candidate order before the full pass
 *   "host_slices"       0 (default: auto, 2 from 524,288 rows), 1 (one
 *                       call), 2-64: row slices of SpjJoinProbeHost
 *   "cell_grid"         1 (default) / 0: per-ring cell grids on the build side
 *                       (clean cells answer point-in-ring tests in O(1)); set
 *                       before the build
 *   "grid_rings"        0 (default) / 1: ring-ring and ring-in-ring tests
 *                       answer from the build ring's clean cells when the
 *                       probe ring's box lies in them
 *   "dwithin_arena"     2 (default: auto, on when the probes are not in
 *                       Morton order), 1 on, 0 off: fused ST_DWithin keeps
 *                       the results past a probe's slots in an overflow
 *                       arena (of the slots' size), so only probes it cannot
 *                       hold are traversed again
 *   "dwithin_slots"     64 (default), 0-1024: fused ST_DWithin keeps up to this
 *                       many build ids per probe from its counting pass
 *   "fuse_dwithin"      1 (default) / 0: point-point ST_DWithin decided inside
 *                       the traversal, no candidate pairs (set before the build)
 * The counterpart of the reference's gpu.* session options
 * (rust/sedona-spatial-join-gpu/src/options.rs:20-51). */
int SpjJoinSetOption(SpjJoin* join, const char* key, int64_t value);
/* Build side from a device column (replaces any pushed batches). */
int SpjJoinBuildDevice(SpjJoin* join, const struct SpjDeviceWkb* column);

/* Probe with a host Arrow array; the refined pairs (probe ids offset by
 * probe_base) are delivered through callback, in ascending probe order,
 * possibly in several chunks; a non-zero return from callback stops the
 * probe and is returned.  predicate: a SedonaSpatialRelationPredicate, or
 * SPJ_PREDICATE_DWITHIN with `distance` (or the distance column of
 * SpjJoinSetProbeDistances): the reference's build.distance_ext(probe) <= d
 * (rust/sedona-spatial-join/src/refine/geo.rs:312-321) between points,
 * polygons and multipolygons; the probe rows' rects are expanded by d. */
int SpjJoinProbeArrow(SpjJoin* join, const struct ArrowSchema* schema,
                      const struct ArrowArray* array, int32_t predicate, double distance,
                      uint32_t probe_base,
                      int (*callback)(const uint32_t* build_indices,
                                      const uint32_t* probe_indices, uint64_t length,
                                      void* user_data),
                      void* user_data);

/* Probe with a device column; *d_build / *d_probe receive device arrays of
 * *n_pairs entries, owned by the join and valid until its next probe. */
int SpjJoinProbeDevice(SpjJoin* join, const struct SpjDeviceWkb* column, int32_t predicate,
                       double distance, uint32_t probe_base, const uint32_t** d_build,
                       const uint32_t** d_probe, uint64_t* n_pairs);

/* Probe with a host column given as plain buffers (the same layout as an
 * Arrow binary array); results are copied into caller buffers of capacity
 * `capacity` pairs.  *n_pairs receives the full count; if it exceeds
 * capacity ENOSPC is returned and the buffers' contents are unspecified.
 * A column of 524,288 rows or more is probed in two row slices (option
 * "host_slices" sets another count) by two host threads on two workspaces,
 * so that both slices' kernels and each slice's copies overlap; the pairs
 * and their order are those of one call over the whole column.  Page-locked buffers
 * (cudaHostAlloc / cudaHostRegister) let those copies run asynchronously. */
int SpjJoinProbeHost(SpjJoin* join, int64_t length, const void* offsets,
                     int32_t offsets_are_64bit, const uint8_t* data, const uint8_t* validity,
                     int32_t predicate, double distance, uint32_t probe_base,
                     uint32_t* out_build, uint32_t* out_probe, uint64_t capacity,
                     uint64_t* n_pairs);

/* ST_DWithin with a distance column (rust/sedona-spatial-join/src/
 * operand_evaluator.rs:556-627: the probe rows' rects are expanded by their
 * own distance): the next probes with SPJ_PREDICATE_DWITHIN take distances[i]
 * for probe row i (rows counted within the probed column) instead of their
 * `distance` argument; the column must have n rows.  A negative or NaN
 * distance (a null) matches nothing.  distances is host memory, or device
 * memory when device == 1; it is copied.  NULL clears the column. */
int SpjJoinSetProbeDistances(SpjJoin* join, const double* distances, uint64_t n,
                             int32_t device);

/* The CUDA stream (cudaStream_t) the join launches its kernels on. */
void* SpjJoinStream(SpjJoin* join);
int SpjJoinGetStats(SpjJoin* join, struct SpjJoinStats* out);
int SpjJoinResetStats(SpjJoin* join);

/* ------------------------------------------------------------------------ */
/* Batched probe stream: many uneven record batches of point WKB probed in
 * one CUDA-graph replay (a persistent work-queue kernel decodes every batch,
 * then filter, refine and compaction run once over the whole stream, with no
 * host round trip in between).  Serves SpatialJoinStream's per-batch
 * query_batch loop (rust/sedona-spatial-join/src/stream.rs:1166-1200) without
 * a host round trip per batch.  The SpjJoin it is created from must outlive
 * it.  Relation predicates only; batch rows must be points. */

typedef struct SpjStream SpjStream;

int SpjStreamCreate(SpjJoin* join, SpjStream** out);
void SpjStreamRelease(SpjStream* stream);
const char* SpjStreamLastError(SpjStream* stream);
/* Device columns, one per batch; probe ids are global over the batches in
 * order (batch i starts after the rows of batches 0..i-1). */
int SpjStreamSetBatches(SpjStream* stream, const struct SpjDeviceWkb* batches,
                        int32_t n_batches);
/* One replay over all batches; pairs (device arrays owned by the stream,
 * valid until the next run) grouped by probe row in ascending order. */
int SpjStreamRun(SpjStream* stream, int32_t predicate, const uint32_t** d_build,
                 const uint32_t** d_probe, uint64_t* n_pairs);
/* block: 128 or 256 threads (decode kernel); chunk_rows: rows per work item; leaf_size:
 * LBVH leaf size (rebuilds the index). */
int SpjStreamSetParams(SpjStream* stream, int32_t block, uint32_t chunk_rows, uint32_t leaf_size);
/* Times block x chunk_rows x leaf_size candidates on the current batches,
 * keeps the fastest and returns it; cache_path (may be NULL) stores results
 * per device and workload signature and is consulted first. */
int SpjStreamAutotune(SpjStream* stream, int32_t predicate, const char* cache_path,
                      int32_t* block, uint32_t* chunk_rows, uint32_t* leaf_size);
/* Device time of the last replay (CUDA events around the graph launch),
 * FP64-escalated tests so far and kernel launches per replay. */
int SpjStreamGetStats(SpjStream* stream, double* ms_last, uint64_t* escalations,
                      uint64_t* launches_per_replay);
void* SpjStreamCudaStream(SpjStream* stream);

/* ------------------------------------------------------------------------ */
/* Learned point index: the build points sorted by a 32-bit Hilbert key on a
 * 2^16 x 2^16 grid over their extent, a two-stage piecewise-linear model of
 * key -> rank (a root line picks one of `leaves` per-leaf lines) trained on
 * the GPU, lookups searched within each leaf's measured error and verified
 * exactly; the LBVH over the same points is the fallback (leaves over the
 * window) and the arbiter.  No counterpart in the reference (which has no
 * learned index); it serves point build sides of the join (probe points:
 * exact-point lookups; probe polygons such as range boxes: ST_Intersects /
 * ST_Within / ST_CoveredBy(build point, probe polygon)). */

typedef struct SpjLearned SpjLearned;

struct SpjLearnedConfig {
  const struct GpuSpatialRuntime* runtime;
  uint32_t leaves; /* 0 = 4096 */
  uint32_t window; /* max per-leaf error served by the model, 0 = 4096 */
};

struct SpjLearnedStats {
  uint64_t points, lookups, window_misses, lbvh_fallbacks, search_steps;
  uint32_t leaves, max_err, leaves_over_window, trained;
  /* stage one: radix table of root_entries prefixes of (key - first key)
   * >> root_shift; mean_err: mean over leaves of the max |rank error| */
  double root_shift, root_entries, mean_err, grad_norm_after, ms_build;
  uint64_t ranges; /* build-point ranges (key runs, LBVH leaves) the queries produced */
  /* cumulative query phase times (CUDA events): probe ordering, ranges
   * through the model, candidate evaluation and output */
  double ms_order, ms_ranges, ms_eval;
  uint32_t window;     /* lookups */
  uint32_t window_box; /* the grid cells of range rows */
  uint64_t kernel_launches; /* this library's kernels launched by queries */
};

int SpjLearnedCreate(const struct SpjLearnedConfig* config, SpjLearned** out);
void SpjLearnedRelease(SpjLearned* li);
const char* SpjLearnedLastError(SpjLearned* li);
/* Build from a device WKB column of points (non-point rows are skipped). */
int SpjLearnedBuildDevice(SpjLearned* li, const struct SpjDeviceWkb* points);
/* trained = 0 replaces the trained per-leaf lines with the untrained start
 * (the line through each leaf's first and last key), 1 retrains. */
int SpjLearnedSetTrained(SpjLearned* li, int32_t trained);
/* Probe with a device WKB column; pairs (device arrays owned by the index,
 * valid until its next query) grouped by probe row; probe ids offset by
 * probe_base. */
int SpjLearnedQueryDevice(SpjLearned* li, const struct SpjDeviceWkb* probe, int32_t predicate,
                          uint32_t probe_base, const uint32_t** d_build,
                          const uint32_t** d_probe, uint64_t* n_pairs);
/* Per-leaf squared loss and gradient at host parameters a[L], b[L]
 * (evaluated by the training kernels; for checks against a CPU oracle). */
int SpjLearnedLossAndGrad(SpjLearned* li, const double* a, const double* b, double* loss,
                          double* grad_a, double* grad_b);
/* Host copies of the sorted keys (points entries), leaf starts (L+1), leaf
 * key origins, per-leaf lines and errors (L each). */
int SpjLearnedExport(SpjLearned* li, uint32_t* keys, uint32_t* leaf_start, uint32_t* leaf_kc,
                     double* a, double* b, uint32_t* err);
int SpjLearnedGetStats(SpjLearned* li, struct SpjLearnedStats* out);
void* SpjLearnedStream(SpjLearned* li);
/* The window: the largest per-leaf error the model serves; rows whose leaf
 * error exceeds it take the LBVH fallback.  Sets the window of lookups and
 * of range rows alike.  Queries only; no rebuild. */
int SpjLearnedSetWindow(SpjLearned* li, uint32_t window);
/* Times queries of the sample columns (device WKB) for windows 2^10 .. 2^17
 * and the model's max error (no fallback), best of two runs each: first the
 * window of range rows, then that of lookups; sets both and returns the
 * lookup window in *window (both are in SpjLearnedStats). */
int SpjLearnedAutotuneWindow(SpjLearned* li, const struct SpjDeviceWkb* samples,
                             uint32_t n_samples, int32_t predicate, uint32_t* window);

/* ------------------------------------------------------------------------ */
/* KNN join over point columns                                              */

typedef struct SpjKnn SpjKnn;

struct SpjKnnConfig {
  const struct GpuSpatialRuntime* runtime;
  uint32_t leaf_size;  /* 0 = default */
  int32_t refine_form; /* SPJ_REFINE_* */
};

int SpjKnnCreate(const struct SpjKnnConfig* config, SpjKnn** out);
void SpjKnnRelease(SpjKnn* knn);
const char* SpjKnnLastError(SpjKnn* knn);
/* Build points: n FP64 (x, y) pairs, host memory. */
int SpjKnnBuild(SpjKnn* knn, const double* xy, uint64_t n);
/* For each probe point, the k nearest build points by Euclidean distance,
 * ties broken by build row id; out_idx / out_dist hold n_probe*k entries in
 * (probe, rank) order; slots beyond the build size get UINT32_MAX / +inf.
 * Host or device pointers (device == 1) for all four arrays. */
int SpjKnnQuery(SpjKnn* knn, const double* probe_xy, uint64_t n_probe, uint32_t k,
                uint32_t* out_idx, double* out_dist, int32_t device);
/* The same with variable-length results, as the reference's
 * query_knn(probe, k, use_spheroid = false, include_tie_breakers, ...)
 * returns them per probe (rust/sedona-spatial-join/src/index/spatial_index.rs:52-64,
 * default_spatial_index.rs:306-502): probe i's results are
 * out_idx / out_dist[offsets[i] .. offsets[i + 1]), its k nearest (fewer when
 * the build side is smaller; none for a NaN / empty probe) and, with
 * include_tie_breakers, every other build point whose distance is within
 * 1e-9 of the k-th (DISTANCE_TOLERANCE, spatial_index.rs:32).  offsets
 * (n_probe + 1 entries), out_idx and out_dist are host arrays; probe_xy is
 * host or device memory (device == 1).  *total receives the result count;
 * if it exceeds capacity, only offsets are written and ENOSPC is returned. */
int SpjKnnQueryTies(SpjKnn* knn, const double* probe_xy, uint64_t n_probe, uint32_t k,
                    int32_t include_tie_breakers, int32_t device, uint64_t* offsets,
                    uint32_t* out_idx, double* out_dist, uint64_t capacity, uint64_t* total);
/* query_knn over a WKB column (Arrow binary / large_binary, host memory):
 * the column is decoded on the device; rows must be points, and empty or
 * null rows get no results (default_spatial_index.rs:331-339).  Outputs as
 * SpjKnnQueryTies. */
int SpjKnnQueryArrow(SpjKnn* knn, const struct ArrowSchema* schema,
                     const struct ArrowArray* array, uint32_t k, int32_t include_tie_breakers,
                     uint64_t* offsets, uint32_t* out_idx, double* out_dist, uint64_t capacity,
                     uint64_t* total);
void* SpjKnnStream(SpjKnn* knn);
/* Cumulative counters since SpjKnnCreate: probe points queried, FP64
 * distance keys evaluated, and probes whose k-set the FP32 pass could not
 * prove (answered by the exact kernel). */
int SpjKnnGetStats(SpjKnn* knn, uint64_t* queries, uint64_t* exact_evals, uint64_t* redone);

/* ------------------------------------------------------------------------ */
/* Partitioned (out-of-core) join.                                          */
/*                                                                          */
/* For build sides larger than the device: the reference's out-of-core    */
/* join partitions the build side with a KDB tree built from a sample of   */
/* its boxes (rust/sedona-spatial-join/src/prepare.rs:260-340,             */
/* partitioning/kdb.rs), assigns every build row to the leaf it overlaps   */
/* most and every probe row to the one partition whose build bounds it     */
/* meets (Multi when several: partitioning/flat.rs), spills both sides and */
/* joins partition by partition.  Here both columns stay in host memory:   */
/* their boxes are decoded in row ranges, the tree is built on the host    */
/* and applied on the device, and every pass gathers one partition's build */
/* rows (and its probe rows plus the Multi rows) onto the device -- read   */
/* by the device straight from host memory where it can read pageable      */
/* memory (Grace's coherent link), else gathered by host threads into      */
/* page-locked staging -- and builds and probes them with the join's       */
/* options.  Every pair is delivered once.                                 */

/* A WKB column (Arrow binary / large_binary layout) in host memory. */
struct SpjHostWkb {
  int64_t length;
  const void* offsets;
  int32_t offsets_are_64bit;
  const uint8_t* data;
  const uint8_t* validity; /* LSB bitmap or NULL */
  int64_t validity_offset;
};

struct SpjPartitionOptions {
  uint32_t num_partitions;     /* target KDB leaves; 0: from build_budget_bytes */
  uint32_t sample_rows;        /* build boxes sampled for the tree; 0 = 10,000 */
  uint64_t build_budget_bytes; /* device bytes one partition's build side may take
                                  (about 2.5x its WKB bytes); 0 with 0 partitions:
                                  one partition */
  uint64_t seed;               /* of the sample */
  int32_t host_gather;         /* 1: gather each pass's rows on the host even
                                  where the device can read host memory */
  int32_t record_layout;       /* 1: keep every row's partition for
                                  SpjJoinPartitionLayout (a copy of 4 bytes per
                                  row to the host) */
};

struct SpjPartitionStats {
  uint32_t partitions, passes;
  uint64_t build_rows_max;    /* build rows of the largest partition */
  uint64_t probe_rows_multi;  /* probe rows meeting several partitions */
  uint64_t probe_rows_none;   /* probe rows meeting none (null, empty or outside) */
  uint64_t probe_rows_probed; /* probe rows over all passes */
  uint64_t pairs;
  double ms_boxes, ms_partition, ms_passes; /* host wall time of the phases */
  int32_t direct_host_reads;  /* 1: the device read the columns in host memory */
};

/* The join of two host columns in partition passes.  Each pass's pairs (row
 * ids of the two columns) are delivered through callback; a non-zero return
 * stops the join and is returned.  Within a pass the pairs are grouped by
 * probe row (the partition's own probe rows first, then the Multi rows), in
 * ascending row order within each group; passes run in leaf order.
 * predicate / distance as SpjJoinProbeArrow (a distance column set with
 * SpjJoinSetProbeDistances applies).  The join's build side is replaced:
 * afterwards it holds the last partition.  stats may be NULL. */
int SpjJoinPartitioned(SpjJoin* join, const struct SpjHostWkb* build,
                       const struct SpjHostWkb* probe, int32_t predicate, double distance,
                       const struct SpjPartitionOptions* options,
                       int (*callback)(const uint32_t* build_indices,
                                       const uint32_t* probe_indices, uint64_t length,
                                       void* user_data),
                       void* user_data, struct SpjPartitionStats* stats);
/* The last SpjJoinPartitioned call's partitioning, for checks against the
 * reference's rules.  counts[4] (host) receives the leaves, the samples, the
 * tree's max items per node and max levels; with the other pointers NULL
 * only counts is written.  Otherwise (host arrays): extent[4]; leaves and
 * bounds (4 floats per leaf: min x, min y, max x, max y; the bounds of a
 * partition without build rows are NaN); samples (4 per sample, insertion
 * order); build_part (per build row: leaf, or 0xFFFFFFFF for a row without
 * a box); probe_part (per probe row: leaf, leaves for Multi, leaves + 1 for
 * None); build_part and probe_part only after a call with record_layout. */
int SpjJoinPartitionLayout(SpjJoin* join, uint32_t* counts, float* extent, float* leaves,
                           float* bounds, float* samples, uint32_t* build_part,
                           uint32_t* probe_part);

/* ------------------------------------------------------------------------ */
/* GeoParquet -> device.                                                    */
/*                                                                          */
/* The reference reads GeoParquet with arrow-rs on the CPU                  */
/* (rust/sedona-geoparquet/src/file_opener.rs:125-210; geometry columns and */
/* the primary column from the "geo" key, metadata.rs:382-460) and parses   */
/* the WKB values again on the CPU before the join (operand_evaluator.rs).  */
/* Here the host reads only the footer and the page headers; the column     */
/* chunks go to HBM in one copy and their pages are decompressed (SNAPPY or */
/* stored) and decoded (definition levels, PLAIN and dictionary-encoded     */
/* BYTE_ARRAY values, data pages v1 and v2) by kernels, into a device       */
/* column for SpjJoinBuildDevice / SpjJoinProbeDevice / SpjLearned*.        */
/* Other codecs and encodings, nested columns and GeoParquet's native       */
/* (non-WKB) encodings are rejected with a message.                         */

typedef struct SpjParquet SpjParquet;

/* Opens a file and parses its footer (host only, no device work).  On
 * failure *out is NULL and SpjParquetLastError(NULL) has the message. */
int SpjParquetOpen(const char* path, SpjParquet** out);
void SpjParquetRelease(SpjParquet* file);
/* The handle's last error; with NULL, the calling thread's last
 * SpjParquetOpen / SpjParquetWriteWkb error. */
const char* SpjParquetLastError(SpjParquet* file);
int SpjParquetInfo(SpjParquet* file, int64_t* num_rows, int32_t* num_row_groups,
                   int32_t* num_columns);
/* Leaf column i's name (dotted path), or with i = -1 the GeoParquet primary
 * geometry column; EINVAL when absent or when cap is too small. */
int SpjParquetColumnName(SpjParquet* file, int32_t i, char* buf, uint64_t cap);
int SpjParquetRowGroupRows(SpjParquet* file, int32_t row_group, int64_t* rows);
/* Reads row groups [rg_begin, rg_end) (rg_end < 0: to the last) of a WKB
 * column (NULL: the primary geometry column) onto `device`.  *out receives a
 * device Arrow large_binary column (int64 offsets; validity NULL when the
 * rows have no nulls) owned by the handle and valid until its next read or
 * release.  Synchronous. */
int SpjParquetReadWkb(SpjParquet* file, const char* column, int32_t rg_begin, int32_t rg_end,
                      int32_t device, struct SpjDeviceWkb* out);
/* The last read: device time in ms (H2D copy through the last kernel, CUDA
 * events), bytes read from the file, decompressed page bytes, WKB bytes. */
int SpjParquetGetStats(SpjParquet* file, double* ms_device, uint64_t* file_bytes,
                       uint64_t* page_bytes, uint64_t* value_bytes);
/* The last read's phases (ms, CUDA events): the H2D copy of the chunk bytes,
 * Snappy decompression (k_snappy_frags, k_snappy_pages), page decode
 * (dictionary and data pages: levels, value locations), and the value copy
 * with offsets and validity (k_copy_values, k_offsets64, k_pack_valid). */
int SpjParquetGetPhases(SpjParquet* file, double* ms_h2d, double* ms_decompress,
                        double* ms_decode, double* ms_values);

struct SpjParquetWriteOptions {
  int32_t compression;    /* 0 none, 1 SNAPPY */
  int32_t page_version;   /* 1 or 2 (data page v1 / v2) */
  int64_t row_group_rows; /* 0 = 1,048,576 */
  int64_t page_bytes;     /* values per page, 0 = 1 MiB */
};
/* Writes a host WKB column (Arrow binary / large_binary buffers) as a
 * GeoParquet 1.1 file with one optional BYTE_ARRAY column, PLAIN encoded
 * (the reference's writer: rust/sedona-geoparquet/src/writer.rs); host only.
 * options may be NULL (SNAPPY, v1 pages). */
int SpjParquetWriteWkb(const char* path, const char* column, int64_t length,
                       const void* offsets, int32_t offsets_are_64bit, const uint8_t* data,
                       const uint8_t* validity, int64_t validity_offset,
                       const struct SpjParquetWriteOptions* options);

/* ------------------------------------------------------------------------ */
/* Result materialisation on the device.                                    */
/*                                                                          */
/* The joined batch is built from the refined (build, probe) index pairs by */
/* one Arrow `take` per column (build_batch_from_indices,                   */
/* rust/sedona-spatial-join/src/utils/join_utils.rs:346-405, called from    */
/* build_joined_batch, rust/sedona-spatial-join/src/stream.rs:1466-1502);   */
/* outer, semi, anti and mark joins keep a visited bitmap of build rows     */
/* (mark_build_side_rows_as_visited, stream.rs:1447-1455) and emit the      */
/* unmatched (or matched) rows at the end (get_final_indices_from_bit_map,  */
/* join_utils.rs:95-124).  These entry points do both on device buffers so  */
/* the pairs never leave HBM.  Every pointer except the counts is device    */
/* memory; stream is a cudaStream_t (NULL = default stream); each call      */
/* synchronizes it.  Errors: EINVAL with SpjMaterializeLastError (per       */
/* thread), ENOSPC when an output is too small (the needed size is still    */
/* returned).                                                               */

/* An index of this value gathers a null row (the missing side of an outer
 * join's unmatched rows); so does an index >= n_values. */
#define SPJ_NULL_INDEX 0xFFFFFFFFu

const char* SpjMaterializeLastError(void);
/* out[i] = values[idx[i]] for fixed-width values of width 1, 2, 4, 8 or 16
 * bytes (Arrow primitive / fixed-size columns; a boolean column is gathered
 * by SpjGatherValidity over its value bits); a null index writes zero bytes. */
int SpjGatherFixed(const void* d_values, uint32_t width, uint64_t n_values,
                   const uint32_t* d_idx, uint64_t n, void* d_out, void* stream);
/* The validity bitmap of the gathered rows: bit i (LSB order, written as
 * 32-bit words, so d_out_bitmap holds ceil(n / 32) words and is 4-byte
 * aligned) is set when idx[i] is not null and the source row is valid (bit
 * validity_offset + idx[i] of d_validity; NULL = every row valid).
 * *null_count (host) receives the number of clear bits. */
int SpjGatherValidity(const uint8_t* d_validity, int64_t validity_offset, uint64_t n_values,
                      const uint32_t* d_idx, uint64_t n, uint8_t* d_out_bitmap,
                      uint64_t* null_count, void* stream);
/* Gather of a binary / utf8 column (WKB geometry included): source offsets
 * int32 (offsets_are_64bit = 0) or int64, n_values + 1 of them; output
 * offsets are int64 (n + 1 of them, large_binary layout, always written) and
 * the values' bytes go to d_out_data.  *out_bytes (host) receives the total;
 * when it exceeds capacity, only the offsets are written and ENOSPC is
 * returned.  Null indices give empty values. */
int SpjGatherBinary(const void* d_offsets, int32_t offsets_are_64bit, const uint8_t* d_data,
                    uint64_t n_values, const uint32_t* d_idx, uint64_t n,
                    int64_t* d_out_offsets, uint8_t* d_out_data, uint64_t capacity,
                    uint64_t* out_bytes, void* stream);
/* Set bit idx[i] of a row bitmap (ceil(n_rows / 32) 32-bit words, LSB
 * order, which is Arrow's bitmap layout on a little-endian machine; the
 * caller zeroes it once per build side).  Indices >= n_rows are skipped. */
int SpjVisitedMark(uint32_t* d_bitmap, uint64_t n_rows, const uint32_t* d_idx, uint64_t n,
                   void* stream);
/* The rows whose bit is set (visited = 1: semi joins) or clear (visited = 0:
 * left, left anti and full joins), ascending, into d_out_idx; *count (host)
 * receives how many; when it exceeds capacity nothing is written and ENOSPC
 * is returned.  A mark join reads the bitmap itself. */
int SpjVisitedCollect(const uint32_t* d_bitmap, uint64_t n_rows, int32_t visited,
                      uint32_t* d_out_idx, uint64_t capacity, uint64_t* count, void* stream);

/* ------------------------------------------------------------------------ */
/* Probe without allocating.  No counterpart in the reference interface.     */

/* Largest n_rects one SpjIndexProbeNoAlloc call accepts. */
#define SPJ_NOALLOC_MAX_PROBES (1u << 18)

/* The candidate filter of a built SedonaFloatIndex2D (the same pairs its
 * probe reports: every intersecting (build, probe) rect pair, in ascending
 * probe order) for callers that cannot allocate device memory at probe time,
 * e.g. an executor whose own arena holds the device memory budget, or a
 * latency-critical loop that must not touch the CUDA allocator.  Makes no
 * cudaMalloc / cudaFree and calls no allocating library routine: its scratch
 * is a 4 MiB static device array that every GPU loading the library keeps
 * until exit, which limits a call to SPJ_NOALLOC_MAX_PROBES rects (larger
 * n_rects is rejected with EINVAL and a message from get_last_error).
 * d_rects (n_rects x [min_x, min_y, max_x, max_y] float32), d_out_build and
 * d_out_probe (capacity entries each) are device pointers; *n_pairs (host)
 * receives the pair count, and if it exceeds capacity nothing is written and
 * ENOSPC is returned.  stream is a cudaStream_t (NULL = default stream); the
 * call synchronizes it.  The first call on a device looks up the static
 * array's device address (no allocation), so make it before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race
 * and must be serialized by the caller.  Before anything is launched the call
 * rejects (EINVAL + message) a d_rects that is not 16-byte aligned (each rect
 * is read as one 16-byte load), outputs that are not 4-byte aligned, and
 * buffers that are not device memory of the index's device.  A traversal
 * fault (a damaged tree) fails the call and stays recorded in the index:
 * every later probe of that index, through any entry point, fails with the
 * same message until the index is cleared and built again. */
int SpjIndexProbeNoAlloc(struct SedonaFloatIndex2D* index, const float* d_rects,
                         uint32_t n_rects, uint32_t* d_out_build, uint32_t* d_out_probe,
                         uint64_t capacity, uint64_t* n_pairs, void* stream);

/* ------------------------------------------------------------------------ */

/* Number of device (and page-locked host) buffers this library has
 * allocated since it was loaded, summed over all objects and devices.  A
 * caller can read it before and after a call to see that the call allocated
 * nothing. */
uint64_t SpjAllocationCount(void);

int SpjHostRegister(void* ptr, uint64_t bytes);
int SpjHostUnregister(void* ptr);
/* Library version string. */
const char* SpjVersion(void);

#ifdef __cplusplus
}
#endif
#endif
