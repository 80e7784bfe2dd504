// engine.cuh — the join engine behind the C ABI: a decoded, indexed build
// side resident in HBM and a probe pipeline
//   decode probe WKB -> f32 filter boxes -> LBVH count / scan / scatter ->
//   refine (tg semantics or DWithin) -> scan / compact
// whose results stay on the device.  This is the GB300 counterpart of the
// reference's GPUSpatialIndex::query_batch
// (rust/sedona-spatial-join-gpu/src/index/gpu_spatial_index.rs:163-229), which
// runs RTSpatialIndex::Probe and RTSpatialRefiner::Refine back to back with
// host round trips in between.
#pragma once
#include <mutex>

#include "geoms.cuh"
#include "dwithin.cuh"
#include "lbvh.cuh"
#include "refine.cuh"

namespace spj {

constexpr int kPredDWithin = 100;  // ST_DWithin(build, probe, distance)

struct EngineConfig {
  // LBVH leaf size; 0 = by build side: 16 for point columns (ST_DWithin and
  // equality traversals test cheap points), 4 otherwise
  uint32_t leaf_size = 0;
  int refine_form = kFastF32;
  bool profile = false;  // time each phase with CUDA events on the engine stream
  // traversal order of the probe rows: 0 = Morton order from kOrderMinRows
  // rows up, 1 = always Morton order, -1 = row order
  int probe_order = 0;
  // point build and probe sides: decide ST_DWithin inside the traversal
  // (FAST_F32 form); otherwise filter, refine and compact
  bool fuse_dwithin = true;
  // fused ST_DWithin: build ids kept per probe by the counting pass (0 = none)
  uint32_t dwithin_slots = 64;
  // fused ST_DWithin: results past the slots go to an overflow arena of the
  // slots' size, so the scatter pass traverses only the probes the arena
  // could not hold (the 24 % of 20M GMM probes with over 64 neighbours hold
  // 80 % of the pairs).  0 off, 1 on, 2 auto: on when the probes are not in
  // Morton order.  20M x 1M GMM points: in row order 297 -> 139 ms per step;
  // in Morton order the counting pass slowed from 38 to 103 ms with it (the
  // scatter pass fell from 33 to 9 ms), so auto leaves it off there
  int dwithin_arena = 2;
  // refine order of the candidates: 0 as listed (by probe row), 2 by build
  // row then probe Morton rank (a warp then tests one build geometry's edges
  // against neighbouring probes: shared loads and similar trip counts; 2M x
  // 50k polygons: 77 vs 104 ms per step), 3 auto: 2 for relation predicates
  // over a build side that is not all points, from kBuildMajorMin candidates
  // up, else 0.  (The probes' Morton order and a band-and-x order inside the
  // build ring measured slower on every workload and were removed.)
  int candidate_order = 3;
  // build-major order within tiles of the probes' Morton-ordered candidate
  // list: -1 auto (tiles of kOrderTileCandidates), n >= 0: 2^n tiles.  A
  // tile's probe rows stay in cache while the refine passes its build rows
  // (2M x 50k polygons: 45.4 ms per step in one tile, 41.8 with 64 tiles,
  // 40.9 with 256-1024)
  int order_tiles = -1;
  // FP32 refine compiled for this many resident 256-thread blocks per SM
  // (4 or 6), or 0 auto: 6 for ST_Intersects / ST_Disjoint in build-major
  // candidate order (a warp's pairs share one build geometry, and more
  // resident warps hide its load latency better than registers do: 2M x
  // 50k polygons 41.0 vs 43.4 ms), else 4 (the containment and touch tests'
  // deeper calls want the registers: ST_Contains on the same inputs 77.1 vs
  // 78.3 ms; 10M points x 50k zones: 96.7 vs 99.4 ms with 6)
  int refine_min_blocks = 0;
  // per-ring cell grids on the build side (clean cells answer point-in-ring
  // tests in O(1)); set before the build
  bool cell_grid = true;
  // ring-ring and ring-in-ring tests answer from the build ring's clean cells
  // when the probe ring's box lies in them (2M buildings x 50k star zones:
  // 63.0 ms per step with it, 52.7 without: the zones' spiky edges leave few
  // buildings inside clean cells, and the lookup costs every pair)
  bool grid_rings = false;
  // FP32 refine in two passes: a cheap pass (isolation exit, first vertex)
  // over every pair queues the pairs it leaves open, a full pass takes the
  // queue (a warp's lanes then hold pairs of similar cost).  0 off, 1 on,
  // 2 auto: on unless the candidates are in build-major order, where a
  // warp's pairs already share one build geometry (2M x 50k polygons: 59.0
  // ms one pass vs 61.0 split in build-major order; 78.0 vs 63.3 as listed);
  // 3 on, with the open pairs' queue sorted back into candidate order
  int refine_split = 2;
  // host probes (SpjJoinProbeHost): 0 auto (2 slices from 524,288 rows up),
  // 1 one call, n > 1 that many slices
  int host_slices = 0;
};
constexpr uint32_t kOrderMinRows = 1u << 16;
constexpr uint64_t kBuildMajorMin = 1ull << 22;  // candidates before build-major order pays
constexpr uint64_t kOrderTileCandidates = 1ull << 19;  // auto order_tiles: candidates per tile

// order_tiles as configured, resolved to a tile count for m candidates
inline uint64_t order_tile_count(int configured, uint64_t m) {
  if (configured >= 0) return 1ull << configured;
  return m / kOrderTileCandidates > 1 ? m / kOrderTileCandidates : 1;
}

// refine_min_blocks as configured, with 0 (auto) resolved by the candidate order and
// the predicate (intersects: ST_Intersects or ST_Disjoint)
inline int refine_blocks(int configured, bool build_major, bool intersects = true) {
  return configured ? configured : (build_major && intersects ? 6 : 4);
}
constexpr uint64_t kMaxSlotBytes = 8ull << 30;  // cap of the fused ST_DWithin slot buffer

// Per-phase device time (CUDA events on the launching stream) and counters.
struct JoinStats {
  double ms_decode = 0, ms_filter = 0, ms_refine = 0, ms_compact = 0;
  uint64_t calls = 0;
  uint64_t probe_rows = 0;
  uint64_t candidates = 0;
  uint64_t results = 0;
  uint64_t escalations = 0;  // segment / distance tests decided in FP64
  uint64_t pairs_evaluated = 0;
  uint64_t kernel_launches = 0;
  uint64_t probe_bytes = 0;  // WKB + offsets bytes of the probe columns
};

// Per-call scratch; one per concurrent caller.
struct Workspace {
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  DeviceGeoms probe;
  DecodeScratch dsc;
  ProbeScratch psc;
  DevBuf boxes_tmp, cand_build, cand_probe, flags, out_build, out_probe, scan_tmp, status;
  DevBuf slots;   // fused ST_DWithin result slots
  DevBuf arena;   // fused ST_DWithin overflow arena: cursor, heads, chunks
  DevBuf rqueue;  // pairs left open by the refine's cheap pass, then its count
  DevBuf wkb_data, wkb_offsets, wkb_validity;  // H2D staging of host columns
  cudaEvent_t ev[6] = {};
  bool last_probe_points = true;
  Workspace();
  ~Workspace();
};

class JoinEngine {
 public:
  JoinEngine(int device, EngineConfig cfg);
  ~JoinEngine();

  int device() const { return device_; }
  EngineConfig& config() { return cfg_; }

  // Build side from a device WKB column (decoded, boxed, indexed, banded),
  // on the engine's own stream; the column must be complete on the device
  // (the caller has synchronized whatever stream wrote it).
  void build(const WkbDeviceColumn& col);
  bool built() const { return built_; }
  // Rebuild the LBVH over the decoded build boxes with another leaf size.
  void reindex(uint32_t leaf_size);
  const DeviceGeoms& build_geoms() const { return bg_; }
  void set_grid_rings(bool on) { bg_.grid_rings = on; }
  const Lbvh& lbvh() const { return bvh_; }

  // Probe with a device WKB column.  Results (device pointers owned by the
  // workspace, valid until its next call) are grouped by probe row in
  // ascending probe order; probe ids are offset by probe_base.
  // d_row (device, one per probe row): ST_DWithin distances per row; a
  // negative or NaN distance matches nothing.
  uint64_t probe(Workspace& ws, const WkbDeviceColumn& col, int predicate, double distance,
                 uint32_t probe_base, const uint32_t** d_build, const uint32_t** d_probe,
                 const double* d_row = nullptr);

  // Refine caller-supplied candidate pairs (device arrays) against an
  // already decoded probe column; output compacted into ws.out_*.
  uint64_t refine_pairs(Workspace& ws, const GeomsView& probe, const uint32_t* cb,
                        const uint32_t* cp, uint64_t m, int predicate, double distance);

  JoinStats stats();
  void reset_stats();

 private:
  void split_points();
  int device_;
  EngineConfig cfg_;
  DeviceGeoms bg_;
  DecodeScratch bsc_;
  Lbvh bvh_;
  PointSplit bsplit_;  // point build sides: ST_DWithin decided in the traversal
  cudaStream_t bs_ = nullptr;  // build stream; owns the frees of bg_/bsc_/bvh_
  bool built_ = false;
  std::mutex stats_mu_;
  JoinStats stats_;
};

// Host Arrow binary column view (after the Arrow C data interface is parsed).
struct HostWkbColumn {
  int64_t n = 0;
  const void* offsets = nullptr;  // int32 or int64, n+1 entries (absolute into data)
  bool offsets64 = false;
  const uint8_t* data = nullptr;
  const uint8_t* validity = nullptr;
  int64_t validity_offset = 0;
};

// Copies a host column into the workspace staging buffers (H2D on ws.stream)
// and returns the device view.  Returns the bytes copied in *bytes.
WkbDeviceColumn stage_column(Workspace& ws, const HostWkbColumn& col, uint64_t* bytes);

}  // namespace spj
