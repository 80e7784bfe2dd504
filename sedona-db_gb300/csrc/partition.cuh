// partition.cuh — partitioned (out-of-core) spatial join: the build side is
// split into spatial partitions that are indexed one at a time, so a build
// side larger than the device's memory joins in passes, with both columns
// left in host memory.
//
// The partitioning follows the reference's out-of-core join
// (rust/sedona-spatial-join/src/prepare.rs:260-340): a KDB tree built from a
// sample of build boxes (partitioning/kdb.rs:116-459; max items per node =
// samples / partitions, at most `partitions` levels) assigns every build row
// to the leaf it overlaps most (partition_no_multi, kdb.rs:542-566); each
// probe row goes to the one partition whose build rows' bounds it meets, to
// all of them when it meets several (Multi), or to none
// (FlatPartitioner::partition over the partitions' actual bounds,
// partitioning/flat.rs:55-77).  A pass k joins partition k's build rows with
// the probe rows of partition k and of Multi.  A pair (b, p) whose boxes meet
// is found exactly once: in b's partition, whose bounds contain b's box and
// so meet p's.
#pragma once
#include <functional>
#include <vector>

#include "engine.cuh"

namespace spj {

struct PartitionOptions {
  uint32_t num_partitions = 0;    // target KDB leaves; 0: from build_budget_bytes
  uint32_t sample_rows = 0;       // build boxes sampled for the tree (0: 10,000)
  uint64_t build_budget_bytes = 0;  // device bytes per partition's build side (0: one)
  uint64_t seed = 0;
  bool host_gather = false;       // stage each pass's rows on the host
  bool record_layout = false;     // copy every row's partition to the layout
};

struct PartitionStats {
  uint32_t partitions = 0, passes = 0;
  uint64_t build_rows_max = 0;
  uint64_t probe_rows_multi = 0, probe_rows_none = 0, probe_rows_probed = 0;
  uint64_t pairs = 0;
  double ms_boxes = 0, ms_partition = 0, ms_passes = 0;
  bool direct_host_reads = false;
};

// The last run's partitioning, for checks against the reference's rules.
struct PartitionLayout {
  std::vector<float4> samples;       // the sampled build boxes, in insertion order
  float4 extent{};                   // the build boxes' union
  uint32_t max_items = 0, max_levels = 0;
  std::vector<float4> leaves;        // KDB leaf extents by leaf id
  std::vector<float4> bounds;        // per partition: union of its build boxes
  std::vector<uint32_t> build_part;  // per build row: leaf id, or 0xFFFFFFFF
  std::vector<uint32_t> probe_part;  // per probe row: leaf id, leaves = Multi, leaves+1 = None
};

// Runs the join in passes; every pass's pairs (global row ids, grouped by
// probe row within its Regular and Multi groups) go to sink, which returns
// non-zero to stop (that value is returned).  d_dist: ST_DWithin distance
// column on the device (one per probe row) or null.
using PairSink = std::function<int(const uint32_t* build, const uint32_t* probe, uint64_t n)>;
int run_partitioned(JoinEngine& eng, Workspace& ws, const HostWkbColumn& build,
                    const HostWkbColumn& probe, int predicate, double distance,
                    const double* d_dist, const PartitionOptions& opt, PartitionStats* stats,
                    PartitionLayout* layout, const PairSink& sink);

}  // namespace spj
