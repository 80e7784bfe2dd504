// dwithin.cuh — ST_DWithin between point columns, decided inside the LBVH
// traversal: no candidate pairs are materialized.  The count pass and the
// scatter pass run the same deterministic test on every (build point, probe
// box) overlap the traversal finds, so the scatter writes exactly the counted
// pairs, grouped by probe row, in the same order as the filter + refine +
// compact path.
//
// Test per overlap: the FP32 distance of the (hi, lo) splits of both points
// (v = hi + lo, hi = RN32(v), lo = RN32(v - hi)), whose error is at most
// 2^-20 of the distance plus 2^-44 of the coordinate magnitude; a pair whose
// error interval lies entirely below or above the FP32 neighbours of d is
// decided, any other gets the exact correctly rounded hypot test.
#pragma once
#include "lbvh.cuh"

namespace spj {

// Build points in LBVH order: FP64, and FP32 (hi.x, hi.y, lo.x, lo.y).
struct PointSplit {
  uint32_t n = 0;
  float bmag = 0;  // max |x| + |y| over the points, rounded up
  bool ok = false; // every |coordinate| <= kSplitMaxCoord (FP32 squares stay finite)
  DevBuf xy, hl, tmp;
};
constexpr double kSplitMaxCoord = 1e18;

// pts: the build column's npts points (row order); bvh over their boxes.
void build_point_split(const double2* pts, uint32_t npts, const Lbvh& bvh, PointSplit& out,
                       cudaStream_t s);

// The two passes.  probe_box: the probe points' boxes expanded by d
// (expand_boxes); probe_pt: the probe points.  The count pass writes
// counts[probe row], keeps the first K build ids of each probe in
// slots[row * K ..] (slots may be null), and adds the escalations / overlaps
// tested to st->counters[0] / [1]; the scatter pass writes pairs at
// offs[probe row]: rows with <= K results by a coalesced copy of their slots,
// the others by traversing again.
// Overflow arena of the counting pass: a probe's results past its K slots
// go to chunks of kArenaChunkWords words (word 0: the next chunk, or
// kArenaEnd; then kArenaChunkWords - 1 build ids), taken with one atomic per
// chunk from *cursor.  head[probe] is its first chunk, kArenaEnd when it has
// none, or kArenaFailed when the arena ran out (that probe is traversed again
// by the scatter pass).
constexpr uint32_t kArenaChunkWords = 32;
constexpr uint32_t kArenaEnd = 0xFFFFFFFFu;
constexpr uint32_t kArenaFailed = 0xFFFFFFFEu;
struct DwithinArena {
  uint32_t* words = nullptr;
  uint32_t chunks = 0;
  unsigned long long* cursor = nullptr;  // 64-bit: failed takes never wrap it
  uint32_t* head = nullptr;
};

// d_row (device, one per probe row) replaces d when given.
void dwithin_count(const LbvhView& t, const PointSplit& bs, const float4* probe_box,
                   const double2* probe_pt, uint32_t n, double d, const uint32_t* order,
                   uint32_t* counts, DeviceStatus* st, cudaStream_t s, uint32_t* slots = nullptr,
                   uint32_t K = 0, DwithinArena arena = DwithinArena(),
                   const double* d_row = nullptr);
void dwithin_scatter(const LbvhView& t, const PointSplit& bs, const float4* probe_box,
                     const double2* probe_pt, uint32_t n, double d, const uint32_t* order,
                     const uint64_t* offs, uint32_t probe_base, uint32_t* out_build,
                     uint32_t* out_probe, uint64_t capacity, cudaStream_t s,
                     const uint32_t* counts = nullptr, const uint32_t* slots = nullptr,
                     uint32_t K = 0, DwithinArena arena = DwithinArena(),
                     const double* d_row = nullptr);

}  // namespace spj
