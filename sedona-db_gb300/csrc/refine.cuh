// refine.cuh — candidate-pair refinement kernels (relation predicates,
// ST_DWithin) and flag compaction.
#pragma once
#include "geoms.cuh"

namespace spj {

// Predicate codes: enum SedonaSpatialRelationPredicate order
// (c/sedona-libgpuspatial/libgpuspatial/include/gpuspatial/gpuspatial_c.h:142-151).
enum Predicate : int {
  kEquals = 0,
  kDisjoint = 1,
  kTouches = 2,
  kContains = 3,
  kCovers = 4,
  kIntersects = 5,
  kWithin = 6,
  kCoveredBy = 7,
};

enum RefineForm : int {
  kPlainF64 = 0,  // every segment test through the FP64 sequence, no band index
  kFastF32 = 1,   // y-band index + FP32 classification + FP64 escalation
};

// flags[k] = pred(build[cb[k]], probe[cp[k] - probe_base]) for k < m.
// counters: status->counters[0] += FP64 escalations, [1] += pairs evaluated.
// With m_dev the pair count is read on the device (CUDA-graph replays) and m
// is the capacity of cb/cp/flags; flags past the count are cleared.  With
// perm (a permutation of [0, m)), candidates are evaluated in that order
// (flags still land at their own index); with perm and m_dev together, perm
// is a permutation of [0, *m_dev) and the caller clears the flags past it.
// min_blocks (4 or 6) selects the FP32 form compiled for that many resident
// 256-thread blocks per SM: fewer registers, more warps to hide the latency
// of divergent pairs.  queue (m entries) and qn (one device word) split the
// FP32 refine into a cheap pass over all pairs that queues the pairs it
// cannot decide, then a full pass over the queue (ordered_queue: sorted back
// into perm's order first); same flags.
void refine_relation(const GeomsView& build, const GeomsView& probe, const uint32_t* cb,
                     const uint32_t* cp, uint64_t m, uint32_t probe_base, int predicate, int form,
                     uint8_t* flags, DeviceStatus* st, cudaStream_t s,
                     const uint64_t* m_dev = nullptr, const uint32_t* perm = nullptr,
                     int min_blocks = 4, uint32_t* queue = nullptr, uint32_t* qn = nullptr,
                     bool ordered_queue = false);

// flags[k] = distance(build, probe) <= d.  Point pairs: hypot, decided by an
// FP64 squared-distance test outside a 1e-14 relative band around d^2 and by
// expansion arithmetic inside it.  Pairs with a polygon: the reference's
// FP64 distance (distance.cuh).  d is one value, or with d_row (device, one
// per probe row, indexed by probe id - probe_base) the probe row's; a
// negative or NaN distance keeps nothing.  Both forms run the same code.
void refine_dwithin(const GeomsView& build, const GeomsView& probe, const uint32_t* cb,
                    const uint32_t* cp, uint64_t m, uint32_t probe_base, double distance, int form,
                    uint8_t* flags, DeviceStatus* st, cudaStream_t s,
                    const uint32_t* perm = nullptr, const double* d_row = nullptr);

}  // namespace spj
