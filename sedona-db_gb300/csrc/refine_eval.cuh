// refine_eval.cuh — the device side of the relation-predicate refine: tg
// dispatch per predicate (one lane per pair) and the refine kernels.
// Included by the translation units that launch them (refine.cu,
// refine_split.cu, refine_blocks.cu), which compile in parallel; each gets
// its own copy of the kernels it instantiates.
#pragma once
#include "exact.cuh"
#include "predicates.cuh"
#include "prims.cuh"
#include "refine.cuh"
#include "relate.cuh"

#include <cmath>

namespace spj {
namespace {


using namespace pred;
using exact::dwithin_exact;

constexpr int kUnsupportedResult = -1;

// RN32 coordinates of a point row: the decoder stores them as its degenerate
// filter box (x, y, x, y), so no f64 -> f32 conversion is needed here.
__device__ __forceinline__ float2 pt32(const GeomsView& G, uint32_t i) {
  const float4 b = G.box[i];
  return make_float2(b.x, b.y);
}

__device__ __forceinline__ uint32_t nparts(const GeomsView& G, uint32_t i) {
  return G.row_part[i + 1] - G.row_part[i];
}

// tg.c:5740-5760 intersects dispatch.  kCheap: ring pairs may come back
// kDeferred (see ring_intersects_ring); the pair is then deferred unless
// another ring pair already decides it true.  Parts with holes take tg's
// polygon path (relate.cuh).
template <bool kFast, bool kCheap = false>
__device__ int g_intersects(const GeomsView& GA, uint32_t ia, const GeomsView& GB, uint32_t ib,
                            uint32_t& esc) {
  const uint8_t ka = GA.kind[ia], kb = GB.kind[ib];
  if (ka == kEmpty || kb == kEmpty) return 0;
  if (ka == kPoint && kb == kPoint) return pteq(GA.pt[ia], GB.pt[ib]);
  if (ka == kPoint || kb == kPoint) {
    const GeomsView& GP = ka == kPoint ? GA : GB;  // the point
    const GeomsView& GY = ka == kPoint ? GB : GA;  // the polygonal side
    const uint32_t ip = ka == kPoint ? ia : ib, iy = ka == kPoint ? ib : ia;
    const double2 p = GP.pt[ip];
    const float2 p32 = pt32(GP, ip);
    for (uint32_t q = GY.row_part[iy]; q < GY.row_part[iy + 1]; q++)
      if (poly_contains_point<kFast>(GY, q, p, p32, true, esc)) return 1;
    return 0;
  }
  bool deferred = false;
  for (uint32_t qa = GA.row_part[ia]; qa < GA.row_part[ia + 1]; qa++) {
    const uint32_t ra = GA.part_ring[qa];
    const bool sa = GA.part_ring[qa + 1] - ra == 1;
    for (uint32_t qb = GB.row_part[ib]; qb < GB.row_part[ib + 1]; qb++) {
      const uint32_t rb = GB.part_ring[qb];
      const bool sb = GB.part_ring[qb + 1] - rb == 1;
      if (!(sa && sb)) {
        if (poly_intersects_poly<kFast>(GA, qa, GB, qb, esc)) return 1;
        continue;
      }
      const int r = ring_intersects_ring<kFast, kCheap>(GA, ra, GB, rb, esc);
      if (r == 1) return 1;
      if (r == kDeferred) deferred = true;
    }
  }
  return deferred ? kDeferred : 0;
}

// tg.c:6538-6556 contains dispatch (point 'other' cases)
template <bool kFast>
__device__ int g_contains(const GeomsView& GA, uint32_t ia, const GeomsView& GB, uint32_t ib,
                          uint32_t& esc) {
  const uint8_t ka = GA.kind[ia], kb = GB.kind[ib];
  if (ka == kEmpty || kb == kEmpty) return 0;
  if (ka == kPoint && kb == kPoint) return pteq(GA.pt[ia], GB.pt[ib]);
  if (ka == kPoint) return 0;  // tg.c:1157-1162
  if (kb == kPoint) {
    const double2 p = GB.pt[ib];
    const float2 p32 = pt32(GB, ib);
    for (uint32_t q = GA.row_part[ia]; q < GA.row_part[ia + 1]; q++)
      if (poly_contains_point<kFast>(GA, q, p, p32, false, esc)) return 1;
    return 0;
  }
  return row_contains_rows<kFast>(GA, ia, GB, ib, esc);
}

// tg.c:6028-6046 covers dispatch
template <bool kFast>
__device__ int g_covers(const GeomsView& GA, uint32_t ia, const GeomsView& GB, uint32_t ib,
                        uint32_t& esc) {
  const uint8_t ka = GA.kind[ia], kb = GB.kind[ib];
  if (ka == kEmpty || kb == kEmpty) return 0;
  if (ka == kPoint && kb == kPoint) return pteq(GA.pt[ia], GB.pt[ib]);
  if (kb == kPoint) {
    const double2 p = GB.pt[ib];
    const float2 p32 = pt32(GB, ib);
    for (uint32_t q = GA.row_part[ia]; q < GA.row_part[ia + 1]; q++)
      if (poly_contains_point<kFast>(GA, q, p, p32, true, esc)) return 1;
    return 0;
  }
  if (ka == kPoint) {
    // tg.c:1152-1155 per part: the part's rect is the point itself (every
    // part; an empty part of a multipolygon fails, tg.c:5770-5795)
    if (has_empty_parts(GB, ib)) return 0;
    const double2 p = GA.pt[ia];
    for (uint32_t q = GB.row_part[ib]; q < GB.row_part[ib + 1]; q++) {
      const uint32_t r = GB.part_ring[q];
      if (ring_npts(GB, r) < 3) return 0;
      const Rect64 R = GB.ring_rect[r];
      if (!(pteq(p, make_double2(R.x, R.y)) && pteq(p, make_double2(R.z, R.w)))) return 0;
    }
    return 1;
  }
  return row_covers_rows<kFast>(GA, ia, GB, ib, esc);
}

// tg.c:6771-6789 touches dispatch
template <bool kFast>
__device__ int g_touches(const GeomsView& GA, uint32_t ia, const GeomsView& GB, uint32_t ib,
                         uint32_t& esc) {
  const uint8_t ka = GA.kind[ia], kb = GB.kind[ib];
  if (ka == kEmpty || kb == kEmpty) return 0;
  if (ka == kPoint && kb == kPoint) return 0;
  if (ka == kPolygon && kb == kPoint) {
    const double2 p = GB.pt[ib];
    return poly_touches_point<kFast>(GA, GA.row_part[ia], p, pt32(GB, ib), esc);
  }
  if (ka == kPoint) {
    // tg_point_touches_poly per part, any part (tg.c:6575-6625)
    const double2 p = GA.pt[ia];
    for (uint32_t q = GB.row_part[ib]; q < GB.row_part[ib + 1]; q++)
      if (poly_touches_point<kFast>(GB, q, p, pt32(GA, ia), esc)) return 1;
    return 0;
  }
  return row_touches_row<kFast>(GA, ia, GB, ib, esc);
}

template <bool kFast, bool kCheap = false>
__device__ int eval(const GeomsView& B, uint32_t b, const GeomsView& P, uint32_t p, int predicate,
                    uint32_t& esc) {
  switch (predicate) {
    case kIntersects:
      return g_intersects<kFast, kCheap>(B, b, P, p, esc);
    case kDisjoint: {
      const int r = g_intersects<kFast, kCheap>(B, b, P, p, esc);
      return r == kDeferred ? r : !r;
    }
    case kContains:
      return g_contains<kFast>(B, b, P, p, esc);
    case kWithin:
      return g_contains<kFast>(P, p, B, b, esc);
    case kCovers:
      return g_covers<kFast>(B, b, P, p, esc);
    case kCoveredBy:
      return g_covers<kFast>(P, p, B, b, esc);
    case kTouches:
      return g_touches<kFast>(B, b, P, p, esc);
    case kEquals: {
      int w = g_contains<kFast>(P, p, B, b, esc);
      if (w <= 0) return w;
      return g_contains<kFast>(B, b, P, p, esc);
    }
  }
  return kUnsupportedResult;
}

__device__ __forceinline__ void flush_counters(DeviceStatus* st, uint32_t esc, uint32_t pairs) {
  // warp-aggregate, one atomic per warp
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    esc += __shfl_xor_sync(0xffffffffu, esc, o);
    pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (esc) atomicAdd(&st->counters[0], (unsigned long long)esc);
    if (pairs) atomicAdd(&st->counters[1], (unsigned long long)pairs);
  }
}

// With perm, thread slot u evaluates candidate perm[u] (a permutation that
// puts spatially neighbouring probes' candidates next to each other) and
// writes its flag in place.  kMinBlocks trades registers for occupancy.
//
// kPhase 0: every pair in full.  kPhase 1 (FP32 form): the cheap tier only;
// pairs it leaves undecided are appended to queue (count in *qn) with no
// flag written.  kPhase 2: the queued pairs (slots u < *qn of queue, used as
// perm) in full.  Splitting the work this way keeps a warp's lanes on pairs
// of similar cost: a few pairs near a zone's edges take ten times the steps
// of an isolated one, and would otherwise hold 31 idle lanes.
template <bool kFast, int kMinBlocks, int kPhase = 0>
__global__ void __launch_bounds__(256, kMinBlocks)
    k_refine(GeomsView B, GeomsView P, const uint32_t* __restrict__ cb,
             const uint32_t* __restrict__ cp, uint64_t m, uint32_t probe_base, int predicate,
             uint8_t* __restrict__ flags, DeviceStatus* st, const uint64_t* __restrict__ m_dev,
             const uint32_t* __restrict__ perm, uint32_t* __restrict__ queue = nullptr,
             uint32_t* __restrict__ qn = nullptr,
             const uint32_t* __restrict__ slot_perm = nullptr, uint32_t chunk_trips = 0) {
  // slot_perm (the split refine with an ordered queue): phase 1 queues the
  // slots u of perm instead of the candidates (the host sorts them), and
  // phase 2 maps a queued slot back through slot_perm
  uint32_t esc = 0, pairs = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // with m_dev the pair count lives on the device (graph replays) and m is
  // the buffer capacity: flags past the count are cleared
  const uint64_t mm = m_dev ? min(*m_dev, m) : m;
  // every lane runs the same number of loop trips so the warp-wide flush
  // below sees all 32 lanes
  // chunk_trips > 0: each block takes chunk_trips consecutive runs of
  // blockDim.x slots (kRefineChunkTrips); 0: the grid strides over all slots
  // (the stream graph, whose pair count lives on the device)
  const uint64_t start = chunk_trips
                             ? blockIdx.x * (uint64_t)blockDim.x * chunk_trips + threadIdx.x
                             : blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t step = chunk_trips ? (uint64_t)blockDim.x : stride;
  const uint64_t trips = chunk_trips ? chunk_trips : (m + stride - 1) / stride;
  const uint64_t nq = kPhase == 2 ? min((uint64_t)*qn, m) : 0;
  for (uint64_t t = 0; t < trips; t++) {
    const uint64_t u = start + t * step;
    if (u >= m) continue;
    if (kPhase == 2 && u >= nq) continue;
    // a permutation with a device-side count covers slots [0, mm) only (the
    // caller clears the flags past mm)
    if (kPhase != 2 && perm != nullptr && m_dev != nullptr && u >= mm) continue;
    uint64_t k = perm ? (uint64_t)perm[u] : u;
    if (kPhase == 2 && slot_perm != nullptr) k = k < m ? (uint64_t)slot_perm[k] : ~0ull;
    if (k >= mm) {
      if (kPhase != 2 && k < m) flags[k] = 0;
      continue;
    }
    const uint32_t b = cb[k], p = cp[k] - probe_base;
    int r = eval<kFast, kPhase == 1>(B, b, P, p, predicate, esc);
    if (kPhase == 1 && r == kDeferred) {
      // one atomic per group of lanes that reach this point together
      const unsigned act = __activemask();
      const int lane = threadIdx.x & 31, leader = __ffs(act) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(qn, (uint32_t)__popc(act));
      base = __shfl_sync(act, base, leader);
      queue[base + __popc(act & ((1u << lane) - 1u))] = slot_perm ? (uint32_t)u : (uint32_t)k;
      continue;
    }
    pairs++;
    if (r < 0) {
      status_fail(st, kUnsupported, k);
      r = 0;
    }
    flags[k] = (uint8_t)r;
  }
  flush_counters(st, esc, pairs);
}

}  // namespace

// Launch parameters shared by the refine launchers.
struct RefineLaunch {
  GeomsView build, probe;
  const uint32_t *cb, *cp;
  uint64_t m;
  uint32_t probe_base;
  int predicate;
  uint8_t* flags;
  DeviceStatus* st;
  const uint64_t* m_dev;
  const uint32_t* perm;
  uint32_t *queue, *qn;
  cudaStream_t s;
};

// The one-pass refine kernels give each block kRefineChunkTrips consecutive
// runs of 256 pairs: consecutive pairs share build rows (and, in probe
// order, neighbouring probes), whose band entries and vertices then stay in
// the SM's L1 from one trip to the next.  On the 2M x 50k polygon join the
// refine step measured 49.6 ms with the grid striding over all pairs, 46.2 /
// 45.4 / 45.2 / 45.5 ms with 1 / 2 / 4 / 8 runs per block.
constexpr uint32_t kRefineChunkTrips = 4;
inline unsigned refine_grid(uint64_t m, uint32_t trips) {
  if (trips == 0) return (unsigned)grid_for((int64_t)m, 256, kNumSMs * 16);
  const uint64_t per = 256ull * trips;
  const uint64_t g = (m + per - 1) / per;
  return (unsigned)(g ? g : 1);
}
// refine_split.cu: the cheap pass then the full pass over its queue
// (min_blocks 4 or 6); ordered (with a perm): the queue is sorted back into
// the perm's order before the full pass
void launch_refine_split(const RefineLaunch& a, int min_blocks, bool ordered = false);
// refine_blocks.cu: one pass, FP32 form built for 6 resident blocks per SM
void launch_refine_blocks6(const RefineLaunch& a);

}  // namespace spj
