// refine.cu — relation-predicate and ST_DWithin refinement of candidate
// pairs, one thread per candidate, plus order-preserving compaction.
//
// Replaces the reference's RTSpatialRefiner::Refine
// (c/sedona-libgpuspatial/libgpuspatial/src/rt_spatial_refiner.cu:134-242),
// which re-parses probe WKB on the CPU each call and runs OptiX PIP
// (src/rt/shaders/polygon_point_query.cu) or a recursive DE-9IM relate
// (src/relate_engine.cu:294-336).  Here both sides are already decoded in HBM
// and the predicate is the tg semantics the reference CPU join uses.
#include "exact.cuh"
#include "predicates.cuh"
#include "prims.cuh"
#include "refine.cuh"

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

// tg.c:5740-5760 intersects dispatch
template <bool kFast>
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
  bool unsupported = false;
  for (uint32_t qa = GA.row_part[ia]; qa < GA.row_part[ia + 1]; qa++) {
    const uint32_t ra = GA.part_ring[qa];
    const bool sa = GA.part_ring[qa + 1] - ra == 1;
    for (uint32_t qb = GB.row_part[ib]; qb < GB.row_part[ib + 1]; qb++) {
      const uint32_t rb = GB.part_ring[qb];
      const bool sb = GB.part_ring[qb + 1] - rb == 1;
      if (!(sa && sb)) {
        unsupported = true;
        continue;
      }
      if (ring_intersects_ring<kFast>(GA, ra, GB, rb, esc)) return 1;
    }
  }
  return unsupported ? kUnsupportedResult : 0;
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
  return kUnsupportedResult;
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
  if (ka == kPoint && kb == kPolygon) {
    // tg.c:1152-1155: the polygon's rect is the point itself
    const uint32_t r = GB.part_ring[GB.row_part[ib]];
    if (ring_npts(GB, r) < 3) return 0;
    const Rect64 R = GB.ring_rect[r];
    const double2 p = GA.pt[ia];
    return pteq(p, make_double2(R.x, R.y)) && pteq(p, make_double2(R.z, R.w));
  }
  return kUnsupportedResult;
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
  if (ka == kPoint && kb == kPolygon) {
    const double2 p = GA.pt[ia];
    return poly_touches_point<kFast>(GB, GB.row_part[ib], p, pt32(GA, ia), esc);
  }
  return kUnsupportedResult;
}

template <bool kFast>
__device__ int eval(const GeomsView& B, uint32_t b, const GeomsView& P, uint32_t p, int predicate,
                    uint32_t& esc) {
  switch (predicate) {
    case kIntersects:
      return g_intersects<kFast>(B, b, P, p, esc);
    case kDisjoint: {
      int r = g_intersects<kFast>(B, b, P, p, esc);
      return r < 0 ? r : !r;
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

// --- group-cooperative dispatch (FP32 form): kG lanes per pair -------------
// Mirrors g_intersects / g_contains / g_covers / eval above, with the ring
// loops split across the group (predicates.cuh); touches runs the
// sequential code in every lane (same inputs, same answer).

template <int kG>
__device__ int g_intersects_group(const GeomsView& GA, uint32_t ia, const GeomsView& GB,
                                  uint32_t ib, uint32_t& esc, unsigned gm, int gl) {
  const uint8_t ka = GA.kind[ia], kb = GB.kind[ib];
  if (ka == kEmpty || kb == kEmpty) return 0;
  if (ka == kPoint && kb == kPoint) return pteq(GA.pt[ia], GB.pt[ib]);
  if (ka == kPoint || kb == kPoint) {
    const GeomsView& GP = ka == kPoint ? GA : GB;
    const GeomsView& GY = ka == kPoint ? GB : GA;
    const uint32_t ip = ka == kPoint ? ia : ib, iy = ka == kPoint ? ib : ia;
    const double2 p = GP.pt[ip];
    const float2 p32 = pt32(GP, ip);
    for (uint32_t q = GY.row_part[iy]; q < GY.row_part[iy + 1]; q++)
      if (poly_contains_point_group<kG>(GY, q, p, p32, true, esc, gm, gl)) return 1;
    return 0;
  }
  bool unsupported = false;
  for (uint32_t qa = GA.row_part[ia]; qa < GA.row_part[ia + 1]; qa++) {
    const uint32_t ra = GA.part_ring[qa];
    const bool sa = GA.part_ring[qa + 1] - ra == 1;
    for (uint32_t qb = GB.row_part[ib]; qb < GB.row_part[ib + 1]; qb++) {
      const uint32_t rb = GB.part_ring[qb];
      const bool sb = GB.part_ring[qb + 1] - rb == 1;
      if (!(sa && sb)) {
        unsupported = true;
        continue;
      }
      if (ring_intersects_ring_group<kG>(GA, ra, GB, rb, esc, gm, gl)) return 1;
    }
  }
  return unsupported ? kUnsupportedResult : 0;
}

template <int kG>
__device__ int g_contains_group(const GeomsView& GA, uint32_t ia, const GeomsView& GB, uint32_t ib,
                                uint32_t& esc, unsigned gm, int gl) {
  const uint8_t ka = GA.kind[ia], kb = GB.kind[ib];
  if (ka == kEmpty || kb == kEmpty) return 0;
  if (ka == kPoint && kb == kPoint) return pteq(GA.pt[ia], GB.pt[ib]);
  if (ka == kPoint) return 0;
  if (kb == kPoint) {
    const double2 p = GB.pt[ib];
    const float2 p32 = pt32(GB, ib);
    for (uint32_t q = GA.row_part[ia]; q < GA.row_part[ia + 1]; q++)
      if (poly_contains_point_group<kG>(GA, q, p, p32, false, esc, gm, gl)) return 1;
    return 0;
  }
  return kUnsupportedResult;
}

template <int kG>
__device__ int g_covers_group(const GeomsView& GA, uint32_t ia, const GeomsView& GB, uint32_t ib,
                              uint32_t& esc, unsigned gm, int gl) {
  const uint8_t ka = GA.kind[ia], kb = GB.kind[ib];
  if (ka == kEmpty || kb == kEmpty) return 0;
  if (ka == kPoint && kb == kPoint) return pteq(GA.pt[ia], GB.pt[ib]);
  if (kb == kPoint) {
    const double2 p = GB.pt[ib];
    const float2 p32 = pt32(GB, ib);
    for (uint32_t q = GA.row_part[ia]; q < GA.row_part[ia + 1]; q++)
      if (poly_contains_point_group<kG>(GA, q, p, p32, true, esc, gm, gl)) return 1;
    return 0;
  }
  return g_covers<true>(GA, ia, GB, ib, esc);  // point covering a polygon: no ring loops
}

template <int kG>
__device__ int eval_group(const GeomsView& B, uint32_t b, const GeomsView& P, uint32_t p,
                          int predicate, uint32_t& esc, unsigned gm, int gl) {
  switch (predicate) {
    case kIntersects:
      return g_intersects_group<kG>(B, b, P, p, esc, gm, gl);
    case kDisjoint: {
      const int r = g_intersects_group<kG>(B, b, P, p, esc, gm, gl);
      return r < 0 ? r : !r;
    }
    case kContains:
      return g_contains_group<kG>(B, b, P, p, esc, gm, gl);
    case kWithin:
      return g_contains_group<kG>(P, p, B, b, esc, gm, gl);
    case kCovers:
      return g_covers_group<kG>(B, b, P, p, esc, gm, gl);
    case kCoveredBy:
      return g_covers_group<kG>(P, p, B, b, esc, gm, gl);
    case kTouches:
      return g_touches<true>(B, b, P, p, esc);
    case kEquals: {
      const int w = g_contains_group<kG>(P, p, B, b, esc, gm, gl);
      if (w <= 0) return w;
      return g_contains_group<kG>(B, b, P, p, esc, gm, gl);
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
template <bool kFast, int kMinBlocks>
__global__ void __launch_bounds__(256, kMinBlocks)
    k_refine(GeomsView B, GeomsView P, const uint32_t* __restrict__ cb,
             const uint32_t* __restrict__ cp, uint64_t m, uint32_t probe_base, int predicate,
             uint8_t* __restrict__ flags, DeviceStatus* st, const uint64_t* __restrict__ m_dev,
             const uint32_t* __restrict__ perm) {
  uint32_t esc = 0, pairs = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // with m_dev the pair count lives on the device (graph replays) and m is
  // the buffer capacity: flags past the count are cleared
  const uint64_t mm = m_dev ? min(*m_dev, m) : m;
  // every lane runs the same number of loop trips so the warp-wide flush
  // below sees all 32 lanes
  const uint64_t start = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t trips = (m + stride - 1) / stride;
  for (uint64_t t = 0; t < trips; t++) {
    const uint64_t u = start + t * stride;
    if (u >= m) continue;
    const uint64_t k = perm ? (uint64_t)perm[u] : u;
    if (k >= mm) {
      if (k < m) flags[k] = 0;
      continue;
    }
    const uint32_t b = cb[k], p = cp[k] - probe_base;
    int r = eval<kFast>(B, b, P, p, predicate, esc);
    pairs++;
    if (r < 0) {
      status_fail(st, kUnsupported, k);
      r = 0;
    }
    flags[k] = (uint8_t)r;
  }
  flush_counters(st, esc, pairs);
}

// Group-cooperative FP32 refine: kG consecutive lanes take one candidate
// (grid-stride over candidates per group); the group's leader writes the
// flag.  Same contract as k_refine (m_dev: device-side count, flags past it
// cleared).
template <int kG, int kMinBlocks>
__global__ void __launch_bounds__(256, kMinBlocks)
    k_refine_group(GeomsView B, GeomsView P, const uint32_t* __restrict__ cb,
                   const uint32_t* __restrict__ cp, uint64_t m, uint32_t probe_base,
                   int predicate, uint8_t* __restrict__ flags, DeviceStatus* st,
                   const uint64_t* __restrict__ m_dev) {
  uint32_t esc = 0, pairs = 0;
  const int lane = threadIdx.x & 31;
  const int gl = lane & (kG - 1);
  const unsigned gm = kG == 32 ? 0xffffffffu : (((1u << kG) - 1u) << (lane & ~(kG - 1)));
  const uint64_t gid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / kG;
  const uint64_t ng = ((uint64_t)gridDim.x * blockDim.x) / kG;
  const uint64_t mm = m_dev ? min(*m_dev, m) : m;
  for (uint64_t k = gid; k < m; k += ng) {
    if (k >= mm) {
      if (gl == 0) flags[k] = 0;
      continue;
    }
    const uint32_t b = cb[k], p = cp[k] - probe_base;
    int r = eval_group<kG>(B, b, P, p, predicate, esc, gm, gl);
    if (gl == 0) {
      pairs++;
      if (r < 0) {
        status_fail(st, kUnsupported, k);
        r = 0;
      }
      flags[k] = (uint8_t)r;
    }
  }
  flush_counters(st, esc, pairs);
}

// ---------------------------------------------------------------------------
// ST_DWithin

__global__ void __launch_bounds__(256)
    k_dwithin(GeomsView B, GeomsView P, const uint32_t* __restrict__ cb,
              const uint32_t* __restrict__ cp, uint64_t m, uint32_t probe_base, double d,
              uint8_t* __restrict__ flags, DeviceStatus* st, const uint32_t* __restrict__ perm) {
  uint32_t esc = 0, pairs = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t start = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t trips = (m + stride - 1) / stride;
  for (uint64_t t = 0; t < trips; t++) {
    const uint64_t u = start + t * stride;
    if (u >= m) continue;
    const uint64_t k = perm ? (uint64_t)perm[u] : u;
    if (k >= m) continue;
    const uint32_t bi = cb[k], pi = cp[k] - probe_base;
    pairs++;
    if (B.kind[bi] != kPoint || P.kind[pi] != kPoint) {
      status_fail(st, kUnsupported, k);
      flags[k] = 0;
      continue;
    }
    const double2 b = B.pt[bi], p = P.pt[pi];
    // FP64 squared distance of the reference's deltas against d^2 with a
    // relative band of 1e-14, far above the few ulps of rounding in s2 and
    // d2: outside the band the comparison is exact; inside it, expansion
    // arithmetic decides.  (An FP32 first tier with a coordinate-magnitude
    // error bound sent 0.56% of the pairs of the 20M x 1M workload to the
    // expansion, which cost more on GB300 than the FP64 test it saves.)
    int r = -1;
    {
      const double dx = __dsub_rn(b.x, p.x), dy = __dsub_rn(b.y, p.y);
      const double s2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      const double d2 = __dmul_rn(d, d);
      if (s2 < __dmul_rn(d2, 1.0 - 1e-14)) r = 1;
      else if (s2 > __dmul_rn(d2, 1.0 + 1e-14)) r = 0;
    }
    if (r < 0) {
      esc++;
      r = dwithin_exact(b, p, d) ? 1 : 0;
    }
    flags[k] = (uint8_t)r;
  }
  flush_counters(st, esc, pairs);
}

__global__ void k_compact(const uint32_t* __restrict__ cb, const uint32_t* __restrict__ cp,
                          const uint8_t* __restrict__ flags, const uint64_t* __restrict__ pos,
                          uint64_t m, uint32_t* __restrict__ ob, uint32_t* __restrict__ op,
                          uint64_t out_cap) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < m;
       k += (uint64_t)gridDim.x * blockDim.x) {
    if (flags[k]) {
      const uint64_t o = pos[k];
      if (o >= out_cap) continue;  // bounded by the output capacity
      ob[o] = cb[k];
      op[o] = cp[k];
    }
  }
}

}  // namespace

void refine_relation(const GeomsView& build, const GeomsView& probe, const uint32_t* cb,
                     const uint32_t* cp, uint64_t m, uint32_t probe_base, int predicate, int form,
                     uint8_t* flags, DeviceStatus* st, cudaStream_t s, const uint64_t* m_dev,
                     const uint32_t* perm, int min_blocks, int group) {
  if (m == 0) return;
  if (form == kFastF32 && perm == nullptr && (group == 4 || group == 8 || group == 16)) {
    const int gg = grid_for((int64_t)m * group, 256, kNumSMs * 16);
#define SPJ_GROUP_LAUNCH(G, MB)                                                            \
  k_refine_group<G, MB><<<gg, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, predicate, \
                                           flags, st, m_dev)
    const bool wide = min_blocks <= 2;  // 128 registers, two blocks per SM
    if (group == 4) {
      if (wide) SPJ_GROUP_LAUNCH(4, 2);
      else SPJ_GROUP_LAUNCH(4, 4);
    } else if (group == 8) {
      if (wide) SPJ_GROUP_LAUNCH(8, 2);
      else SPJ_GROUP_LAUNCH(8, 4);
    } else {
      if (wide) SPJ_GROUP_LAUNCH(16, 2);
      else SPJ_GROUP_LAUNCH(16, 4);
    }
#undef SPJ_GROUP_LAUNCH
    SPJ_CUDA(cudaGetLastError());
    return;
  }
  const int g = grid_for((int64_t)m, 256, kNumSMs * 16);
  if (form == kFastF32 && min_blocks == 6)
    k_refine<true, 6><<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, predicate, flags, st,
                                        m_dev, perm);
  else if (form == kFastF32 && min_blocks == 5)
    k_refine<true, 5><<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, predicate, flags, st,
                                        m_dev, perm);
  else if (form == kFastF32 && min_blocks == 3)
    k_refine<true, 3><<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, predicate, flags, st,
                                        m_dev, perm);
  else if (form == kFastF32 && min_blocks == 2)
    k_refine<true, 2><<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, predicate, flags, st,
                                        m_dev, perm);
  else if (form == kFastF32)
    k_refine<true, 4><<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, predicate, flags, st,
                                        m_dev, perm);
  else
    k_refine<false, 1><<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, predicate, flags,
                                         st, m_dev, perm);
  SPJ_CUDA(cudaGetLastError());
}

void refine_dwithin(const GeomsView& build, const GeomsView& probe, const uint32_t* cb,
                    const uint32_t* cp, uint64_t m, uint32_t probe_base, double distance, int form,
                    uint8_t* flags, DeviceStatus* st, cudaStream_t s, const uint32_t* perm) {
  if (m == 0) return;
  (void)form;  // one form: see k_dwithin
  const int g = grid_for((int64_t)m, 256, kNumSMs * 16);
  k_dwithin<<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, distance, flags, st, perm);
  SPJ_CUDA(cudaGetLastError());
}

void compact_pairs(const uint32_t* cb, const uint32_t* cp, const uint8_t* flags,
                   const uint64_t* pos, uint64_t m, uint32_t* ob, uint32_t* op, cudaStream_t s,
                   uint64_t out_cap) {
  if (m == 0) return;
  k_compact<<<grid_for((int64_t)m, 256, kNumSMs * 16), 256, 0, s>>>(cb, cp, flags, pos, m, ob, op,
                                                                     out_cap);
  SPJ_CUDA(cudaGetLastError());
}

}  // namespace spj
