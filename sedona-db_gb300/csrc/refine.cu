// refine.cu — relation-predicate and ST_DWithin refinement of candidate
// pairs, one thread per candidate, plus order-preserving compaction.
//
// Replaces the reference's RTSpatialRefiner::Refine
// (c/sedona-libgpuspatial/libgpuspatial/src/rt_spatial_refiner.cu:134-242),
// which re-parses probe WKB on the CPU each call and runs OptiX PIP
// (src/rt/shaders/polygon_point_query.cu) or a recursive DE-9IM relate
// (src/relate_engine.cu:294-336).  Here both sides are already decoded in HBM
// and the predicate is the tg semantics the reference CPU join uses.
#include "distance.cuh"
#include "refine_eval.cuh"

namespace spj {
namespace {

using namespace pred;
using exact::dwithin_exact;

// ---------------------------------------------------------------------------
// ST_DWithin

__global__ void __launch_bounds__(256)
    k_dwithin(GeomsView B, GeomsView P, const uint32_t* __restrict__ cb,
              const uint32_t* __restrict__ cp, uint64_t m, uint32_t probe_base, double d,
              const double* __restrict__ d_row, uint8_t* __restrict__ flags, DeviceStatus* st,
              const uint32_t* __restrict__ perm) {
  const double d0 = d;
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
    // the probe row's distance (a per-row column or one value); a negative
    // or NaN distance keeps nothing
    const double d = d_row ? d_row[pi] : d0;
    if (!(d >= 0)) {
      flags[k] = 0;
      continue;
    }
    if (B.kind[bi] != kPoint || P.kind[pi] != kPoint) {
      // polygons: the reference's distance in FP64, compared with d
      esc++;
      flags[k] = row_distance<true>(B, bi, P, pi, esc) <= d ? 1 : 0;
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

}  // namespace

void refine_relation(const GeomsView& build, const GeomsView& probe, const uint32_t* cb,
                     const uint32_t* cp, uint64_t m, uint32_t probe_base, int predicate, int form,
                     uint8_t* flags, DeviceStatus* st, cudaStream_t s, const uint64_t* m_dev,
                     const uint32_t* perm, int min_blocks, uint32_t* queue, uint32_t* qn,
                     bool ordered_queue) {
  if (m == 0) return;
  const RefineLaunch a{build, probe, cb,    cp,   m,     probe_base, predicate,
                       flags, st,    m_dev, perm, queue, qn,         s};
  if (form == kFastF32 && queue && qn) {
    launch_refine_split(a, min_blocks, ordered_queue);
    return;
  }
  if (form == kFastF32 && min_blocks == 6) {
    launch_refine_blocks6(a);
    return;
  }
  const uint32_t trips = m_dev ? 0 : kRefineChunkTrips;
  const unsigned g = refine_grid(m, trips);
  if (form == kFastF32)
    k_refine<true, 4><<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, predicate, flags, st,
                                        m_dev, perm, nullptr, nullptr, nullptr, trips);
  else
    k_refine<false, 1><<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, predicate, flags,
                                         st, m_dev, perm, nullptr, nullptr, nullptr, trips);
  SPJ_CUDA(cudaGetLastError());
}

void refine_dwithin(const GeomsView& build, const GeomsView& probe, const uint32_t* cb,
                    const uint32_t* cp, uint64_t m, uint32_t probe_base, double distance, int form,
                    uint8_t* flags, DeviceStatus* st, cudaStream_t s, const uint32_t* perm,
                    const double* d_row) {
  if (m == 0) return;
  (void)form;  // one form: see k_dwithin
  const int g = grid_for((int64_t)m, 256, kNumSMs * 16);
  k_dwithin<<<g, 256, 0, s>>>(build, probe, cb, cp, m, probe_base, distance, d_row, flags, st,
                              perm);
  SPJ_CUDA(cudaGetLastError());
}


}  // namespace spj
