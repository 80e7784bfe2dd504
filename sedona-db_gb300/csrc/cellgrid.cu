// cellgrid.cu — per-ring cell grids for the FP32 refine.
//
// A ring with at least kGridMinSegs segments gets a G x G grid over its
// outward f32 rect.  A cell is clean when no edge of the ring touches the
// closed cell, proven on f32 values: the edge's RN32 bbox strictly separated
// from the cell (a strict comparison of RN values proves the exact one), or
// all four cell corners strictly on one side of the edge (decided orient32,
// whose static bound covers the rounding of the edge's coordinates).  Edges
// whose y-range misses the cell's are strictly separated in y and are not
// listed in the bands the cell spans, so only those bands are scanned.
// Every point of a clean cell has the same tg answer (the isolation-exit
// argument in predicates.cuh); the cell stores it, evaluated at the cell
// centre with the regular point-in-ring code.
#include "geoms.cuh"
#include "predicates.cuh"
#include "prims.cuh"

#include <cmath>

namespace spj {
namespace {

using namespace pred;

__device__ __forceinline__ uint32_t grid_dim(int nsegs) {
  if (nsegs < kGridMinSegs) return 0;
  uint32_t g = 2u * (uint32_t)ceilf(sqrtf((float)nsegs));
  return g < 8u ? 8u : (g > 32u ? 32u : g);
}

__global__ void k_grid_count(uint32_t nr, const int32_t* __restrict__ nsegs,
                             uint32_t* __restrict__ cells) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += gridDim.x * blockDim.x) {
    const uint32_t g = grid_dim(nsegs[r]);
    cells[r] = g * g;
  }
}

// Outward f32 origin / step of one axis: [lo, lo + n step] covers [a, b].
__device__ __forceinline__ bool grid_axis(double a, double b, int n, float& o, float& step) {
  float lo = __double2float_rd(a), hi = __double2float_ru(b);
  if (!(hi > lo) || !isfinite(lo) || !isfinite(hi)) return false;
  step = __fdiv_ru(__fsub_ru(hi, lo), (float)n);
  if (!(step > 0.0f) || !isfinite(step)) return false;
  o = lo;
  for (int t = 0; t < 64 && grid_edge(o, step, n) < hi; t++) step = next_upf(step);
  return grid_edge(o, step, n) >= hi;
}

// One block per ring (grid-stride over rings), threads over the cells.
__global__ void __launch_bounds__(256)
    k_grid_fill(GeomsView G, const uint64_t* __restrict__ cell_off, uint2* __restrict__ meta,
                float4* __restrict__ rect, uint8_t* __restrict__ status) {
  __shared__ float4 s_rect;
  __shared__ int s_ok;
  for (uint32_t r = blockIdx.x; r < G.nrings; r += gridDim.x) {
    const uint32_t g = grid_dim(G.ring_nsegs[r]);
    if (threadIdx.x == 0) {
      float ox = 0, oy = 0, sx = 0, sy = 0;
      const Rect64 R = G.ring_rect[r];
      const bool ok = g > 0 && G.ring_bands != nullptr && G.band_param[r].y >= 0.0f &&
                      grid_axis(R.x, R.z, (int)g, ox, sx) && grid_axis(R.y, R.w, (int)g, oy, sy);
      s_ok = ok ? 1 : 0;
      s_rect = make_float4(ox, oy, sx, sy);
      meta[r] = make_uint2((uint32_t)cell_off[r], ok ? g : 0u);
      rect[r] = s_rect;
    }
    __syncthreads();
    if (s_ok) {
      const float4 q = s_rect;
      const uint32_t B = G.ring_bands[r];
      const int nb = (int)(G.ring_bands[r + 1] - B) - 1;
      const float2 prm = G.band_param[r];
      for (uint32_t c = threadIdx.x; c < g * g; c += blockDim.x) {
        const int i = (int)(c % g), j = (int)(c / g);
        const float x0 = grid_edge(q.x, q.z, i), x1 = grid_edge(q.x, q.z, i + 1);
        const float y0 = grid_edge(q.y, q.w, j), y1 = grid_edge(q.y, q.w, j + 1);
        const int b0 = band_of(y0, prm.x, prm.y, nb), b1 = band_of(y1, prm.x, prm.y, nb);
        bool clean = true;
        for (uint32_t k = G.band_off[B + b0]; k < G.band_off[B + b1 + 1] && clean; k++) {
          const float4 sg = G.band_seg[k];
          const float2 a = make_float2(sg.x, sg.y), b = make_float2(sg.z, sg.w);
          if (fmax0f(a.x, b.x) < x0 || fmin0f(a.x, b.x) > x1 || fmax0f(a.y, b.y) < y0 ||
              fmin0f(a.y, b.y) > y1)
            continue;
          const int s0 = orient32(a, b, make_float2(x0, y0));
          if (s0 != 0 && orient32(a, b, make_float2(x1, y0)) == s0 &&
              orient32(a, b, make_float2(x1, y1)) == s0 && orient32(a, b, make_float2(x0, y1)) == s0)
            continue;
          clean = false;
        }
        uint8_t st = 0;
        if (clean) {
          // the centre, an f32 point strictly inside the cell
          const float cx = __fmul_rn(0.5f, __fadd_rn(x0, x1));
          const float cy = __fmul_rn(0.5f, __fadd_rn(y0, y1));
          uint32_t esc = 0;
          const bool in = ring_pip_fast(G, r, make_double2((double)cx, (double)cy),
                                        make_float2(cx, cy), true, esc)
                              .hit;
          st = in ? 1 : 2;
        }
        status[cell_off[r] + c] = st;
      }
    }
    __syncthreads();
  }
}

}  // namespace

void build_cell_grid(DeviceGeoms& g, DecodeScratch& sc, cudaStream_t s) {
  const uint32_t nr = g.nrings;
  g.has_grid = false;
  if (nr == 0 || !g.has_bands) return;
  g.grid_meta.reserve(((size_t)nr + 1) * sizeof(uint2), s);
  g.grid_rect.reserve(((size_t)nr + 1) * sizeof(float4), s);
  sc.counts.reserve(((size_t)nr + 1) * 4, s);
  sc.scans.reserve(((size_t)nr + 1) * 8, s);
  k_grid_count<<<grid_for(nr, 256), 256, 0, s>>>(nr, g.ring_nsegs.as<int32_t>(),
                                                 sc.counts.as<uint32_t>());
  scan_u32_u64(sc.counts.as<uint32_t>(), sc.scans.as<uint64_t>(), nr, sc.tmp, s);
  uint64_t total = 0;
  SPJ_CUDA(cudaMemcpyAsync(&total, sc.scans.as<uint64_t>() + nr, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  SPJ_CHECK(total < 0xFFFFFFFFull, "cell grid too large");
  g.grid_status.reserve(total + 16, s);
  // the grid is built with the point-in-ring code of a view without a grid
  GeomsView v = g.view();
  k_grid_fill<<<grid_for(nr, 1, kNumSMs * 8), 256, 0, s>>>(
      v, sc.scans.as<uint64_t>(), g.grid_meta.as<uint2>(), g.grid_rect.as<float4>(),
      g.grid_status.as<uint8_t>());
  SPJ_CUDA(cudaGetLastError());
  SPJ_CUDA(cudaStreamSynchronize(s));
  g.has_grid = true;
}

}  // namespace spj
