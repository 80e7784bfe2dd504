// wkb_decode.cu — Arrow binary WKB -> device SoA geometry columns.
//
// Replaces the reference's CPU thread-pool parse + H2D copy
// (c/sedona-libgpuspatial/libgpuspatial/include/gpuspatial/loader/
//  parallel_wkb_loader.hpp:579-790) with device kernels:
//   1. k_wkb_count   thread per row: validate the WKB, classify the row and
//                    count its parts / rings / vertices; point rows are fully
//                    decoded here (point, f32 box) — a point column needs
//                    nothing else.
//   2. three scans   row -> part / ring / vertex starts
//   3. k_wkb_struct  thread per polygonal row: part -> ring and ring -> vertex
//                    offsets and each ring's source byte position
//   4. k_wkb_coords  warp per ring: coalesced copy of the ring's coordinates
//                    (aligned 32-bit loads + funnel shifts, WKB doubles are
//                    unaligned), f32 copy, ring rect by warp reduction,
//                    tg's segment count
//   5. k_row_box     thread per polygonal row: outward-rounded f32 box
// Algorithmic bytes: WKB bytes + offsets in; per vertex 16 B (f64) + 8 B
// (f32) out; per row 16 B box + 16 B point + 1 B kind out.
#include "geoms.cuh"
#include "prims.cuh"
#include "relate_flags.cuh"
#include "wkb_read.cuh"

namespace spj {
namespace {

using namespace wkb;

// f64 interval -> f32 outward (rust/sedona-spatial-join/src/utils/bounds.rs:147-162)
__device__ __forceinline__ void outward(double lo, double hi, float& flo, float& fhi) {
  float a = __double2float_rn(lo), b = __double2float_rn(hi);
  if ((double)a > lo) a = next_downf(a);
  if ((double)b < hi) b = next_upf(b);
  flo = a;
  fhi = b;
}

__device__ __forceinline__ float4 nan_box() {
  float q = __int_as_float(0x7fc00000);
  return make_float4(q, q, q, q);
}

// Row header: byte order + type, 2D only.  Returns status code.
__device__ __forceinline__ uint32_t rd_header(const uint8_t* d, uint64_t p, uint64_t end,
                                              uint64_t len, bool al, bool& le, uint32_t& type) {
  if (p + 5 > end) return kWkbTruncated;
  uint8_t bo = d[p];
  if (bo > 1) return kWkbByteOrder;
  le = bo == 1;
  uint32_t t = read_u32(d, p + 1, len, al, le);
  if (t & 0xE0000000u) return kWkbDims;
  if (t >= 1000) return kWkbDims;
  type = t;
  return kOk;
}

// Walk a polygon body at p (after its header); counts rings and vertices
// (points + 1 closing copy per ring).  Returns status; advances p.
__device__ __forceinline__ uint32_t walk_polygon(const uint8_t* d, uint64_t& p, uint64_t end,
                                                 uint64_t len, bool al, bool le, uint32_t& nrings,
                                                 uint64_t& nverts) {
  if (p + 4 > end) return kWkbTruncated;
  nrings = read_u32(d, p, len, al, le);
  p += 4;
  if ((uint64_t)nrings * 4 > end - p) return kWkbCount;
  nverts = 0;
  for (uint32_t r = 0; r < nrings; r++) {
    if (p + 4 > end) return kWkbTruncated;
    uint32_t np = read_u32(d, p, len, al, le);
    p += 4;
    if ((uint64_t)np * 16 > end - p) return kWkbCount;
    p += (uint64_t)np * 16;
    nverts += (uint64_t)np + 1;
  }
  return kOk;
}

template <bool kOff64>
__global__ void k_wkb_count(WkbDeviceColumn col, bool al, uint8_t* __restrict__ kind,
                            double2* __restrict__ pt, float4* __restrict__ box,
                            uint32_t* __restrict__ cparts, uint32_t* __restrict__ crings,
                            uint32_t* __restrict__ cverts, DeviceStatus* st, bool points_only,
                            uint8_t* __restrict__ rflags = nullptr,
                            unsigned long long* __restrict__ any_rflag = nullptr) {
  const uint8_t* d = col.data;
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < col.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint8_t k = kEmpty;
    bool empty_part = false;
    uint32_t np = 0, nr = 0;
    uint64_t nv = 0;
    double2 q = make_double2(qnan, qnan);
    float4 b = nan_box();
    uint32_t code = kOk;
    if (row_valid(col.validity, col.validity_offset, i)) {
      uint64_t s, e;
      row_range<kOff64>(col.offsets, i, s, e);
      bool le;
      uint32_t type;
      code = (e < s || e > col.data_len) ? kWkbTruncated : rd_header(d, s, e, col.data_len, al, le, type);
      if (code == kOk) {
        if (type == 1) {
          if (s + 21 > e) {
            code = kWkbTruncated;
          } else {
            uint32_t w[4];
            load_words<4>(d, s + 5, col.data_len, al, w);
            double x = wkb_f64(w[0], w[1], le), y = wkb_f64(w[2], w[3], le);
            if (!(isnan(x) && isnan(y))) {  // POINT EMPTY is NaN NaN
              k = kPoint;
              q = make_double2(x, y);
              // GPU factory: round-to-nearest degenerate box (join_provider.rs:128-132)
              float fx = __double2float_rn(x), fy = __double2float_rn(y);
              b = make_float4(fx, fy, fx, fy);
            }
          }
        } else if (points_only) {
          code = kWkbType;  // caller asked for the point path; host retries generally
        } else if (type == 3) {
          uint64_t p = s + 5;
          uint32_t rings;
          uint64_t verts;
          code = walk_polygon(d, p, e, col.data_len, al, le, rings, verts);
          if (code == kOk && rings > 0) {
            k = kPolygon;
            np = 1;
            nr = rings;
            nv = verts;
          }
        } else if (type == 6) {
          uint64_t p = s + 5;
          if (p + 4 > e) {
            code = kWkbTruncated;
          } else {
            uint32_t nparts = read_u32(d, p, col.data_len, al, le);
            p += 4;
            for (uint32_t j = 0; j < nparts && code == kOk; j++) {
              bool le2;
              uint32_t t2;
              code = rd_header(d, p, e, col.data_len, al, le2, t2);
              if (code != kOk) break;
              if (t2 != 3) {
                code = kWkbType;
                break;
              }
              p += 5;
              uint32_t rings;
              uint64_t verts;
              code = walk_polygon(d, p, e, col.data_len, al, le2, rings, verts);
              if (code == kOk && rings > 0) {
                np++;
                nr += rings;
                nv += verts;
              } else if (code == kOk) {
                empty_part = true;  // skipped; remembered for covers / contains
              }
            }
            if (code == kOk && np > 0) k = kMultiPolygon;
          }
        } else {
          code = kWkbType;
        }
      }
      if (nv > 0xFFFFFFFFull) code = kWkbCount;
    }
    if (code != kOk) {
      status_fail(st, code, (uint64_t)i);
      k = kEmpty;
      np = nr = 0;
      nv = 0;
    }
    kind[i] = k;
    pt[i] = q;
    box[i] = b;
    if (!points_only) {
      cparts[i] = np;
      crings[i] = nr;
      cverts[i] = (uint32_t)nv;
    }
    if (rflags) {
      const bool f = empty_part && k == kMultiPolygon;
      rflags[i] = f ? 1 : 0;
      if (f) atomicOr(any_rflag, 1ull);
    }
  }
}

template <bool kOff64>
__global__ void k_wkb_struct(WkbDeviceColumn col, bool al, const uint8_t* __restrict__ kind,
                             const uint64_t* __restrict__ spart, const uint64_t* __restrict__ sring,
                             const uint64_t* __restrict__ svert, uint32_t* __restrict__ part_ring,
                             uint32_t* __restrict__ ring_vtx, uint64_t* __restrict__ ring_src,
                             uint32_t* __restrict__ ring_npts) {
  const uint8_t* d = col.data;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < col.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint8_t k = kind[i];
    if (k != kPolygon && k != kMultiPolygon) continue;
    uint64_t s, e;
    row_range<kOff64>(col.offsets, i, s, e);
    bool le = d[s] == 1;
    uint32_t P = (uint32_t)spart[i], R = (uint32_t)sring[i], V = (uint32_t)svert[i];
    uint64_t p = s + 5;
    uint32_t nparts = 1;
    bool multi = k == kMultiPolygon;
    if (multi) {
      nparts = read_u32(d, p, col.data_len, al, le);
      p += 4;
    }
    for (uint32_t j = 0; j < nparts; j++) {
      bool ple = le;
      if (multi) {
        ple = d[p] == 1;
        p += 5;
      }
      uint32_t nr = read_u32(d, p, col.data_len, al, ple);
      p += 4;
      if (nr == 0) continue;  // empty part, skipped when counting
      part_ring[P++] = R;
      for (uint32_t r = 0; r < nr; r++) {
        uint32_t npts = read_u32(d, p, col.data_len, al, ple);
        p += 4;
        ring_vtx[R] = V;
        ring_src[R] = p | (ple ? (1ull << 63) : 0ull);
        ring_npts[R] = npts;
        R++;
        V += npts + 1;
        p += (uint64_t)npts * 16;
      }
    }
  }
}

__device__ __forceinline__ bool feq(double x, double y) { return !((x < y) | (x > y)); }

// kG lanes per ring (8 for columns of small rings such as building
// footprints, 32 otherwise); consecutive groups take consecutive rings.
// Each ring is a chain of dependent loads (its source offset, then its
// points, then the closing copy), so more rings in flight per warp is what
// shortens the pass.
template <int kG>
__global__ void k_wkb_coords(const uint8_t* __restrict__ d, uint64_t len, bool al,
                             uint32_t nrings, const uint64_t* __restrict__ ring_src,
                             const uint32_t* __restrict__ ring_npts,
                             const uint32_t* __restrict__ ring_vtx, double2* __restrict__ xy,
                             float2* __restrict__ xy32, Rect64* __restrict__ ring_rect,
                             float4* __restrict__ ring_rect32, int32_t* __restrict__ ring_nsegs) {
  const int lane = threadIdx.x & (kG - 1);
  const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kG;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) / kG;
  // every group of the warp runs the same number of trips, so the shuffles
  // below always see the whole warp
  const int64_t trips = ((int64_t)nrings + nw - 1) / nw;
  for (int64_t t = 0; t < trips; t++) {
    const int64_t r = wid + t * nw;
    const bool live = r < nrings;
    const uint64_t src = live ? ring_src[r] : 0;
    const bool le = (src >> 63) != 0;
    const uint64_t o = src & ~(1ull << 63);
    const uint32_t npts = live ? ring_npts[r] : 0;
    const uint32_t V = live ? ring_vtx[r] : 0;
    double mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    for (uint32_t j = lane; j < npts; j += kG) {
      uint32_t w[4];
      load_words<4>(d, o + 16ull * j, len, al, w);
      double x = wkb_f64(w[0], w[1], le), y = wkb_f64(w[2], w[3], le);
      xy[V + j] = make_double2(x, y);
      xy32[V + j] = make_float2(__double2float_rn(x), __double2float_rn(y));
      // tg.c process_points: plain < / > comparisons
      if (x < mnx) mnx = x;
      if (y < mny) mny = y;
      if (x > mxx) mxx = x;
      if (y > mxy) mxy = y;
    }
#pragma unroll
    for (int m = kG / 2; m > 0; m >>= 1) {
      double a = __shfl_xor_sync(0xffffffffu, mnx, m);
      double b = __shfl_xor_sync(0xffffffffu, mny, m);
      double c = __shfl_xor_sync(0xffffffffu, mxx, m);
      double e = __shfl_xor_sync(0xffffffffu, mxy, m);
      if (a < mnx) mnx = a;
      if (b < mny) mny = b;
      if (c > mxx) mxx = c;
      if (e > mxy) mxy = e;
    }
    __syncwarp();
    if (live && lane == 0) {
      ring_rect[r] = make_rect64(mnx, mny, mxx, mxy);
      ring_rect32[r] = make_float4(__double2float_rn(mnx), __double2float_rn(mny),
                                   __double2float_rn(mxx), __double2float_rn(mxy));
      int32_t ns = 0;
      if (npts >= 3) {
        double2 f = xy[V], l = xy[V + npts - 1];
        ns = (feq(l.x, f.x) && feq(l.y, f.y)) ? (int32_t)npts - 1 : (int32_t)npts;
      }
      ring_nsegs[r] = ns;
      // the extra closing point (tg.c:2220)
      double2 f = npts ? xy[V] : make_double2(0.0, 0.0);
      xy[V + npts] = f;
      xy32[V + npts] = make_float2(__double2float_rn(f.x), __double2float_rn(f.y));
    }
  }
}

__global__ void k_row_box(uint32_t n, const uint8_t* __restrict__ kind,
                          const uint32_t* __restrict__ row_part,
                          const uint32_t* __restrict__ part_ring,
                          const Rect64* __restrict__ ring_rect, float4* __restrict__ box) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint8_t k = kind[i];
    if (k != kPolygon && k != kMultiPolygon) continue;
    uint32_t r0 = part_ring[row_part[i]], r1 = part_ring[row_part[i + 1]];
    double mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    for (uint32_t r = r0; r < r1; r++) {
      Rect64 q = ring_rect[r];
      mnx = fmin(mnx, q.x);
      mny = fmin(mny, q.y);
      mxx = fmax(mxx, q.z);
      mxy = fmax(mxy, q.w);
    }
    float4 b;
    outward(mnx, mxx, b.x, b.z);
    outward(mny, mxy, b.y, b.w);
    box[i] = b;
  }
}

// tg's ring flags (tg.c:1910-2113 process_points), one thread per ring
// (tg_ring_flags in relate_flags.cuh: the same walk as tg, in its order).
__global__ void k_ring_flags(uint32_t nrings, const uint32_t* __restrict__ ring_vtx,
                             const double2* __restrict__ xy, uint8_t* __restrict__ flags) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrings;
       r += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t V = ring_vtx[r];
    const uint32_t npts = ring_vtx[r + 1] - V - 1;  // as stored in the WKB
    flags[r] = tg_ring_flags(xy + V, npts);
  }
}

__global__ void k_u64_to_u32(const uint64_t* __restrict__ in, uint32_t* __restrict__ out,
                             int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (uint32_t)in[i];
}

__global__ void k_set_u32(uint32_t* p, uint32_t v) { *p = v; }

// ---------------------------------------------------------------------------
// y-band edge index

__device__ __forceinline__ int band_of(float y32, float y0, float inv_h, int nb) {
  float t = __fmul_rn(__fsub_rn(y32, y0), inv_h);
  if (!(t >= 0.0f)) return 0;
  float f = floorf(t);
  if (f >= (float)(nb - 1)) return nb - 1;
  return (int)f;
}

__device__ __forceinline__ int bands_for(int32_t nsegs) {
  if (nsegs <= 0 || nsegs > 65535) return 1;
  int nb = nsegs / 4;
  if (nb < 1) nb = 1;
  if (nb > 256) nb = 256;
  return nb;
}

__global__ void k_band_count(uint32_t nrings, const int32_t* __restrict__ nsegs,
                             const uint32_t* __restrict__ ring_vtx,
                             const Rect64* __restrict__ ring_rect,
                             const double2* __restrict__ xy, uint32_t* __restrict__ nbp1,
                             uint32_t* __restrict__ nent, float2* __restrict__ param) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrings;
       r += (int64_t)gridDim.x * blockDim.x) {
    int32_t ns = nsegs[r];
    int nb = bands_for(ns);
    Rect64 rc = ring_rect[r];
    float y0 = __double2float_rd(rc.y);
    float span = __fsub_ru(__double2float_ru(rc.w), y0);
    float inv = span > 0.0f ? __fdiv_rn((float)nb, span) : 0.0f;
    if (ns > 65535) inv = -1.0f;  // no index: kernels scan every edge
    param[r] = make_float2(y0, inv);
    uint32_t cnt = 0;
    if (inv >= 0.0f) {
      const uint32_t V = ring_vtx[r];
      for (int32_t i = 0; i < ns; i++) {
        double ya = xy[V + i].y, yb = xy[V + i + 1].y;
        float lo = __double2float_rn(ya < yb ? ya : yb);
        float hi = __double2float_rn(ya > yb ? ya : yb);
        cnt += band_of(hi, y0, inv, nb) - band_of(lo, y0, inv, nb) + 1;
      }
    }
    nbp1[r] = (uint32_t)nb + 1;
    nent[r] = cnt;
  }
}

__global__ void k_band_fill(uint32_t nrings, const int32_t* __restrict__ nsegs,
                            const uint32_t* __restrict__ ring_vtx, const double2* __restrict__ xy,
                            const float2* __restrict__ xy32, const float2* __restrict__ param,
                            const uint32_t* __restrict__ ring_bands,
                            const uint64_t* __restrict__ ent_start,
                            uint32_t* __restrict__ band_off, uint16_t* __restrict__ band_edges,
                            float4* __restrict__ band_seg, uint32_t* __restrict__ band_id) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrings;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t ns = nsegs[r];
    const uint32_t B = ring_bands[r];
    const int nb = (int)(ring_bands[r + 1] - B) - 1;
    const float2 pr = param[r];
    uint32_t* off = band_off + B;
    for (int b = 0; b <= nb; b++) off[b] = 0;
    if (pr.y < 0.0f) {
      off[0] = off[1] = (uint32_t)ent_start[r];
      continue;
    }
    const uint32_t V = ring_vtx[r];
    for (int32_t i = 0; i < ns; i++) {
      double ya = xy[V + i].y, yb = xy[V + i + 1].y;
      int lo = band_of(__double2float_rn(ya < yb ? ya : yb), pr.x, pr.y, nb);
      int hi = band_of(__double2float_rn(ya > yb ? ya : yb), pr.x, pr.y, nb);
      for (int b = lo; b <= hi; b++) off[b + 1]++;
    }
    uint32_t acc = (uint32_t)ent_start[r];
    for (int b = 0; b <= nb; b++) {
      acc += off[b];
      off[b] = acc;
    }
    // off[b] now = end of band b-1 = start of band b; fill with a cursor walk
    for (int32_t i = 0; i < ns; i++) {
      double ya = xy[V + i].y, yb = xy[V + i + 1].y;
      int lo = band_of(__double2float_rn(ya < yb ? ya : yb), pr.x, pr.y, nb);
      int hi = band_of(__double2float_rn(ya > yb ? ya : yb), pr.x, pr.y, nb);
      const float2 a32 = xy32[V + i], b32 = xy32[V + i + 1];
      const float4 sg = make_float4(a32.x, a32.y, b32.x, b32.y);
      for (int b = lo; b <= hi; b++) {
        band_seg[off[b]] = sg;
        band_id[off[b]] = B + (uint32_t)b;
        band_edges[off[b]++] = (uint16_t)i;
      }
    }
    // cursors advanced to the band ends: shift back to starts
    for (int b = nb; b > 0; b--) off[b] = off[b - 1];
    off[0] = (uint32_t)ent_start[r];
  }
}

// Sort key of a band entry: its f32 segment's xmax, descending, NaN first
// (NaN never satisfies the scans' "xmax < x" stop test, so it must come
// before every entry they may stop at).  The map from f32 to an unsigned key
// that orders like the floats is the sign-flip of the IEEE bits.
__global__ void k_band_xkeys(uint32_t n, const float4* __restrict__ seg, uint32_t* __restrict__ keys,
                             uint32_t* __restrict__ vals) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const float4 g = seg[e];
    const float x = g.x > g.z ? g.x : g.z;
    uint32_t k = 0;
    if (!isnan(x)) {
      const uint32_t u = __float_as_uint(x);
      k = ~(u ^ ((u >> 31) ? 0xFFFFFFFFu : 0x80000000u));
    }
    keys[e] = k;
    vals[e] = e;
  }
}

__global__ void k_gather_band_id(uint32_t n, const uint32_t* __restrict__ band_id,
                                 const uint32_t* __restrict__ perm, uint32_t* __restrict__ out) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x)
    out[e] = band_id[perm[e]];
}

__global__ void k_band_permute(uint32_t n, const uint32_t* __restrict__ perm,
                               const float4* __restrict__ seg_in,
                               const uint16_t* __restrict__ edge_in, float4* __restrict__ seg_out,
                               uint16_t* __restrict__ edge_out) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const uint32_t q = perm[e];
    seg_out[e] = seg_in[q];
    edge_out[e] = edge_in[q];
  }
}

}  // namespace

void reset_status(DevBuf& status, cudaStream_t s) {
  status.reserve(sizeof(DeviceStatus), s);
  SPJ_CUDA(cudaMemsetAsync(status.get(), 0, sizeof(DeviceStatus), s));
  // first_bad = all ones (no failure)
  SPJ_CUDA(cudaMemsetAsync(status.get(), 0xFF, sizeof(unsigned long long), s));
}

void check_status(DevBuf& status, cudaStream_t s, const char* what) {
  unsigned long long v = 0;
  SPJ_CUDA(cudaMemcpyAsync(&v, status.get(), sizeof v, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  if (v != ~0ull) {
    uint32_t code = (uint32_t)(v >> 40);
    uint64_t row = v & 0xFFFFFFFFFFull;
    throw Error(std::string(what) + ": row " + std::to_string(row) + ": " + status_message(code));
  }
}

static bool aligned4(const void* p) { return ((uintptr_t)p & 3u) == 0; }

void decode_wkb(const WkbDeviceColumn& col, DeviceGeoms& out, DecodeScratch& sc,
                bool points_hint, cudaStream_t s) {
  SPJ_CHECK(col.n >= 0 && col.n < (int64_t)0xFFFFFFFF, "decode: too many rows");
  const int64_t n = col.n;
  out.n = (uint32_t)n;
  out.kind.reserve(n + 1, s);
  out.pt.reserve((n + 1) * sizeof(double2), s);
  out.box.reserve((n + 1) * sizeof(float4), s);
  const bool al = aligned4(col.data);
  const int block = 256;
  const int grid = grid_for(n, block, kNumSMs * 32);

  if (points_hint) {
    reset_status(sc.status, s);
    if (col.offsets64)
      k_wkb_count<true><<<grid, block, 0, s>>>(col, al, out.kind.as<uint8_t>(),
                                               out.pt.as<double2>(), out.box.as<float4>(),
                                               nullptr, nullptr, nullptr,
                                               sc.status.as<DeviceStatus>(), true);
    else
      k_wkb_count<false><<<grid, block, 0, s>>>(col, al, out.kind.as<uint8_t>(),
                                                out.pt.as<double2>(), out.box.as<float4>(),
                                                nullptr, nullptr, nullptr,
                                                sc.status.as<DeviceStatus>(), true);
    SPJ_CUDA(cudaGetLastError());
    unsigned long long v = 0;
    SPJ_CUDA(cudaMemcpyAsync(&v, sc.status.get(), sizeof v, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    if (v == ~0ull) {
      out.nparts = out.nrings = out.nverts = 0;
      out.all_points = true;
      out.any_points = n > 0;
      out.any_polys = false;
      out.row_part.reserve((n + 1) * 4, s);
      SPJ_CUDA(cudaMemsetAsync(out.row_part.get(), 0, (n + 1) * 4, s));
      out.part_ring.reserve(4, s);
      SPJ_CUDA(cudaMemsetAsync(out.part_ring.get(), 0, 4, s));
      out.ring_vtx.reserve(4, s);
      SPJ_CUDA(cudaMemsetAsync(out.ring_vtx.get(), 0, 4, s));
      out.has_bands = false;
      out.has_row_flags = false;
      out.has_ring_flags = false;
      return;
    }
    // a non-point row: fall through to the general path
  }

  sc.counts.reserve((size_t)3 * (n + 1) * 4, s);
  uint32_t* cparts = sc.counts.as<uint32_t>();
  uint32_t* crings = cparts + (n + 1);
  uint32_t* cverts = crings + (n + 1);
  sc.scans.reserve((size_t)3 * (n + 1) * 8, s);
  uint64_t* spart = sc.scans.as<uint64_t>();
  uint64_t* sring = spart + (n + 1);
  uint64_t* svert = sring + (n + 1);
  reset_status(sc.status, s);
  out.row_flags.reserve(n + 1, s);
  // counters[7] of the status word: set when some row had empty parts
  unsigned long long* any_rflag = &sc.status.as<DeviceStatus>()->counters[7];
  if (col.offsets64)
    k_wkb_count<true><<<grid, block, 0, s>>>(col, al, out.kind.as<uint8_t>(), out.pt.as<double2>(),
                                             out.box.as<float4>(), cparts, crings, cverts,
                                             sc.status.as<DeviceStatus>(), false,
                                             out.row_flags.as<uint8_t>(), any_rflag);
  else
    k_wkb_count<false><<<grid, block, 0, s>>>(col, al, out.kind.as<uint8_t>(),
                                              out.pt.as<double2>(), out.box.as<float4>(), cparts,
                                              crings, cverts, sc.status.as<DeviceStatus>(), false,
                                              out.row_flags.as<uint8_t>(), any_rflag);
  SPJ_CUDA(cudaGetLastError());
  scan_u32_u64(cparts, spart, n, sc.tmp, s);
  scan_u32_u64(crings, sring, n, sc.tmp, s);
  scan_u32_u64(cverts, svert, n, sc.tmp, s);
  uint64_t tot[4];
  SPJ_CUDA(cudaMemcpyAsync(&tot[3], any_rflag, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(&tot[0], spart + n, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(&tot[1], sring + n, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(&tot[2], svert + n, 8, cudaMemcpyDeviceToHost, s));
  check_status(sc.status, s, "WKB decode");  // syncs
  SPJ_CHECK(tot[2] < 0xFFFFFFFFull && tot[1] < 0xFFFFFFFFull, "decode: too many vertices");
  out.nparts = (uint32_t)tot[0];
  out.nrings = (uint32_t)tot[1];
  out.nverts = (uint32_t)tot[2];
  out.any_polys = out.nparts > 0;
  out.all_points = out.nparts == 0;
  out.any_points = true;  // conservative; only used as a hint
  out.has_bands = false;
  out.has_row_flags = tot[3] != 0;
  out.has_ring_flags = false;

  out.row_part.reserve((n + 1) * 4, s);
  k_u64_to_u32<<<grid_for(n + 1, 256), 256, 0, s>>>(spart, out.row_part.as<uint32_t>(), n + 1);
  out.part_ring.reserve(((size_t)out.nparts + 1) * 4, s);
  out.ring_vtx.reserve(((size_t)out.nrings + 1) * 4, s);
  out.ring_nsegs.reserve(((size_t)out.nrings + 1) * 4, s);
  out.ring_rect.reserve(((size_t)out.nrings + 1) * sizeof(Rect64), s);
  out.ring_rect32.reserve(((size_t)out.nrings + 1) * sizeof(float4), s);
  out.xy.reserve(((size_t)out.nverts + 1) * sizeof(double2), s);
  out.xy32.reserve(((size_t)out.nverts + 1) * sizeof(float2), s);
  sc.ring_src.reserve(((size_t)out.nrings + 1) * 12, s);
  uint64_t* ring_src = sc.ring_src.as<uint64_t>();
  uint32_t* ring_npts = reinterpret_cast<uint32_t*>(ring_src + out.nrings + 1);
  k_set_u32<<<1, 1, 0, s>>>(out.part_ring.as<uint32_t>() + out.nparts, out.nrings);
  k_set_u32<<<1, 1, 0, s>>>(out.ring_vtx.as<uint32_t>() + out.nrings, out.nverts);
  if (out.nparts > 0) {
    if (col.offsets64)
      k_wkb_struct<true><<<grid, block, 0, s>>>(col, al, out.kind.as<uint8_t>(), spart, sring,
                                                svert, out.part_ring.as<uint32_t>(),
                                                out.ring_vtx.as<uint32_t>(), ring_src, ring_npts);
    else
      k_wkb_struct<false><<<grid, block, 0, s>>>(col, al, out.kind.as<uint8_t>(), spart, sring,
                                                 svert, out.part_ring.as<uint32_t>(),
                                                 out.ring_vtx.as<uint32_t>(), ring_src, ring_npts);
    // (nverts counts each ring's extra closing vertex; a group's trips over
    // a ring's vertices issue independent loads, so 8 lanes also serve rings
    // of up to a few dozen points)
    if ((uint64_t)out.nverts <= 24ull * out.nrings)
      k_wkb_coords<8><<<grid_for((int64_t)out.nrings * 8, 256, kNumSMs * 32), 256, 0, s>>>(
          col.data, col.data_len, al, out.nrings, ring_src, ring_npts,
          out.ring_vtx.as<uint32_t>(), out.xy.as<double2>(), out.xy32.as<float2>(),
          out.ring_rect.as<Rect64>(), out.ring_rect32.as<float4>(), out.ring_nsegs.as<int32_t>());
    else
      k_wkb_coords<32><<<grid_for((int64_t)out.nrings * 32, 256, kNumSMs * 32), 256, 0, s>>>(
          col.data, col.data_len, al, out.nrings, ring_src, ring_npts,
          out.ring_vtx.as<uint32_t>(), out.xy.as<double2>(), out.xy32.as<float2>(),
          out.ring_rect.as<Rect64>(), out.ring_rect32.as<float4>(), out.ring_nsegs.as<int32_t>());
    k_row_box<<<grid, block, 0, s>>>(out.n, out.kind.as<uint8_t>(), out.row_part.as<uint32_t>(),
                                     out.part_ring.as<uint32_t>(), out.ring_rect.as<Rect64>(),
                                     out.box.as<float4>());
  }
  SPJ_CUDA(cudaGetLastError());
}

void build_ring_flags(DeviceGeoms& g, cudaStream_t s) {
  g.ring_flags.reserve((size_t)g.nrings + 1, s);
  if (g.nrings > 0)
    k_ring_flags<<<grid_for(g.nrings, 128, kNumSMs * 16), 128, 0, s>>>(
        g.nrings, g.ring_vtx.as<uint32_t>(), g.xy.as<double2>(), g.ring_flags.as<uint8_t>());
  SPJ_CUDA(cudaGetLastError());
  g.has_ring_flags = true;
}

void build_band_index(DeviceGeoms& g, DecodeScratch& sc, cudaStream_t s) {
  const uint32_t nr = g.nrings;
  g.band_param.reserve(((size_t)nr + 1) * sizeof(float2), s);
  g.ring_bands.reserve(((size_t)nr + 1) * 4, s);
  if (nr == 0) {
    g.has_bands = true;
    SPJ_CUDA(cudaMemsetAsync(g.ring_bands.get(), 0, 4, s));
    g.band_off.reserve(4, s);
    g.band_edges.reserve(4, s);
    g.band_seg.reserve(16, s);
    return;
  }
  sc.counts.reserve((size_t)2 * (nr + 1) * 4, s);
  uint32_t* nbp1 = sc.counts.as<uint32_t>();
  uint32_t* nent = nbp1 + (nr + 1);
  sc.scans.reserve((size_t)2 * (nr + 1) * 8, s);
  uint64_t* sb = sc.scans.as<uint64_t>();
  uint64_t* se = sb + (nr + 1);
  const int grid = grid_for(nr, 128, kNumSMs * 8);
  k_band_count<<<grid, 128, 0, s>>>(nr, g.ring_nsegs.as<int32_t>(), g.ring_vtx.as<uint32_t>(),
                                    g.ring_rect.as<Rect64>(), g.xy.as<double2>(), nbp1, nent,
                                    g.band_param.as<float2>());
  scan_u32_u64(nbp1, sb, nr, sc.tmp, s);
  scan_u32_u64(nent, se, nr, sc.tmp, s);
  uint64_t tb = 0, te = 0;
  SPJ_CUDA(cudaMemcpyAsync(&tb, sb + nr, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(&te, se + nr, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  SPJ_CHECK(tb < 0xFFFFFFFFull && te < 0xFFFFFFFFull, "band index too large");
  k_u64_to_u32<<<grid_for(nr + 1, 256), 256, 0, s>>>(sb, g.ring_bands.as<uint32_t>(), nr + 1);
  g.band_off.reserve((size_t)(tb + 1) * 4, s);
  g.band_edges.reserve((size_t)(te + 1) * 2, s);
  g.band_seg.reserve((size_t)(te + 1) * 16, s);
  // entries in edge order first, then each band sorted by xmax descending
  // (stable: band-major after two LSD sorts), so the FP32 scans stop at the
  // first entry strictly left of the point or box they test
  DevBuf seg0((size_t)(te + 1) * 16, s), edge0((size_t)(te + 1) * 2, s);
  DevBuf bid((size_t)(te + 1) * 4, s), keys((size_t)(te + 1) * 4, s),
      vals((size_t)(te + 1) * 4, s), akeys((size_t)(te + 1) * 4, s),
      avals((size_t)(te + 1) * 4, s);
  k_band_fill<<<grid, 128, 0, s>>>(nr, g.ring_nsegs.as<int32_t>(), g.ring_vtx.as<uint32_t>(),
                                   g.xy.as<double2>(), g.xy32.as<float2>(),
                                   g.band_param.as<float2>(), g.ring_bands.as<uint32_t>(), se,
                                   g.band_off.as<uint32_t>(), edge0.as<uint16_t>(),
                                   seg0.as<float4>(), bid.as<uint32_t>());
  SPJ_CUDA(cudaGetLastError());
  const uint32_t ne = (uint32_t)te;
  if (ne > 0) {
    const int eg = grid_for(ne, 256, kNumSMs * 8);
    k_band_xkeys<<<eg, 256, 0, s>>>(ne, seg0.as<float4>(), keys.as<uint32_t>(),
                                    vals.as<uint32_t>());
    radix_sort_pairs(keys.as<uint32_t>(), vals.as<uint32_t>(), akeys.as<uint32_t>(),
                     avals.as<uint32_t>(), ne, 32, sc.tmp, s);
    k_gather_band_id<<<eg, 256, 0, s>>>(ne, bid.as<uint32_t>(), vals.as<uint32_t>(),
                                        keys.as<uint32_t>());
    int bits = 1;
    while (bits < 32 && (tb >> bits) != 0) bits++;
    radix_sort_pairs(keys.as<uint32_t>(), vals.as<uint32_t>(), akeys.as<uint32_t>(),
                     avals.as<uint32_t>(), ne, bits, sc.tmp, s);
    k_band_permute<<<eg, 256, 0, s>>>(ne, vals.as<uint32_t>(), seg0.as<float4>(),
                                      edge0.as<uint16_t>(), g.band_seg.as<float4>(),
                                      g.band_edges.as<uint16_t>());
    SPJ_CUDA(cudaGetLastError());
  }
  g.has_bands = true;
}

}  // namespace spj
