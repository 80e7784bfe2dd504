// learned.cu — learned point index (see learned.cuh): Hilbert keys, device
// radix sort, GPU training of the two-stage piecewise-linear model, and the
// lookup / range kernels with LBVH fallback.
#include <cmath>

#include "learned.cuh"
#include "predicates.cuh"
#include "prims.cuh"
#include "refine.cuh"

namespace spj {

struct LearnedView {
  uint32_t n, L, window;  // window: lookups; window_box: the cells of range rows
  uint32_t window_box;
  const uint32_t* keys;
  const uint32_t* ids;
  const double2* xy;
  const float2* xy32;
  const uint32_t* start;  // L + 1
  const double* a;
  const double* b;
  // per leaf (a, b - start) in FP32: the query-time prediction of the
  // position inside the leaf (the window search verifies its answer)
  const float2* ab32;
  const uint32_t* kc;
  const uint32_t* err;
  const uint16_t* root_tab;  // root_p + 1 entries: leaves whose first key's prefix < p
  uint32_t root_shift, root_p;
  uint32_t k0;
  float x0, y0, sx, sy;
};

namespace {

using namespace pred;

constexpr int kLeafThreads = 256;
constexpr uint32_t kMaxCells = 256;

// Hilbert index of cell (x, y) on a 2^16 x 2^16 grid (the classic
// rotate-and-reflect walk from the top quadrant level down).
__device__ __forceinline__ uint32_t hilbert16(uint32_t x, uint32_t y) {
  const uint32_t n = 1u << 16;
  uint32_t d = 0;
  for (uint32_t s = n >> 1; s > 0; s >>= 1) {
    const uint32_t rx = (x & s) ? 1u : 0u, ry = (y & s) ? 1u : 0u;
    d += s * s * ((3u * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {
        x = n - 1 - x;
        y = n - 1 - y;
      }
      const uint32_t t = x;
      x = y;
      y = t;
    }
  }
  return d;
}

// grid cell of an RN32 coordinate: monotone, so every point inside a box
// falls in the box's cell range
__device__ __forceinline__ uint32_t cell_of(float v, float v0, float s) {
  const float t = __fmul_rn(__fsub_rn(v, v0), s);
  if (!(t >= 0.0f)) return 0;
  if (t >= 65535.0f) return 65535;
  return (uint32_t)t;
}

__device__ __forceinline__ uint32_t key_of(const LearnedView& v, float2 p) {
  return hilbert16(cell_of(p.x, v.x0, v.sx), cell_of(p.y, v.y0, v.sy));
}

// Stage one: the leaf holding lower_bound(q).  Leaves are equal-count rank
// ranges; the answer is the last leaf whose first key is < q (leaf 0 when
// none is).  A radix table over key prefixes narrows the leaves to the few
// whose first key shares q's prefix, then a short binary search over those
// first keys (kc) finishes.
__device__ __forceinline__ uint32_t root_leaf(const LearnedView& v, uint32_t q) {
  if (v.n == 0 || q <= v.k0) return 0;
  uint32_t p = (q - v.k0) >> v.root_shift;
  if (p > v.root_p - 1) p = v.root_p - 1;
  uint32_t lo = v.root_tab[p], hi = v.root_tab[p + 1];
  // leaves < lo: first key's prefix < p (first key < q); leaves >= hi:
  // prefix > p (first key > q); find the first leaf in [lo, hi) with key >= q
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (v.kc[mid] < q) lo = mid + 1;
    else hi = mid;
  }
  return lo ? lo - 1 : 0;
}

__device__ __forceinline__ uint32_t bsearch_first_ge(const uint32_t* keys, uint32_t lo,
                                                     uint32_t hi, uint32_t q, uint32_t& steps) {
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    steps++;
    if (keys[mid] < q) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// lower_bound(q) over the sorted keys; exact (verified); `bad` is set when
// the leaf's error exceeds the window (the caller takes the LBVH instead)
__device__ __forceinline__ uint32_t learned_lower_bound(const LearnedView& v, uint32_t q,
                                                        uint32_t& steps, uint32_t& misses,
                                                        bool& bad) {
  const uint32_t l = root_leaf(v, q);
  const uint32_t e = v.err[l];
  bad = e > v.window;
  if (bad) return 0;
  // the answer lies in [start_l, start_{l+1}] (the first key of leaf l is
  // < q unless l == 0, and leaf l+1's first key is >= q)
  const uint32_t s_lo = v.start[l];
  const uint32_t s_hi = min(v.start[l + 1] + 1u, v.n);
  // The window around the prediction, relative to the leaf start, in FP32:
  // e was measured on the FP64 line, and the FP32 line (a leaf-local
  // intercept, so the values stay within the leaf's size) differs from it
  // by far less than one position, covered by two more on each side.  GB300's
  // FP64 rate made the FP64 form the range phase's busiest pipe.  The window
  // is verified below either way.
  const float2 ab = v.ab32[l];
  const float predl =
      __fmaf_rn(ab.x, (float)((int64_t)q - (int64_t)v.kc[l]), ab.y);
  const float span = (float)(s_hi - s_lo);
  uint32_t lo = s_lo, hi = s_hi;
  if (isfinite(predl)) {
    const float flo = floorf(predl) - (float)e - 3.0f;
    const float fhi = ceilf(predl) + (float)e + 4.0f;
    if (flo > 0.0f) lo = s_lo + (uint32_t)fminf(flo, span);
    if (fhi < span) hi = s_lo + (uint32_t)fmaxf(fhi, 0.0f);
  }
  if (hi < lo) hi = lo;
  uint32_t p = bsearch_first_ge(v.keys, lo, hi, q, steps);
  const bool ok_lo = p == 0 || v.keys[p - 1] < q;
  const bool ok_hi = p == v.n || v.keys[p] >= q;
  if (!(ok_lo && ok_hi)) {
    // outside the measured error (q between keys at a leaf edge): the
    // leaf's whole range, then (never needed by construction) everything
    misses++;
    p = bsearch_first_ge(v.keys, s_lo, s_hi, q, steps);
    if (!((p == 0 || v.keys[p - 1] < q) && (p == v.n || v.keys[p] >= q)))
      p = bsearch_first_ge(v.keys, 0, v.n, q, steps);
  }
  return p;
}

// --- build ------------------------------------------------------------------

__global__ void k_point_flags(const uint8_t* __restrict__ kind, uint32_t n, uint8_t* flag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flag[i] = kind[i] == kPoint ? 1 : 0;
}

__global__ void k_compact(const uint8_t* __restrict__ flag, const uint64_t* __restrict__ pos,
                          uint32_t n, uint32_t* __restrict__ ids) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (flag[i]) ids[pos[i]] = i;
}

__device__ __forceinline__ uint32_t f2o(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_extent(const float4* __restrict__ box, const uint32_t* __restrict__ ids,
                         uint32_t m, uint32_t* ext) {
  float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const float4 b = box[ids[i]];
    mnx = fminf(mnx, b.x);
    mny = fminf(mny, b.y);
    mxx = fmaxf(mxx, b.x);
    mxy = fmaxf(mxy, b.y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&ext[0], f2o(mnx));
    atomicMin(&ext[1], f2o(mny));
    atomicMax(&ext[2], f2o(mxx));
    atomicMax(&ext[3], f2o(mxy));
  }
}

__global__ void k_keys(LearnedView v, const float4* __restrict__ box,
                       const uint32_t* __restrict__ ids, uint32_t m, uint32_t* __restrict__ keys) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const float4 b = box[ids[i]];
    keys[i] = key_of(v, make_float2(b.x, b.y));
  }
}

__global__ void k_gather(const double2* __restrict__ pt, const float4* __restrict__ box,
                         const uint32_t* __restrict__ ids, uint32_t m, double2* __restrict__ xy,
                         float2* __restrict__ xy32) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint32_t id = ids[i];
    xy[i] = pt[id];
    const float4 b = box[id];
    xy32[i] = make_float2(b.x, b.y);
  }
}

// block reduction of 6 doubles (blockDim == kLeafThreads)
__device__ __forceinline__ void block_sum6(double (&v)[6], double (*sm)[kLeafThreads / 32]) {
  for (int o = 16; o > 0; o >>= 1)
    for (int c = 0; c < 6; c++) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int c = 0; c < 6; c++) sm[c][w] = v[c];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int c = 0; c < 6; c++) {
      double t = 0;
      for (int j = 0; j < kLeafThreads / 32; j++) t += sm[c][j];
      v[c] = t;
    }
  }
  __syncthreads();
}

// Untrained start: the line through the leaf's first and last (key, rank).
__global__ void k_leaf_init(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                            uint32_t L, uint32_t n, double* a, double* b, uint32_t* kc) {
  for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < L; l += gridDim.x * blockDim.x) {
    const uint32_t s = start[l], e = start[l + 1];
    if (s >= e) {
      a[l] = 0;
      b[l] = (double)s;
      kc[l] = s < n ? keys[s] : 0xFFFFFFFFu;  // keeps first keys non-decreasing
      continue;
    }
    kc[l] = keys[s];
    const double dx = (double)(keys[e - 1] - keys[s]);
    a[l] = dx > 0 ? (double)(e - 1 - s) / dx : 0.0;
    b[l] = (double)s;
  }
}

// Forward + backward over one leaf per CTA: residual e = a x + b - r,
// loss = sum e^2, grad = (sum 2 e x, sum 2 e), Hessian = 2 (sum x^2, sum x, n).
__global__ void __launch_bounds__(kLeafThreads)
    k_leaf_fwd_bwd(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                   const uint32_t* __restrict__ kc, const double* __restrict__ a,
                   const double* __restrict__ b, double* __restrict__ out /* L x 6 */) {
  __shared__ double sm[6][kLeafThreads / 32];
  const uint32_t l = blockIdx.x;
  const uint32_t s = start[l], e = start[l + 1];
  const double al = a[l], bl = b[l];
  const uint32_t k = kc[l];
  double v[6] = {0, 0, 0, 0, 0, 0};
  for (uint32_t i = s + threadIdx.x; i < e; i += kLeafThreads) {
    const double x = (double)(keys[i] - k), r = (double)i;
    const double res = __fma_rn(al, x, bl) - r;  // forward
    v[0] = __fma_rn(res, res, v[0]);            // loss
    v[1] = __fma_rn(2.0 * res, x, v[1]);        // d/da
    v[2] += 2.0 * res;                          // d/db
    v[3] = __fma_rn(2.0 * x, x, v[3]);          // H_aa
    v[4] += 2.0 * x;                            // H_ab
    v[5] += 2.0;                                // H_bb
  }
  block_sum6(v, sm);
  if (threadIdx.x == 0)
    for (int c = 0; c < 6; c++) out[(size_t)l * 6 + c] = v[c];
}

// One Newton step per leaf: (a, b) -= H^-1 g (exact for the quadratic loss).
__global__ void k_leaf_newton(const double* __restrict__ fb, uint32_t L, double* a, double* b) {
  for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < L; l += gridDim.x * blockDim.x) {
    const double* f = fb + (size_t)l * 6;
    const double ga = f[1], gb = f[2], haa = f[3], hab = f[4], hbb = f[5];
    if (hbb <= 0) continue;  // empty leaf
    const double det = haa * hbb - hab * hab;
    if (!(fabs(det) > 1e-12 * fabs(haa * hbb))) {
      b[l] -= gb / hbb;  // single distinct key: constant model
      continue;
    }
    a[l] -= (hbb * ga - hab * gb) / det;
    b[l] -= (haa * gb - hab * ga) / det;
  }
}

__global__ void __launch_bounds__(kLeafThreads)
    k_leaf_err(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
               const uint32_t* __restrict__ kc, const double* __restrict__ a,
               const double* __restrict__ b, uint32_t* __restrict__ err) {
  __shared__ double sm[kLeafThreads / 32];
  const uint32_t l = blockIdx.x;
  const uint32_t s = start[l], e = start[l + 1];
  double m = 0;
  for (uint32_t i = s + threadIdx.x; i < e; i += kLeafThreads) {
    const double pred = __fma_rn(a[l], (double)(keys[i] - kc[l]), b[l]);
    m = fmax(m, fabs(pred - (double)i));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 1; j < kLeafThreads / 32; j++) m = fmax(m, sm[j]);
    m = fmax(m, sm[0]);
    err[l] = m > 4.0e9 ? 0xFFFFFFFFu : (uint32_t)ceil(m);
  }
}

// The query-time FP32 copy of each leaf's line: slope, and the intercept
// relative to the leaf's first position.
__global__ void k_leaf_ab32(uint32_t L, const double* __restrict__ a, const double* __restrict__ b,
                            const uint32_t* __restrict__ start, float2* __restrict__ out) {
  for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < L; l += gridDim.x * blockDim.x)
    out[l] = make_float2(__double2float_rn(a[l]),
                         __double2float_rn(__dsub_rn(b[l], (double)start[l])));
}

// --- queries --------------------------------------------------------------

__device__ __forceinline__ bool in_box(float2 p, float4 b) {
  return !(p.x < b.x || p.x > b.z || p.y < b.y || p.y > b.w);
}

// pred(build point, probe polygon row) for range rows
__device__ __forceinline__ bool range_pred(const GeomsView& P, uint32_t pr, double2 pt,
                                           float2 pt32, bool aoe, uint32_t& esc) {
  for (uint32_t q = P.row_part[pr]; q < P.row_part[pr + 1]; q++)
    if (poly_contains_point<true>(P, q, pt, pt32, aoe, esc)) return true;
  return false;
}

// First index >= lo whose key is not q (lo itself when keys[lo] != q):
// gallop, then bisect.
__device__ __forceinline__ uint32_t run_end(const uint32_t* keys, uint32_t n, uint32_t lo,
                                            uint32_t q, uint32_t& steps) {
  if (lo >= n || keys[lo] != q) return lo;
  uint32_t a = lo, b = lo + 1, step = 1;
  while (b < n && keys[b] == q) {  // keys[a] == q throughout
    a = b;
    step <<= 1;
    b = (n - a > step) ? a + step : n;
    steps++;
  }
  while (b - a > 1) {  // keys[a] == q, b == n or keys[b] != q
    const uint32_t mid = a + ((b - a) >> 1);
    steps++;
    if (keys[mid] == q) a = mid;
    else b = mid;
  }
  return b;
}

// Probe row classes: what a row contributes for the predicate.
enum RowClass : int { kRowNone = 0, kRowLookup = 1, kRowRange = 2 };

// pred(build point, probe row): point rows are equality lookups (touches is
// always false for two points, tg.c:1102-1106); polygon rows are ranges:
// within -> the polygon contains the point, intersects / coveredby -> covers;
// contains / equals are always false for a point (tg.c:1157-1162).  Other
// predicates are not supported (status, reported once in the counting pass).
__device__ __forceinline__ int row_class(uint8_t kind, int predicate, DeviceStatus* st,
                                         uint32_t row, bool report) {
  if (kind == kPoint) {
    if (predicate == kTouches) return kRowNone;
    if (predicate == kDisjoint) {
      if (report) status_fail(st, kUnsupported, row);
      return kRowNone;
    }
    return kRowLookup;
  }
  if (kind == kPolygon || kind == kMultiPolygon) {
    if (predicate == kContains || predicate == kEquals) return kRowNone;
    if (predicate != kIntersects && predicate != kCoveredBy && predicate != kWithin) {
      if (report) status_fail(st, kUnsupported, row);
      return kRowNone;
    }
    return kRowRange;
  }
  return kRowNone;
}

constexpr uint32_t kRangeSorted = 0;  // ranks in the key-sorted build points
constexpr uint32_t kRangeLeaf = 1;    // an LBVH leaf (sorted primitive indices)

// A row's first kRangeCache ranges are kept by the counting pass (start,
// len | kind << 31), so the writing pass copies them instead of searching
// again; rows with more ranges search again.
constexpr uint32_t kRangeCache = 8;

// ranges are written at pos < cap only (the count pass sized them)
template <int kPass>
__device__ __forceinline__ void put_range(uint4* ranges, uint64_t& pos, uint32_t& cnt,
                                          uint32_t start, uint32_t len, uint32_t row,
                                          uint32_t kind, uint64_t cap, uint2* cache) {
  if (len == 0) return;
  if (kPass) {
    if (pos < cap) ranges[pos] = make_uint4(start, len, row, kind);
    pos++;
  } else {
    if (cnt < kRangeCache) cache[(size_t)row * kRangeCache + cnt] = make_uint2(start, len | (kind << 31));
    cnt++;
  }
}

// The LBVH leaves whose boxes overlap q, as ranges (the fallback).
template <int kPass>
__device__ void leaf_ranges(const LbvhView& t, float4 q, int* stack, uint32_t row, uint4* ranges,
                            uint64_t& pos, uint32_t& cnt, uint64_t cap, uint2* cache) {
  if (t.nprims == 0) return;
  const uint64_t max_steps = 2ull * t.nleaves + 2;
  uint64_t steps = 0;
  int sp = 0, node = t.nleaves > 1 ? 0 : ~0;
  while (true) {
    if (++steps > max_steps) {  // each node is visited at most once
      traversal_fault(t, kTooLong, row);
      break;
    }
    if (node < 0) {
      const uint32_t c = (uint32_t)(~node);
      if (c >= t.nleaves) {
        traversal_fault(t, kBadLeaf, c);
        break;
      }
      const uint32_t b0 = c * t.leaf_size, b1 = min(b0 + t.leaf_size, t.nprims);
      put_range<kPass>(ranges, pos, cnt, b0, b1 - b0, row, kRangeLeaf, cap, cache);
    } else {
      if ((uint32_t)node + 1 >= t.nleaves) {
        traversal_fault(t, kBadNode, (unsigned)node);
        break;
      }
      const float4 lb = t.node_box[2 * node], rb = t.node_box[2 * node + 1];
      const int2 ch = t.node_child[node];
      const bool hl = box_overlap(lb, q), hr = box_overlap(rb, q);
      if (hl && hr) {
        if (sp >= kTravStack) {  // deeper than any tree built here: record, stop
          traversal_fault(t, kStackOverflow, (unsigned)row);
          break;
        }
        stack[sp * 128] = ch.y;
        sp++;
        node = ch.x;
        continue;
      }
      if (hl || hr) {
        node = hl ? ch.x : ch.y;
        continue;
      }
    }
    if (sp == 0) break;
    sp--;
    node = stack[sp * 128];
  }
}

// Sort key of a probe row (its lookup key, or its box centre's), so that
// neighbouring threads search neighbouring parts of the model and the keys.
__global__ void k_row_keys(LearnedView v, GeomsView P, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ vals) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
    const float4 b = P.box[i];
    uint32_t key = 0xFFFFFFFFu;
    if (b.x <= b.z && b.y <= b.w)
      key = key_of(v, make_float2(0.5f * b.x + 0.5f * b.z, 0.5f * b.y + 0.5f * b.w));
    keys[i] = key;
    vals[i] = i;
  }
}

// Phase A: per probe row, the build-point ranges that can hold its pairs:
// for a lookup the run of its key among the sorted keys (found through the
// model), for a box the runs of the grid cells it covers, and LBVH leaves
// where the model's error exceeds the window or the box covers too many
// cells.  Pass 0 counts, pass 1 writes at the scanned offsets (row order).
template <int kPass>
__global__ void __launch_bounds__(128)
    k_learned_ranges(LearnedView v, LbvhView t, GeomsView P, int predicate,
                     const uint32_t* __restrict__ order, uint32_t* __restrict__ rcount,
                     const uint64_t* __restrict__ roff, uint4* __restrict__ ranges,
                     uint64_t cap, uint2* __restrict__ cache, unsigned long long* __restrict__ ctr,
                     DeviceStatus* st) {
  __shared__ int stack[kTravStack * 128];
  // steps: the model-guided lower_bound searches; rsteps: the runs of equal
  // keys after them (independent of the model, not counted)
  uint32_t steps = 0, misses = 0, fallbacks = 0, lookups = 0, rsteps = 0;
  for (uint32_t jj = blockIdx.x * blockDim.x + threadIdx.x; jj < P.n;
       jj += gridDim.x * blockDim.x) {
    const uint32_t i = order ? order[jj] : jj;
    if (i >= P.n) {
      traversal_fault(t, kBadProbe, i);
      continue;
    }
    const int cls = row_class(P.kind[i], predicate, st, i, kPass == 0);
    uint32_t cnt = 0;
    uint64_t pos = kPass ? roff[i] : 0;
    if (kPass) {
      const uint64_t nr = roff[i + 1] - pos;
      if (nr <= kRangeCache) {  // kept by the counting pass
        for (uint32_t c = 0; c < (uint32_t)nr; c++) {
          const uint2 e = cache[(size_t)i * kRangeCache + c];
          if (pos < cap) ranges[pos] = make_uint4(e.x, e.y & 0x7FFFFFFFu, i, e.y >> 31);
          pos++;
        }
        continue;
      }
    }
    if (cls == kRowLookup) {
      const float4 pb = P.box[i];
      const uint32_t q = key_of(v, make_float2(pb.x, pb.y));
      bool bad = false;
      lookups++;
      const uint32_t lo = learned_lower_bound(v, q, steps, misses, bad);
      if (!bad) {
        const uint32_t hi = run_end(v.keys, v.n, lo, q, rsteps);
        put_range<kPass>(ranges, pos, cnt, lo, hi - lo, i, kRangeSorted, cap, cache);
      } else {
        fallbacks++;
        leaf_ranges<kPass>(t, pb, stack + threadIdx.x, i, ranges, pos, cnt, cap, cache);
      }
    } else if (cls == kRowRange) {
      const float4 bx = P.box[i];  // outward f32 box of the probe polygon
      const uint32_t cx0 = cell_of(bx.x, v.x0, v.sx), cx1 = cell_of(bx.z, v.x0, v.sx);
      const uint32_t cy0 = cell_of(bx.y, v.y0, v.sy), cy1 = cell_of(bx.w, v.y0, v.sy);
      const uint64_t ncell = (uint64_t)(cx1 - cx0 + 1) * (cy1 - cy0 + 1);
      if (bx.x <= bx.z && bx.y <= bx.w) {  // (an empty box has no pairs)
        bool use_tree = ncell > kMaxCells;
        // a cell whose leaf is over the window sends the row to the LBVH
        for (uint32_t cy = cy0; cy <= cy1 && !use_tree; cy++)
          for (uint32_t cx = cx0; cx <= cx1 && !use_tree; cx++)
            use_tree = v.err[root_leaf(v, hilbert16(cx, cy))] > v.window_box;
        if (!use_tree) {
          for (uint32_t cy = cy0; cy <= cy1; cy++) {
            for (uint32_t cx = cx0; cx <= cx1; cx++) {
              const uint32_t q = hilbert16(cx, cy);
              bool bad = false;
              lookups++;
              // (the leaf's error is within window_box, checked above; the
              // search below uses it whatever the lookup window is)
              LearnedView vb = v;
              vb.window = 0xFFFFFFFFu;
              const uint32_t lo = learned_lower_bound(vb, q, steps, misses, bad);
              const uint32_t hi = run_end(v.keys, v.n, lo, q, rsteps);
              put_range<kPass>(ranges, pos, cnt, lo, hi - lo, i, kRangeSorted, cap, cache);
            }
          }
        } else {
          fallbacks++;
          leaf_ranges<kPass>(t, bx, stack + threadIdx.x, i, ranges, pos, cnt, cap, cache);
        }
      }
    }
    if (!kPass) rcount[i] = cnt;
  }
  if (kPass == 0) {
    for (int o = 16; o > 0; o >>= 1) {
      steps += __shfl_xor_sync(0xffffffffu, steps, o);
      misses += __shfl_xor_sync(0xffffffffu, misses, o);
      fallbacks += __shfl_xor_sync(0xffffffffu, fallbacks, o);
      lookups += __shfl_xor_sync(0xffffffffu, lookups, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(&ctr[0], (unsigned long long)lookups);
      atomicAdd(&ctr[1], (unsigned long long)misses);
      atomicAdd(&ctr[2], (unsigned long long)fallbacks);
      atomicAdd(&ctr[3], (unsigned long long)steps);
    }
  }
}

// Phase B: the candidates of the ranges, load-balanced.  A warp takes 32
// consecutive ranges, scans their lengths, and walks the concatenated
// candidates 32 at a time, each lane finding its range by a 5-step search
// over the scan; lookups test point equality, boxes the RN32 in-box test and
// then the polygon predicate.  Pass 0 counts per chunk of 32 ranges, pass 1
// writes with ballot ranks at the chunk's scanned offset, so pairs stay in
// range order (grouped by probe row).
// Words of hit masks per chunk of 32 ranges: ceil(candidates / 32).
__global__ void k_chunk_words(const uint4* __restrict__ ranges, uint64_t nranges,
                              uint32_t* __restrict__ words) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nchunks = (nranges + 31) / 32;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t chunk = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; chunk < nchunks;
       chunk += nwarps) {
    const uint64_t r = chunk * 32 + lane;
    uint32_t len = r < nranges ? ranges[r].y : 0;
    for (int o = 16; o > 0; o >>= 1) len += __shfl_xor_sync(0xffffffffu, len, o);
    if (lane == 0) words[chunk] = (len + 31) / 32;
  }
}

template <int kPass>
__global__ void __launch_bounds__(128)
    k_learned_eval(LearnedView v, LbvhView t, GeomsView B, GeomsView P, uint32_t probe_base,
                   int predicate, const uint4* __restrict__ ranges, uint64_t nranges,
                   uint32_t* __restrict__ ccount, const uint64_t* __restrict__ coff,
                   const uint64_t* __restrict__ woff, uint32_t* __restrict__ masks,
                   uint64_t nwords, uint32_t* __restrict__ ob, uint32_t* __restrict__ op,
                   uint64_t cap, unsigned long long* __restrict__ ctr) {
  const bool aoe = predicate != kWithin;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nchunks = (nranges + 31) / 32;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint32_t esc = 0;
  for (uint64_t chunk = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; chunk < nchunks;
       chunk += nwarps) {
    const uint64_t r = chunk * 32 + lane;
    const uint4 R = r < nranges ? ranges[r] : make_uint4(0, 0, 0, 0);
    uint32_t incl = R.y;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += x;
    }
    const uint32_t excl = incl - R.y;
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint64_t pos = kPass ? coff[chunk] : 0;
    const uint64_t w0 = woff[chunk];
    uint32_t cnt = 0;
    for (uint32_t base = 0; base < total; base += 32) {
      const uint64_t w = w0 + base / 32;
      const uint32_t tt = base + lane;
      // owner: the last lane whose exclusive offset is <= tt (it has len > 0)
      int L = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const uint32_t e = __shfl_sync(0xffffffffu, excl, L + step);
        if (e <= tt) L += step;
      }
      const uint32_t start = __shfl_sync(0xffffffffu, R.x, L);
      const uint32_t row = __shfl_sync(0xffffffffu, R.z, L);
      const uint32_t kind = __shfl_sync(0xffffffffu, R.w, L);
      const uint32_t eL = __shfl_sync(0xffffffffu, excl, L);
      bool hit = false;
      uint32_t id = 0;
      if (kPass == 0 && tt < total) {
        const uint32_t j = start + (tt - eL);
        double2 pt;
        float2 pt32;
        if (kind == kRangeSorted) {
          pt = v.xy[j];
          pt32 = v.xy32[j];
        } else {
          const float4 sb = t.sorted_box[j];
          pt32 = make_float2(sb.x, sb.y);
          pt = B.pt[t.sorted_id[j]];
        }
        if (P.kind[row] == kPoint) hit = pteq(pt, P.pt[row]);
        else hit = in_box(pt32, P.box[row]) && range_pred(P, row, pt, pt32, aoe, esc);
      }
      // pass 0 keeps the hit mask, pass 1 reads it back instead of testing again
      unsigned m;
      if (kPass == 0) {
        m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0 && w < nwords) masks[w] = m;
      } else {
        m = w < nwords ? masks[w] : 0u;
        hit = (m >> lane) & 1u;
        if (hit) {
          const uint32_t j = start + (tt - eL);
          id = kind == kRangeSorted ? v.ids[j] : t.sorted_id[j];
        }
      }
      if (kPass) {
        if (hit) {
          const uint64_t o = pos + __popc(m & ((1u << lane) - 1u));
          if (o < cap) {
            ob[o] = id;
            op[o] = row + probe_base;
          }
        }
        pos += __popc(m);
      } else {
        cnt += __popc(m);
      }
    }
    if (!kPass && lane == 0) ccount[chunk] = cnt;
  }
  if (kPass == 0) {
    for (int o = 16; o > 0; o >>= 1) esc += __shfl_xor_sync(0xffffffffu, esc, o);
    if (lane == 0 && esc) atomicAdd(&ctr[4], (unsigned long long)esc);
  }
}

float o2f_host(uint32_t u) {
  uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
  float f;
  memcpy(&f, &v, 4);
  return f;
}

}  // namespace

LearnedIndex::LearnedIndex(uint32_t leaves, uint32_t window)
    : L_(leaves), window_(window), window_box_(window) {
  SPJ_CHECK(leaves >= 1 && leaves <= 65535, "leaves must be in [1, 65535]");
  for (auto& e : ev_) SPJ_CUDA(cudaEventCreate(&e));
}

LearnedIndex::~LearnedIndex() {
  cudaDeviceSynchronize();
  for (auto& e : ev_)
    if (e) cudaEventDestroy(e);
}

void LearnedIndex::set_window(uint32_t window) { set_windows(window, window); }

void LearnedIndex::set_windows(uint32_t window, uint32_t window_box) {
  window_ = window;
  window_box_ = window_box;
  uint32_t over = 0;
  for (uint32_t l = 0; l < L_ && l < host_err_.size(); l++)
    if (host_start_[l + 1] > host_start_[l] && host_err_[l] > window_) over++;
  stats_.leaves_over_window = over;
}

static LearnedView make_view(uint32_t n, uint32_t L, uint32_t window, const DevBuf& keys,
                             const DevBuf& ids, const DevBuf& xy, const DevBuf& xy32,
                             const DevBuf& start, const DevBuf& a, const DevBuf& b,
                             const DevBuf& ab32, const DevBuf& kc, const DevBuf& err,
                             const DevBuf& root_tab,
                             uint32_t root_shift, uint32_t root_p, uint32_t k0, float x0,
                             float y0, float sx, float sy) {
  LearnedView v;
  v.n = n;
  v.L = L;
  v.window = window;
  v.window_box = window;
  v.keys = keys.as<uint32_t>();
  v.ids = ids.as<uint32_t>();
  v.xy = xy.as<double2>();
  v.xy32 = xy32.as<float2>();
  v.start = start.as<uint32_t>();
  v.a = a.as<double>();
  v.b = b.as<double>();
  v.ab32 = ab32.as<float2>();
  v.kc = kc.as<uint32_t>();
  v.err = err.as<uint32_t>();
  v.root_tab = root_tab.as<uint16_t>();
  v.root_shift = root_shift;
  v.root_p = root_p;
  v.k0 = k0;
  v.x0 = x0;
  v.y0 = y0;
  v.sx = sx;
  v.sy = sy;
  return v;
}

#define SPJ_LVIEW()                                                                           \
  make_view(n_, L_, window_, keys_, ids_, xy_, xy32_, leaf_start_, leaf_a_, leaf_b_, leaf_ab32_, \
            leaf_kc_, leaf_err_, root_tab_, root_shift_, root_p_, k0_, x0_, y0_, sx_, sy_)

void LearnedIndex::build(const DeviceGeoms& pts, const Lbvh& bvh, cudaStream_t s) {
  bv_ = pts.view();
  tv_ = bvh.view();
  const uint32_t N = pts.n;
  DevBuf flag((size_t)N + 1, s), pos(((size_t)N + 1) * 8, s);
  k_point_flags<<<grid_for(N, 256), 256, 0, s>>>(pts.kind.as<uint8_t>(), N, flag.as<uint8_t>());
  scan_u8_u64(flag.as<uint8_t>(), pos.as<uint64_t>(), N, tmp_, s);
  uint64_t m64 = 0;
  SPJ_CUDA(cudaMemcpyAsync(&m64, pos.as<uint64_t>() + N, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  n_ = (uint32_t)m64;
  const uint32_t m = n_;
  keys_.reserve(((size_t)m + 1) * 4, s);
  ids_.reserve(((size_t)m + 1) * 4, s);
  k_compact<<<grid_for(N, 256), 256, 0, s>>>(flag.as<uint8_t>(), pos.as<uint64_t>(), N,
                                              ids_.as<uint32_t>());
  DevBuf ext(16, s);
  const uint32_t init[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u};
  SPJ_CUDA(cudaMemcpyAsync(ext.get(), init, 16, cudaMemcpyHostToDevice, s));
  if (m) k_extent<<<grid_for(m, 256), 256, 0, s>>>(pts.box.as<float4>(), ids_.as<uint32_t>(), m,
                                                    ext.as<uint32_t>());
  uint32_t he[4];
  SPJ_CUDA(cudaMemcpyAsync(he, ext.get(), 16, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  if (m) {
    x0_ = o2f_host(he[0]);
    y0_ = o2f_host(he[1]);
    const float x1 = o2f_host(he[2]), y1 = o2f_host(he[3]);
    sx_ = x1 > x0_ ? 65536.0f / (x1 - x0_) : 0.0f;
    sy_ = y1 > y0_ ? 65536.0f / (y1 - y0_) : 0.0f;
  }
  LearnedView v = SPJ_LVIEW();
  if (m) k_keys<<<grid_for(m, 256), 256, 0, s>>>(v, pts.box.as<float4>(), ids_.as<uint32_t>(),
                                                  m, keys_.as<uint32_t>());
  {
    DevBuf ak(((size_t)m + 1) * 4, s), av(((size_t)m + 1) * 4, s);
    radix_sort_pairs(keys_.as<uint32_t>(), ids_.as<uint32_t>(), ak.as<uint32_t>(),
                     av.as<uint32_t>(), m, 32, tmp_, s);
  }
  xy_.reserve(((size_t)m + 1) * 16, s);
  xy32_.reserve(((size_t)m + 1) * 8, s);
  if (m) k_gather<<<grid_for(m, 256), 256, 0, s>>>(pts.pt.as<double2>(), pts.box.as<float4>(),
                                                    ids_.as<uint32_t>(), m, xy_.as<double2>(),
                                                    xy32_.as<float2>());
  leaf_start_.reserve(((size_t)L_ + 1) * 4, s);
  leaf_a_.reserve(((size_t)L_ + 1) * 8, s);
  leaf_b_.reserve(((size_t)L_ + 1) * 8, s);
  leaf_kc_.reserve(((size_t)L_ + 1) * 4, s);
  leaf_err_.reserve(((size_t)L_ + 1) * 4, s);
  counters_.reserve(64, s);
  fit_root(s);
  train(true, s);
}

void LearnedIndex::fit_root(cudaStream_t s) {
  const uint32_t m = n_;
  // equal-count leaves: leaf l covers ranks [l*m/L, (l+1)*m/L)
  std::vector<uint32_t> st(L_ + 1);
  for (uint32_t l = 0; l <= L_; l++) st[l] = (uint32_t)((uint64_t)l * m / L_);
  SPJ_CUDA(cudaMemcpyAsync(leaf_start_.get(), st.data(), st.size() * 4, cudaMemcpyHostToDevice, s));
  k_leaf_init<<<grid_for(L_, 256), 256, 0, s>>>(keys_.as<uint32_t>(), leaf_start_.as<uint32_t>(),
                                                L_, m, leaf_a_.as<double>(), leaf_b_.as<double>(),
                                                leaf_kc_.as<uint32_t>());
  std::vector<uint32_t> kc(L_);
  uint32_t kend = 0;
  SPJ_CUDA(cudaMemcpyAsync(kc.data(), leaf_kc_.get(), (size_t)L_ * 4, cudaMemcpyDeviceToHost, s));
  if (m)
    SPJ_CUDA(cudaMemcpyAsync(&kend, keys_.as<uint32_t>() + (m - 1), 4, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  // stage-one radix table over key prefixes: entry p counts the leaves whose
  // first key has a prefix below p
  k0_ = m ? kc[0] : 0;
  const uint32_t span = m ? kend - k0_ : 0;
  int bits = 0;
  while (bits < 32 && (span >> bits) != 0) bits++;
  root_shift_ = bits > 16 ? (uint32_t)(bits - 16) : 0u;
  root_p_ = (span >> root_shift_) + 1;
  std::vector<uint16_t> tab(root_p_ + 1);
  uint32_t l = 0;
  for (uint32_t p = 0; p <= root_p_; p++) {
    while (l < L_ && kc[l] != 0xFFFFFFFFu && ((kc[l] - k0_) >> root_shift_) < p) l++;
    tab[p] = (uint16_t)l;
  }
  root_tab_.reserve(tab.size() * 2, s);
  SPJ_CUDA(cudaMemcpyAsync(root_tab_.get(), tab.data(), tab.size() * 2, cudaMemcpyHostToDevice, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  stats_.root_shift = root_shift_;
  stats_.root_entries = root_p_;
  stats_.leaves = L_;
  stats_.points = m;
}

void LearnedIndex::train(bool trained, cudaStream_t s) {
  k_leaf_init<<<grid_for(L_, 256), 256, 0, s>>>(keys_.as<uint32_t>(), leaf_start_.as<uint32_t>(),
                                                L_, n_, leaf_a_.as<double>(), leaf_b_.as<double>(),
                                                leaf_kc_.as<uint32_t>());
  DevBuf fb((size_t)L_ * 6 * 8, s);
  if (trained) {
    k_leaf_fwd_bwd<<<L_, kLeafThreads, 0, s>>>(keys_.as<uint32_t>(), leaf_start_.as<uint32_t>(),
                                               leaf_kc_.as<uint32_t>(), leaf_a_.as<double>(),
                                               leaf_b_.as<double>(), fb.as<double>());
    k_leaf_newton<<<grid_for(L_, 256), 256, 0, s>>>(fb.as<double>(), L_, leaf_a_.as<double>(),
                                                    leaf_b_.as<double>());
    // gradient after the step (~0 up to rounding): reported as a check
    k_leaf_fwd_bwd<<<L_, kLeafThreads, 0, s>>>(keys_.as<uint32_t>(), leaf_start_.as<uint32_t>(),
                                               leaf_kc_.as<uint32_t>(), leaf_a_.as<double>(),
                                               leaf_b_.as<double>(), fb.as<double>());
    std::vector<double> h((size_t)L_ * 6);
    SPJ_CUDA(cudaMemcpyAsync(h.data(), fb.get(), h.size() * 8, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    double g = 0;
    for (uint32_t l = 0; l < L_; l++) {
      // relative to the gradient scale of the leaf
      const double scale = std::sqrt(h[l * 6 + 3] * h[l * 6 + 5]) + 1.0;
      g = std::max(g, std::fabs(h[l * 6 + 2]) / std::sqrt(h[l * 6 + 5] + 1.0) / scale);
    }
    stats_.grad_norm_after = g;
  }
  measure_errors(s);
}

void LearnedIndex::measure_errors(cudaStream_t s) {
  k_leaf_err<<<L_, kLeafThreads, 0, s>>>(keys_.as<uint32_t>(), leaf_start_.as<uint32_t>(),
                                         leaf_kc_.as<uint32_t>(), leaf_a_.as<double>(),
                                         leaf_b_.as<double>(), leaf_err_.as<uint32_t>());
  leaf_ab32_.reserve(((size_t)L_ + 1) * sizeof(float2), s);
  k_leaf_ab32<<<grid_for(L_, 256), 256, 0, s>>>(L_, leaf_a_.as<double>(), leaf_b_.as<double>(),
                                                leaf_start_.as<uint32_t>(),
                                                leaf_ab32_.as<float2>());
  std::vector<uint32_t> e(L_), st(L_ + 1);
  SPJ_CUDA(cudaMemcpyAsync(e.data(), leaf_err_.get(), (size_t)L_ * 4, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(st.data(), leaf_start_.get(), ((size_t)L_ + 1) * 4,
                           cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  host_err_ = e;
  host_start_ = st;
  uint32_t mx = 0, over = 0, nonempty = 0;
  double sum = 0;
  for (uint32_t l = 0; l < L_; l++) {
    if (st[l + 1] == st[l]) continue;
    nonempty++;
    mx = std::max(mx, e[l]);
    sum += e[l];
    if (e[l] > window_) over++;
  }
  stats_.max_err = mx;
  stats_.mean_err = nonempty ? sum / nonempty : 0;
  stats_.leaves_over_window = over;
  SPJ_CUDA(cudaGetLastError());
}

void LearnedIndex::loss_and_grad(const std::vector<double>& a, const std::vector<double>& b,
                                 std::vector<double>& loss, std::vector<double>& ga,
                                 std::vector<double>& gb, cudaStream_t s) {
  SPJ_CHECK(a.size() == L_ && b.size() == L_, "parameter arrays must have one entry per leaf");
  DevBuf da((size_t)L_ * 8, s), db((size_t)L_ * 8, s), fb((size_t)L_ * 6 * 8, s);
  SPJ_CUDA(cudaMemcpyAsync(da.get(), a.data(), (size_t)L_ * 8, cudaMemcpyHostToDevice, s));
  SPJ_CUDA(cudaMemcpyAsync(db.get(), b.data(), (size_t)L_ * 8, cudaMemcpyHostToDevice, s));
  k_leaf_fwd_bwd<<<L_, kLeafThreads, 0, s>>>(keys_.as<uint32_t>(), leaf_start_.as<uint32_t>(),
                                             leaf_kc_.as<uint32_t>(), da.as<double>(),
                                             db.as<double>(), fb.as<double>());
  std::vector<double> h((size_t)L_ * 6);
  SPJ_CUDA(cudaMemcpyAsync(h.data(), fb.get(), h.size() * 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  loss.resize(L_);
  ga.resize(L_);
  gb.resize(L_);
  for (uint32_t l = 0; l < L_; l++) {
    loss[l] = h[l * 6];
    ga[l] = h[l * 6 + 1];
    gb[l] = h[l * 6 + 2];
  }
}

uint64_t LearnedIndex::query(const GeomsView& probe, uint32_t probe_base, int predicate,
                             DevBuf& out_build, DevBuf& out_probe, cudaStream_t s) {
  const uint32_t np = probe.n;
  scratch_.reserve(sizeof(DeviceStatus), s);
  reset_status(scratch_, s);
  SPJ_CUDA(cudaMemsetAsync(counters_.get(), 0, 64, s));
  LearnedView v = SPJ_LVIEW();
  v.window_box = window_box_;
  DeviceStatus* st = scratch_.as<DeviceStatus>();
  auto* ctr = counters_.as<unsigned long long>();
  if (np == 0) {
    out_build.reserve(4, s);
    out_probe.reserve(4, s);
    return 0;
  }
  // row keys, 4 radix passes (5 each), ranges x2 + scan (3); with ranges:
  // chunk words + scan, eval x2 + scan
  stats_.kernel_launches += 1 + 20 + 2 + 3;
  // probe rows in key order (locality of the model and key searches)
  SPJ_CUDA(cudaEventRecord(ev_[0], s));
  const size_t rb = ((size_t)np + 1) * 4;
  order_.reserve(rb, s);
  okeys_.reserve(rb, s);
  akeys_.reserve(rb, s);
  avals_.reserve(rb, s);
  k_row_keys<<<grid_for(np, 256), 256, 0, s>>>(v, probe, okeys_.as<uint32_t>(),
                                               order_.as<uint32_t>());
  radix_sort_pairs(okeys_.as<uint32_t>(), order_.as<uint32_t>(), akeys_.as<uint32_t>(),
                   avals_.as<uint32_t>(), np, 32, tmp_, s);
  SPJ_CUDA(cudaEventRecord(ev_[1], s));
  // phase A: ranges per row
  counts_.reserve(rb, s);
  offs_.reserve(((size_t)np + 1) * 8, s);
  rcache_.reserve(((size_t)np + 1) * kRangeCache * sizeof(uint2), s);
  const int ga = grid_for(np, 128, kNumSMs * 16);
  k_learned_ranges<0><<<ga, 128, 0, s>>>(v, tv_, probe, predicate, order_.as<uint32_t>(),
                                         counts_.as<uint32_t>(), nullptr, nullptr, 0,
                                         rcache_.as<uint2>(), ctr, st);
  scan_u32_u64(counts_.as<uint32_t>(), offs_.as<uint64_t>(), np, tmp_, s);
  uint64_t nr = 0;
  SPJ_CUDA(cudaMemcpyAsync(&nr, offs_.as<uint64_t>() + np, 8, cudaMemcpyDeviceToHost, s));
  check_status(scratch_, s, "learned query");  // syncs
  check_traversal(tv_, s);
  ranges_.reserve((nr + 1) * sizeof(uint4), s);
  k_learned_ranges<1><<<ga, 128, 0, s>>>(v, tv_, probe, predicate, order_.as<uint32_t>(), nullptr,
                                         offs_.as<uint64_t>(), ranges_.as<uint4>(), nr,
                                         rcache_.as<uint2>(), ctr, st);
  SPJ_CUDA(cudaEventRecord(ev_[2], s));
  // phase B: candidates of the ranges, a warp per 32 ranges
  const uint64_t nch = (nr + 31) / 32;
  ccount_.reserve((nch + 1) * 4, s);
  coff_.reserve((nch + 1) * 8, s);
  cwords_.reserve((nch + 1) * 4, s);
  woff_.reserve((nch + 1) * 8, s);
  const int gb = grid_for((int64_t)(nch * 32), 128, kNumSMs * 16);
  uint64_t total = 0;
  if (nch) {
    stats_.kernel_launches += 1 + 3 + 2 + 3;
    k_chunk_words<<<gb, 128, 0, s>>>(ranges_.as<uint4>(), nr, cwords_.as<uint32_t>());
    scan_u32_u64(cwords_.as<uint32_t>(), woff_.as<uint64_t>(), (int64_t)nch, tmp_, s);
    uint64_t nw = 0;
    SPJ_CUDA(cudaMemcpyAsync(&nw, woff_.as<uint64_t>() + nch, 8, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    masks_.reserve((nw + 1) * 4, s);
    k_learned_eval<0><<<gb, 128, 0, s>>>(v, tv_, bv_, probe, probe_base, predicate,
                                         ranges_.as<uint4>(), nr, ccount_.as<uint32_t>(), nullptr,
                                         woff_.as<uint64_t>(), masks_.as<uint32_t>(), nw, nullptr,
                                         nullptr, 0, ctr);
    scan_u32_u64(ccount_.as<uint32_t>(), coff_.as<uint64_t>(), (int64_t)nch, tmp_, s);
    SPJ_CUDA(cudaMemcpyAsync(&total, coff_.as<uint64_t>() + nch, 8, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    out_build.reserve((total + 1) * 4, s);
    out_probe.reserve((total + 1) * 4, s);
    k_learned_eval<1><<<gb, 128, 0, s>>>(v, tv_, bv_, probe, probe_base, predicate,
                                         ranges_.as<uint4>(), nr, nullptr, coff_.as<uint64_t>(),
                                         woff_.as<uint64_t>(), masks_.as<uint32_t>(), nw,
                                         out_build.as<uint32_t>(), out_probe.as<uint32_t>(), total,
                                         ctr);
  } else {
    out_build.reserve(4, s);
    out_probe.reserve(4, s);
  }
  SPJ_CUDA(cudaEventRecord(ev_[3], s));
  unsigned long long h[8];
  SPJ_CUDA(cudaMemcpyAsync(h, counters_.get(), 64, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  SPJ_CUDA(cudaGetLastError());
  check_traversal(tv_, s);
  stats_.lookups += h[0];
  stats_.window_misses += h[1];
  stats_.lbvh_fallbacks += h[2];
  stats_.search_steps += h[3];
  stats_.ranges += nr;
  float ms = 0;
  cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
  stats_.ms_order += ms;
  cudaEventElapsedTime(&ms, ev_[1], ev_[2]);
  stats_.ms_ranges += ms;
  cudaEventElapsedTime(&ms, ev_[2], ev_[3]);
  stats_.ms_eval += ms;
  return total;
}

void LearnedIndex::export_model(std::vector<uint32_t>& keys, std::vector<uint32_t>& leaf_start,
                                std::vector<uint32_t>& leaf_kc, std::vector<double>& a,
                                std::vector<double>& b, std::vector<uint32_t>& err,
                                cudaStream_t s) {
  keys.resize(n_);
  leaf_start.resize(L_ + 1);
  leaf_kc.resize(L_);
  a.resize(L_);
  b.resize(L_);
  err.resize(L_);
  if (n_) SPJ_CUDA(cudaMemcpyAsync(keys.data(), keys_.get(), (size_t)n_ * 4, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(leaf_start.data(), leaf_start_.get(), ((size_t)L_ + 1) * 4,
                           cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(leaf_kc.data(), leaf_kc_.get(), (size_t)L_ * 4, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(a.data(), leaf_a_.get(), (size_t)L_ * 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(b.data(), leaf_b_.get(), (size_t)L_ * 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(err.data(), leaf_err_.get(), (size_t)L_ * 4, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
}

}  // namespace spj
