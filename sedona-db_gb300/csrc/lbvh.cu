// lbvh.cu — LBVH build (Morton keys, device radix sort, Karras node emit,
// bottom-up refit) and the two-pass probe traversal.
#include "lbvh.cuh"
#include "prims.cuh"

#include <algorithm>

namespace spj {
namespace {

__device__ __forceinline__ bool box_valid(float4 b) {
  return b.x <= b.z && b.y <= b.w;  // false for NaN
}

__device__ __forceinline__ float4 box_union(float4 a, float4 b) {
  return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fmaxf(a.z, b.z), fmaxf(a.w, b.w));
}

// order-preserving float <-> u32 map for atomic min/max
__device__ __forceinline__ uint32_t f2o(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float o2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
#else
  uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
  float f;
  memcpy(&f, &v, 4);
  return f;
#endif
}

__global__ void k_valid_flags(const float4* __restrict__ boxes, uint32_t n,
                              uint8_t* __restrict__ flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    flag[i] = box_valid(boxes[i]) ? 1 : 0;
}

__global__ void k_compact_ids(const uint8_t* __restrict__ flag, const uint64_t* __restrict__ pos,
                              uint32_t n, uint32_t* __restrict__ ids) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (flag[i]) ids[pos[i]] = (uint32_t)i;
}

__global__ void k_bounds(const float4* __restrict__ boxes, const uint32_t* __restrict__ ids,
                         uint32_t m, uint32_t* __restrict__ ext) {
  float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 b = boxes[ids[i]];
    float cx = 0.5f * (b.x + b.z), cy = 0.5f * (b.y + b.w);
    mnx = fminf(mnx, cx);
    mny = fminf(mny, cy);
    mxx = fmaxf(mxx, cx);
    mxy = fmaxf(mxy, cy);
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

__device__ __forceinline__ uint32_t spread16(uint32_t v) {
  v &= 0xFFFFu;
  v = (v | (v << 8)) & 0x00FF00FFu;
  v = (v | (v << 4)) & 0x0F0F0F0Fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}

__global__ void k_morton(const float4* __restrict__ boxes, const uint32_t* __restrict__ ids,
                         uint32_t m, const uint32_t* __restrict__ ext, uint32_t* __restrict__ keys) {
  const float x0 = o2f(ext[0]), y0 = o2f(ext[1]), x1 = o2f(ext[2]), y1 = o2f(ext[3]);
  const float sx = x1 > x0 ? 65535.0f / (x1 - x0) : 0.0f;
  const float sy = y1 > y0 ? 65535.0f / (y1 - y0) : 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 b = boxes[ids[i]];
    float cx = 0.5f * (b.x + b.z), cy = 0.5f * (b.y + b.w);
    uint32_t qx = (uint32_t)fminf(fmaxf((cx - x0) * sx, 0.0f), 65535.0f);
    uint32_t qy = (uint32_t)fminf(fmaxf((cy - y0) * sy, 0.0f), 65535.0f);
    keys[i] = (spread16(qy) << 1) | spread16(qx);
  }
}

__global__ void k_gather_boxes(const float4* __restrict__ boxes, const uint32_t* __restrict__ ids,
                               uint32_t m, float4* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = boxes[ids[i]];
}

// Karras (2012) node emit over leaf keys made unique by the leaf index.
__device__ __forceinline__ int delta(const uint32_t* keys, uint32_t L, uint32_t ls, int i, int j) {
  if (j < 0 || j >= (int)L) return -1;
  uint32_t a = keys[(size_t)i * ls], b = keys[(size_t)j * ls];
  if (a != b) return __clz(a ^ b);
  return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

__global__ void k_karras(const uint32_t* __restrict__ keys, uint32_t L, uint32_t ls,
                         int2* __restrict__ child, int* __restrict__ parent_int,
                         int* __restrict__ parent_leaf) {
  for (int64_t ii = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ii < (int64_t)L - 1;
       ii += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)ii;
    const int d = (delta(keys, L, ls, i, i + 1) - delta(keys, L, ls, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, L, ls, i, i - d);
    int lmax = 2;
    while (delta(keys, L, ls, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
      if (delta(keys, L, ls, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, L, ls, i, j);
    int sp = 0;
    int t = l;
    do {
      t = (t + 1) >> 1;
      if (delta(keys, L, ls, i, i + (sp + t) * d) > dnode) sp += t;
    } while (t > 1);
    const int gamma = i + sp * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    int left = (lo == gamma) ? ~gamma : gamma;
    int right = (hi == gamma + 1) ? ~(gamma + 1) : (gamma + 1);
    child[i] = make_int2(left, right);
    if (left < 0) parent_leaf[~left] = (i << 1) | 0;
    else parent_int[left] = (i << 1) | 0;
    if (right < 0) parent_leaf[~right] = (i << 1) | 1;
    else parent_int[right] = (i << 1) | 1;
  }
}

// Bottom-up refit: each leaf computes its box, writes it into its parent's
// child slot, and the second thread to arrive at a node carries on upward.
__global__ void k_refit(const float4* __restrict__ sbox, uint32_t m, uint32_t L, uint32_t ls,
                        const int* __restrict__ parent_int, const int* __restrict__ parent_leaf,
                        float4* __restrict__ node_box, unsigned* __restrict__ visits) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < L;
       c += (int64_t)gridDim.x * blockDim.x) {
    uint32_t b0 = (uint32_t)c * ls, b1 = min(b0 + ls, m);
    float4 bb = sbox[b0];
    for (uint32_t k = b0 + 1; k < b1; k++) bb = box_union(bb, sbox[k]);
    int slot = parent_leaf[c];
    while (true) {
      int node = slot >> 1;
      node_box[slot] = bb;
      __threadfence();
      unsigned prev = atomicAdd(&visits[node], 1u);
      if (prev == 0) break;  // sibling not done yet; it will continue
      __threadfence();
      // the sibling's box was written by another SM: read past L1
      float4 a = __ldcg(&node_box[2 * node]), b = __ldcg(&node_box[2 * node + 1]);
      bb = box_union(a, b);
      if (node == 0) break;  // root
      slot = parent_int[node];
    }
  }
}

__global__ void k_leaf_boxes(const float4* __restrict__ sbox, uint32_t m, uint32_t L, uint32_t ls,
                             float4* __restrict__ out) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < L; c += gridDim.x * blockDim.x) {
    const uint32_t b0 = c * ls, b1 = min(b0 + ls, m);
    float4 bb = sbox[b0];
    for (uint32_t k = b0 + 1; k < b1; k++) bb = box_union(bb, sbox[k]);
    out[c] = bb;
  }
}

// ---------------------------------------------------------------------------
// traversal

template <bool kScatter>
__global__ void __launch_bounds__(kTravThreads)
    k_probe(LbvhView t, const float4* __restrict__ probe_box, uint32_t nprobe,
            uint32_t* __restrict__ counts, const uint64_t* __restrict__ offs, uint32_t probe_base,
            uint32_t* __restrict__ out_build, uint32_t* __restrict__ out_probe,
            uint64_t cap = ~0ull, const uint32_t* __restrict__ order = nullptr) {
  // per-thread stack in shared memory, [depth][thread] so a warp's pushes hit
  // 32 distinct banks
  __shared__ int stack[kTravStack * kTravThreads];
  __shared__ uint32_t runbuf[kScatter ? kRunBuf * kTravThreads : 1];
  // a traversal visits each node at most once: 2 * nleaves steps bound it
  const uint64_t max_steps = 2ull * t.nleaves + 2;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nprobe;
       j += (int64_t)gridDim.x * blockDim.x) {
    // with an order, thread slot j takes the j-th probe in Morton order of the
    // box centres: a warp's 32 traversals then visit neighbouring subtrees
    // (less divergence, node boxes shared through L1).  Counts and offsets
    // stay indexed by probe row, so the output layout does not change.
    const int64_t pi = order ? (int64_t)order[j] : j;
    if (pi < 0 || pi >= nprobe) {
      traversal_fault(t, kBadProbe, (unsigned)pi);
      continue;
    }
    const float4 q = probe_box[pi];
    uint32_t cnt = 0;
    uint64_t pos = kScatter ? offs[pi] : 0;
    int staged = 0;  // build ids staged in runbuf (scatter pass)
    if (box_valid(q) && t.nprims > 0) {
      int sp = 0;
      int node = t.nleaves > 1 ? 0 : ~0;  // root: internal node 0, or the single leaf
      uint64_t steps = 0;
      while (true) {
        if (++steps > max_steps) {
          traversal_fault(t, kTooLong, (unsigned)pi);
          break;
        }
        if (node < 0) {
          const uint32_t c = (uint32_t)(~node);
          if (c >= t.nleaves) {
            traversal_fault(t, kBadLeaf, c);
            break;
          }
          const uint32_t b0 = c * t.leaf_size;
          const uint32_t b1 = min(b0 + t.leaf_size, t.nprims);
          for (uint32_t k = b0; k < b1; k++) {
            if (box_overlap(t.sorted_box[k], q)) {
              if (kScatter) {
                // writes bounded by the output capacity
                if (out_probe && pos < cap) out_probe[pos] = (uint32_t)pi + probe_base;
                run_put(out_build, cap, runbuf, pos, staged, t.sorted_id[k]);
              } else {
                cnt++;
              }
            }
          }
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
              traversal_fault(t, kStackOverflow, (unsigned)pi);
              break;
            }
            stack[sp * kTravThreads + threadIdx.x] = ch.y;
            sp++;
            node = ch.x;
            continue;
          }
          if (hl) {
            node = ch.x;
            continue;
          }
          if (hr) {
            node = ch.y;
            continue;
          }
        }
        if (sp == 0) break;
        sp--;
        node = stack[sp * kTravThreads + threadIdx.x];
      }
    }
    if (kScatter && staged) run_flush(out_build, cap, runbuf, pos, staged);
    if (!kScatter) counts[pi] = cnt;
  }
}

__global__ void k_expand(GeomsView G, double d0, const double* __restrict__ d_row,
                         float4* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < G.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float q = __int_as_float(0x7fc00000);
    float4 o = make_float4(q, q, q, q);
    const double d = d_row ? d_row[i] : d0;
    const uint8_t k = G.kind[i];
    if (k != 0 && d >= 0) {
      // the row's exact bounds (a point's coordinates, a polygon's ring
      // rects), expanded by d in FP64, then rounded outward
      double2 mn, mx;
      if (k == 1) {
        mn = mx = G.pt[i];
      } else {
        mn = make_double2(INFINITY, INFINITY);
        mx = make_double2(-INFINITY, -INFINITY);
        const uint32_t r0 = G.part_ring[G.row_part[i]], r1 = G.part_ring[G.row_part[i + 1]];
        for (uint32_t r = r0; r < r1; r++) {
          const Rect64 R = G.ring_rect[r];
          mn.x = fmin(mn.x, R.x);
          mn.y = fmin(mn.y, R.y);
          mx.x = fmax(mx.x, R.z);
          mx.y = fmax(mx.y, R.w);
        }
      }
      double lo[2] = {mn.x - d, mn.y - d}, hi[2] = {mx.x + d, mx.y + d};
      float fl[2], fh[2];
      for (int a = 0; a < 2; a++) {
        float x = __double2float_rn(lo[a]), y = __double2float_rn(hi[a]);
        if ((double)x > lo[a]) x = next_downf(x);
        if ((double)y < hi[a]) y = next_upf(y);
        fl[a] = x;
        fh[a] = y;
      }
      o = make_float4(fl[0], fl[1], fh[0], fh[1]);
    }
    out[i] = o;
  }
}

// The tree's root box and the scale of a 16-bit grid over it.
struct RootGrid {
  float4 r;
  float sx, sy;
  __device__ explicit RootGrid(const LbvhView& t) {
    if (t.nleaves > 1) {
      r = box_union(t.node_box[0], t.node_box[1]);
    } else {
      r = t.sorted_box[0];
      for (uint32_t k = 1; k < t.nprims; k++) r = box_union(r, t.sorted_box[k]);
    }
    sx = r.z > r.x ? 65535.0f / (r.z - r.x) : 0.0f;
    sy = r.w > r.y ? 65535.0f / (r.w - r.y) : 0.0f;
  }
  __device__ uint32_t key(float cx, float cy) const {
    const uint32_t qx = (uint32_t)fminf(fmaxf((cx - r.x) * sx, 0.0f), 65535.0f);
    const uint32_t qy = (uint32_t)fminf(fmaxf((cy - r.y) * sy, 0.0f), 65535.0f);
    return (spread16(qy) << 1) | spread16(qx);
  }
};

// Morton key (16 bits per axis) of each probe box centre over the tree's
// root box, with the probe row as the value; empty (NaN) boxes sort last.
__global__ void k_probe_keys(LbvhView t, const float4* __restrict__ probe_box, uint32_t n,
                             uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const RootGrid g(t);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float4 b = probe_box[i];
    keys[i] = box_valid(b) ? g.key(0.5f * b.x + 0.5f * b.z, 0.5f * b.y + 0.5f * b.w)
                           : 0xFFFFFFFFu;
    vals[i] = (uint32_t)i;
  }
}

// The same over FP64 points (their RN32 coordinates); NaN points sort last.
__global__ void k_point_keys(LbvhView t, const double2* __restrict__ xy, uint32_t n,
                             uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const RootGrid g(t);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 p = xy[i];
    keys[i] = isnan(p.x) || isnan(p.y)
                  ? 0xFFFFFFFFu
                  : g.key(__double2float_rn(p.x), __double2float_rn(p.y));
    vals[i] = (uint32_t)i;
  }
}

// out_probe[e] = row + probe_base for every e in [offs[row], offs[row + 1]).
// A warp takes 32 consecutive rows, whose runs form one contiguous range,
// and writes it with coalesced stores, each lane finding the row of its
// element by a 5-step search over the rows' starts.
__global__ void k_fill_probe_ids(const uint64_t* __restrict__ offs, uint32_t n,
                                 uint32_t probe_base, uint32_t* __restrict__ out, uint64_t cap) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; w * 32 < n; w += nw) {
    const uint64_t row = w * 32 + lane;
    const uint64_t st = row < n ? offs[row] : ~0ull;
    const uint64_t r_end = w * 32 + 32 < n ? w * 32 + 32 : n;
    const uint64_t e0 = __shfl_sync(0xffffffffu, st, 0);
    const uint64_t e1 = offs[r_end];
    for (uint64_t base = e0; base < e1; base += 32) {
      const uint64_t e = base + lane;
      int L = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const uint64_t sL = __shfl_sync(0xffffffffu, st, L + step);
        if (sL <= e) L += step;
      }
      if (e < e1 && e < cap) out[e] = (uint32_t)(w * 32 + L) + probe_base;
    }
  }
}

__global__ void k_gather_counts(const uint32_t* __restrict__ order,
                                const uint32_t* __restrict__ counts, uint32_t n,
                                uint32_t* __restrict__ out) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    out[j] = counts[order[j]];
}

// perm[opos[j] + c] = offs[order[j]] + c for c < counts[order[j]] (and, with
// keys, keys[...] = cb[that candidate]).  A warp
// takes 32 consecutive positions j, and its lanes write consecutive perm
// entries (each finds its position by a binary search over the 32 run
// starts), so the stores are coalesced.
__global__ void k_cand_perm(const uint32_t* __restrict__ order, const uint32_t* __restrict__ counts,
                            const uint64_t* __restrict__ offs, const uint64_t* __restrict__ opos,
                            uint32_t n, uint64_t m, uint32_t* __restrict__ perm,
                            const uint32_t* __restrict__ cb = nullptr,
                            uint32_t* __restrict__ keys = nullptr) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; w * 32 < n; w += nw) {
    const uint64_t j = w * 32 + lane;
    const uint32_t pi = j < n ? order[j] : 0xFFFFFFFFu;
    const bool ok = pi < n;
    // this lane's run: [st, st + c) of perm, taken from offs[pi]
    const uint64_t st = j < n ? opos[j] : ~0ull;
    const uint64_t src0 = ok ? offs[pi] : 0;
    const uint32_t c = ok ? counts[pi] : 0;
    const uint64_t jend = w * 32 + 32 < n ? w * 32 + 32 : n;
    const uint64_t e0 = __shfl_sync(0xffffffffu, st, 0);
    const uint64_t e1 = opos[jend];
    for (uint64_t base = e0; base < e1; base += 32) {
      const uint64_t e = base + lane;
      int L = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const uint64_t sL = __shfl_sync(0xffffffffu, st, L + step);
        if (sL <= e) L += step;
      }
      const uint64_t sr = __shfl_sync(0xffffffffu, st, L);
      const uint64_t src = __shfl_sync(0xffffffffu, src0, L) + (e - sr);
      const uint32_t cl = __shfl_sync(0xffffffffu, c, L);
      const bool okl = __shfl_sync(0xffffffffu, ok ? 1 : 0, L) != 0;
      if (e < e1 && okl && e - sr < cl && e < m && src < m) {
        perm[e] = (uint32_t)src;
        if (keys) keys[e] = cb[src];  // the build row, gathered on the way
      }
    }
  }
}

}  // namespace

void fill_probe_ids(const uint64_t* offs, uint32_t n, uint32_t probe_base, uint32_t* out,
                    uint64_t cap, cudaStream_t s) {
  if (n == 0) return;
  k_fill_probe_ids<<<grid_for((int64_t)n, 256), 256, 0, s>>>(offs, n, probe_base, out, cap);
  SPJ_CUDA(cudaGetLastError());
}

void reserve_candidate_order(uint32_t nprobe, uint64_t mcap, ProbeScratch& sc,
                             cudaStream_t s) {
  sc.ocount.reserve(((size_t)nprobe + 1) * 4, s);
  sc.opos.reserve(((size_t)nprobe + 1) * 8, s);
  sc.cperm.reserve((mcap + 1) * 4, s);
  sc.tmp.reserve(std::max(scan_tile_sums_bytes(nprobe), radix_sort_tmp_bytes(nprobe)), s);
}

const uint32_t* candidate_order_into(const uint32_t* order, const uint32_t* counts,
                                     const uint64_t* offs, uint32_t nprobe, uint64_t mcap,
                                     ProbeScratch& sc, cudaStream_t s) {
  if (!order || nprobe == 0 || mcap == 0 || mcap >= 0xFFFFFFFFull) return nullptr;
  reserve_candidate_order(nprobe, mcap, sc, s);
  const int g = grid_for(nprobe, 256);
  k_gather_counts<<<g, 256, 0, s>>>(order, counts, nprobe, sc.ocount.as<uint32_t>());
  scan_u32_u64_into(sc.ocount.as<uint32_t>(), sc.opos.as<uint64_t>(), nprobe,
                    sc.tmp.as<uint64_t>(), s);
  k_cand_perm<<<g, 256, 0, s>>>(order, counts, offs, sc.opos.as<uint64_t>(), nprobe, mcap,
                                sc.cperm.as<uint32_t>());
  SPJ_CUDA(cudaGetLastError());
  return sc.cperm.as<uint32_t>();
}

const uint32_t* candidate_order(const uint32_t* order, uint32_t nprobe, uint64_t m,
                                ProbeScratch& sc, cudaStream_t s, const uint32_t* cb,
                                uint32_t* keys) {
  if (!order || nprobe == 0 || m == 0 || m >= 0xFFFFFFFFull) return nullptr;
  sc.ocount.reserve(((size_t)nprobe + 1) * 4, s);
  sc.opos.reserve(((size_t)nprobe + 1) * 8, s);
  sc.cperm.reserve((m + 1) * 4, s);
  const int g = grid_for(nprobe, 256);
  k_gather_counts<<<g, 256, 0, s>>>(order, sc.counts.as<uint32_t>(), nprobe,
                                    sc.ocount.as<uint32_t>());
  scan_u32_u64(sc.ocount.as<uint32_t>(), sc.opos.as<uint64_t>(), nprobe, sc.tmp, s);
  k_cand_perm<<<g, 256, 0, s>>>(order, sc.counts.as<uint32_t>(), sc.offsets.as<uint64_t>(),
                                sc.opos.as<uint64_t>(), nprobe, m, sc.cperm.as<uint32_t>(), cb,
                                keys);
  SPJ_CUDA(cudaGetLastError());
  return sc.cperm.as<uint32_t>();
}

namespace {

__global__ void k_rank(const uint32_t* __restrict__ order, uint32_t n, uint32_t* __restrict__ rank) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const uint32_t pi = order[j];
    if (pi < n) rank[pi] = j;
  }
}

// key = build id above rbits bits of the probe's Morton rank (scaled), or
// the build id alone (rbits = 0)
__global__ void k_cand_keys(const uint32_t* __restrict__ cb, const uint32_t* __restrict__ cp,
                            uint64_t m, uint32_t probe_base, const uint32_t* __restrict__ rank,
                            uint32_t n, int rbits, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < m;
       k += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t b = cb[k];
    uint32_t key = b;
    if (rbits > 0) {
      const uint32_t p = cp[k] - probe_base;
      const uint32_t r = rank && p < n ? rank[p] : p;
      key = (b << rbits) | (uint32_t)(((uint64_t)r << rbits) / (n ? n : 1));
    }
    keys[k] = key;
    vals[k] = (uint32_t)k;
  }
}

}  // namespace


const uint32_t* build_major_order(const uint32_t* cb, const uint32_t* cp, uint64_t m,
                                  uint32_t probe_base, uint32_t nbuild, const uint32_t* order,
                                  uint32_t nprobe, uint64_t tiles, ProbeScratch& sc,
                                  cudaStream_t s) {
  if (m < 2 || m >= 0xFFFFFFFFull) return nullptr;
  int bb = 1;
  while (bb < 32 && (nbuild - 1) >> bb) bb++;
  if (order && bb <= 24) {
    // the candidates listed in the probes' Morton order (k_cand_perm, coalesced),
    // then a stable sort of that list by build row alone: build row, then the
    // probe's full Morton rank, with ceil(bits / 8) radix passes; with tiles,
    // each tile of the list is sorted in place by the same passes
    sc.ckeys.reserve((m + 1) * 4, s);
    const uint32_t* mperm = candidate_order(order, nprobe, m, sc, s, cb, sc.ckeys.as<uint32_t>());
    if (mperm) {
      sc.ckeys_alt.reserve((m + 1) * 4, s);
      sc.cvals_alt.reserve((m + 1) * 4, s);
      radix_sort_pairs(sc.ckeys.as<uint32_t>(), sc.cperm.as<uint32_t>(),
                       sc.ckeys_alt.as<uint32_t>(), sc.cvals_alt.as<uint32_t>(), (int64_t)m,
                       bb, sc.tmp, s, (int64_t)tiles, false);
      SPJ_CUDA(cudaGetLastError());
      return sc.cperm.as<uint32_t>();
    }
  }
  // build id bits, then the probe's Morton rank in the remaining bits of a
  // 32-bit key (its resolution matters: 8 rank bits for 50k build rows gave
  // 98 ms per step on 2M x 50k polygons, 16 bits 77 ms)
  int bbits = 1;
  while (bbits < 32 && (nbuild - 1) >> bbits) bbits++;
  const int total = 32;
  const int rbits = bbits <= 24 ? total - bbits : 0;
  const bool wide = rbits == 0;
  sc.cperm.reserve((m + 1) * 4, s);
  sc.ckeys.reserve((m + 1) * 4, s);
  sc.ckeys_alt.reserve((m + 1) * 4, s);
  sc.cvals_alt.reserve((m + 1) * 4, s);
  const uint32_t* rank = nullptr;
  if (order && !wide) {
    sc.rank.reserve(((size_t)nprobe + 1) * 4, s);
    k_rank<<<grid_for(nprobe, 256), 256, 0, s>>>(order, nprobe, sc.rank.as<uint32_t>());
    rank = sc.rank.as<uint32_t>();
  }
  k_cand_keys<<<grid_for((int64_t)m, 256), 256, 0, s>>>(cb, cp, m, probe_base, rank, nprobe,
                                                      rbits, sc.ckeys.as<uint32_t>(),
                                                      sc.cperm.as<uint32_t>());
  radix_sort_pairs(sc.ckeys.as<uint32_t>(), sc.cperm.as<uint32_t>(), sc.ckeys_alt.as<uint32_t>(),
                   sc.cvals_alt.as<uint32_t>(), (int64_t)m, total, sc.tmp, s);
  SPJ_CUDA(cudaGetLastError());
  return sc.cperm.as<uint32_t>();
}

void reserve_candidate_keys(uint64_t m, ProbeScratch& sc, cudaStream_t s) {
  sc.cperm.reserve((m + 1) * 4, s);
  sc.ckeys.reserve((m + 1) * 4, s);
  sc.ckeys_alt.reserve((m + 1) * 4, s);
  sc.cvals_alt.reserve((m + 1) * 4, s);
}

const uint32_t* sort_candidate_keys(uint64_t m, int key_bits, ProbeScratch& sc, cudaStream_t s) {
  radix_sort_pairs(sc.ckeys.as<uint32_t>(), sc.cperm.as<uint32_t>(), sc.ckeys_alt.as<uint32_t>(),
                   sc.cvals_alt.as<uint32_t>(), (int64_t)m, key_bits, sc.tmp, s);
  SPJ_CUDA(cudaGetLastError());
  return sc.cperm.as<uint32_t>();
}

static const uint32_t* sort_order(uint32_t n, ProbeScratch& sc, cudaStream_t s) {
  radix_sort_pairs(sc.okeys.as<uint32_t>(), sc.order.as<uint32_t>(), sc.akeys.as<uint32_t>(),
                   sc.avals.as<uint32_t>(), n, 32, sc.tmp, s);
  SPJ_CUDA(cudaGetLastError());
  return sc.order.as<uint32_t>();
}

static void reserve_order(uint32_t n, ProbeScratch& sc, cudaStream_t s) {
  const size_t bytes = ((size_t)n + 1) * 4;
  sc.order.reserve(bytes, s);
  sc.okeys.reserve(bytes, s);
  sc.akeys.reserve(bytes, s);
  sc.avals.reserve(bytes, s);
}

void reserve_probe_order(uint32_t nprobe, ProbeScratch& sc, cudaStream_t s) {
  reserve_order(nprobe, sc, s);
  sc.tmp.reserve(std::max(scan_tile_sums_bytes(nprobe), radix_sort_tmp_bytes(nprobe)), s);
}

const uint32_t* probe_order(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                            ProbeScratch& sc, cudaStream_t s) {
  if (nprobe < 2 || t.nprims == 0) return nullptr;
  reserve_order(nprobe, sc, s);
  k_probe_keys<<<grid_for(nprobe, 256), 256, 0, s>>>(t, probe_box, nprobe, sc.okeys.as<uint32_t>(),
                                                     sc.order.as<uint32_t>());
  return sort_order(nprobe, sc, s);
}

const uint32_t* point_order(const LbvhView& t, const double2* xy, uint32_t n, ProbeScratch& sc,
                            cudaStream_t s) {
  if (n < 2 || t.nprims == 0) return nullptr;
  reserve_order(n, sc, s);
  k_point_keys<<<grid_for(n, 256), 256, 0, s>>>(t, xy, n, sc.okeys.as<uint32_t>(),
                                                sc.order.as<uint32_t>());
  return sort_order(n, sc, s);
}

void build_lbvh(const float4* boxes, uint32_t n, uint32_t leaf_size, Lbvh& out, cudaStream_t s) {
  SPJ_CHECK(leaf_size >= 1 && leaf_size <= 64, "leaf size must be in [1, 64]");
  out.leaf_size = leaf_size;
  DevBuf flag((size_t)n + 1, s), pos(((size_t)n + 1) * 8, s), tmp;
  const int g = grid_for(n, 256);
  k_valid_flags<<<g, 256, 0, s>>>(boxes, n, flag.as<uint8_t>());
  scan_u8_u64(flag.as<uint8_t>(), pos.as<uint64_t>(), n, tmp, s);
  uint64_t m64 = 0;
  SPJ_CUDA(cudaMemcpyAsync(&m64, pos.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  const uint32_t m = (uint32_t)m64;
  out.nprims = m;
  out.nleaves = m ? (m + leaf_size - 1) / leaf_size : 0;
  out.sorted_box.reserve(((size_t)m + 1) * sizeof(float4), s);
  out.sorted_id.reserve(((size_t)m + 1) * 4, s);
  const uint32_t L = out.nleaves;
  out.node_box.reserve((size_t)(L > 1 ? 2 * (L - 1) : 1) * sizeof(float4), s);
  out.node_child.reserve((size_t)(L > 1 ? L - 1 : 1) * sizeof(int2), s);
  out.leaf_box.reserve((size_t)(L > 0 ? L : 1) * sizeof(float4), s);
  out.fault.reserve(8, s);
  SPJ_CUDA(cudaMemsetAsync(out.fault.get(), 0, 8, s));
  if (m == 0) return;
  uint32_t* ids = out.sorted_id.as<uint32_t>();
  k_compact_ids<<<g, 256, 0, s>>>(flag.as<uint8_t>(), pos.as<uint64_t>(), n, ids);
  DevBuf ext(16, s);
  uint32_t init[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u};
  SPJ_CUDA(cudaMemcpyAsync(ext.get(), init, 16, cudaMemcpyHostToDevice, s));
  const int gm = grid_for(m, 256);
  k_bounds<<<gm, 256, 0, s>>>(boxes, ids, m, ext.as<uint32_t>());
  DevBuf keys((size_t)m * 4, s), akeys((size_t)m * 4, s), avals((size_t)m * 4, s);
  k_morton<<<gm, 256, 0, s>>>(boxes, ids, m, ext.as<uint32_t>(), keys.as<uint32_t>());
  radix_sort_pairs(keys.as<uint32_t>(), ids, akeys.as<uint32_t>(), avals.as<uint32_t>(), m, 32,
                   tmp, s);
  k_gather_boxes<<<gm, 256, 0, s>>>(boxes, ids, m, out.sorted_box.as<float4>());
  k_leaf_boxes<<<grid_for(L, 256), 256, 0, s>>>(out.sorted_box.as<float4>(), m, L, leaf_size,
                                                out.leaf_box.as<float4>());
  if (L > 1) {
    DevBuf parent_int((size_t)L * 4, s), parent_leaf((size_t)L * 4, s), visits((size_t)L * 4, s);
    SPJ_CUDA(cudaMemsetAsync(visits.get(), 0, (size_t)L * 4, s));
    k_karras<<<grid_for(L - 1, 256), 256, 0, s>>>(keys.as<uint32_t>(), L, leaf_size,
                                                  out.node_child.as<int2>(),
                                                  parent_int.as<int>(), parent_leaf.as<int>());
    k_refit<<<grid_for(L, 256), 256, 0, s>>>(out.sorted_box.as<float4>(), m, L, leaf_size,
                                             parent_int.as<int>(), parent_leaf.as<int>(),
                                             out.node_box.as<float4>(), visits.as<unsigned>());
  }
  SPJ_CUDA(cudaGetLastError());
  SPJ_CUDA(cudaStreamSynchronize(s));
}

void check_traversal(const LbvhView& t, cudaStream_t s) {
  if (!t.fault) return;
  unsigned f[2] = {0, 0};
  SPJ_CUDA(cudaMemcpyAsync(f, t.fault, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  static const char* what[] = {"", "an out-of-range leaf index", "an out-of-range node index",
                               "an out-of-range probe row", "more steps than the tree has nodes",
                               "a path deeper than its stack"};
  SPJ_CHECK(f[0] == 0, std::string("LBVH traversal met ") + what[f[0] < 6 ? f[0] : 0] + " (" +
                           std::to_string(f[1]) + ")");
}

uint64_t probe_count(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                     ProbeScratch& sc, cudaStream_t s, const uint32_t* order) {
  sc.counts.reserve(((size_t)nprobe + 1) * 4, s);
  sc.offsets.reserve(((size_t)nprobe + 1) * 8, s);
  if (nprobe == 0) return 0;
  const int g = grid_for(nprobe, kTravThreads, kNumSMs * 16);
  k_probe<false><<<g, kTravThreads, 0, s>>>(t, probe_box, nprobe, sc.counts.as<uint32_t>(),
                                            nullptr, 0, nullptr, nullptr, ~0ull, order);
  scan_u32_u64(sc.counts.as<uint32_t>(), sc.offsets.as<uint64_t>(), nprobe, sc.tmp, s);
  uint64_t total = 0;
  SPJ_CUDA(cudaMemcpyAsync(&total, sc.offsets.as<uint64_t>() + nprobe, 8, cudaMemcpyDeviceToHost,
                           s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  check_traversal(t, s);
  return total;
}

void probe_scatter(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                   const ProbeScratch& sc, uint32_t probe_base, uint32_t* out_build,
                   uint32_t* out_probe, cudaStream_t s, const uint32_t* order) {
  if (nprobe == 0) return;
  const int g = grid_for(nprobe, kTravThreads, kNumSMs * 16);
  k_probe<true><<<g, kTravThreads, 0, s>>>(t, probe_box, nprobe, nullptr,
                                           sc.offsets.as<uint64_t>(), probe_base, out_build,
                                           nullptr, ~0ull, order);
  SPJ_CUDA(cudaGetLastError());
  fill_probe_ids(sc.offsets.as<uint64_t>(), nprobe, probe_base, out_probe, ~0ull, s);
}

void probe_count_into(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                      uint32_t* counts, cudaStream_t s, const uint32_t* order) {
  if (nprobe == 0) return;
  const int g = grid_for(nprobe, kTravThreads, kNumSMs * 16);
  k_probe<false><<<g, kTravThreads, 0, s>>>(t, probe_box, nprobe, counts, nullptr, 0, nullptr,
                                            nullptr, ~0ull, order);
  SPJ_CUDA(cudaGetLastError());
}

void probe_scatter_from(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                        const uint64_t* offs, uint32_t probe_base, uint32_t* out_build,
                        uint32_t* out_probe, cudaStream_t s, uint64_t capacity,
                        const uint32_t* order) {
  if (nprobe == 0) return;
  const int g = grid_for(nprobe, kTravThreads, kNumSMs * 16);
  k_probe<true><<<g, kTravThreads, 0, s>>>(t, probe_box, nprobe, nullptr, offs, probe_base,
                                           out_build, nullptr, capacity, order);
  SPJ_CUDA(cudaGetLastError());
  fill_probe_ids(offs, nprobe, probe_base, out_probe, capacity, s);
}

void expand_boxes(const GeomsView& g, double distance, const double* d_row, float4* out,
                  cudaStream_t s) {
  const uint32_t n = g.n;
  if (n == 0) return;
  k_expand<<<grid_for(n, 256), 256, 0, s>>>(g, distance, d_row, out);
  SPJ_CUDA(cudaGetLastError());
}

}  // namespace spj
