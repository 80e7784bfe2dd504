// dwithin.cu — fused ST_DWithin traversal over point columns.
#include "dwithin.cuh"
#include "exact.cuh"

#include <cstring>

namespace spj {
namespace {

// Error bound of the split FP32 distance r = sqrt(d2) against the true
// distance D of the FP64 points: |D - r| <= 2^-20 r + 2^-44 (max|b|_1 +
// |q|_1) + 2^-120.  Per axis, with u = 2^-24: v = hi + lo + e, |e| <= 2^-48
// |v|; the three FP32 roundings of (b.hi - q.hi) + (b.lo - q.lo) give
// |dx - (b - q).x| <= 2u (1 + 2u) |dx| + 3 * 2^-48 (|b.x| + |q.x|); the two axes
// add to <= 2^-22 |d| + 2^-46 (..); the square, sum and square root add
// 2^-23 relative.  2^-20 covers the relative part twice over, 2^-44 the
// absolute part four times over, 2^-120 FP32 results below the normal range.
constexpr float kSplitUp = 1.00000095367431640625f;    // 1 + 2^-20
constexpr float kSplitDown = 0.99999904632568359375f;  // 1 - 2^-20
constexpr float kTwoM44 = 5.684341886080801486968994140625e-14f;
constexpr float kTwoM120 = 7.5231638452626400509999138382223723380394595633413601376560e-37f;

__global__ void k_split_points(const double2* __restrict__ pts, uint32_t npts,
                               const uint32_t* __restrict__ ids, uint32_t m,
                               double2* __restrict__ xy, float4* __restrict__ hl,
                               unsigned* __restrict__ mag) {
  unsigned bm = 0, big = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint32_t id = ids[i];
    if (id >= npts) {  // not a row of the column: recorded, the host raises
      big |= 2u;
      continue;
    }
    const double2 p = pts[id];
    xy[i] = p;
    const float hx = __double2float_rn(p.x), hy = __double2float_rn(p.y);
    // v - RN32(v) is exact in FP64
    hl[i] = make_float4(hx, hy, __double2float_rn(__dsub_rn(p.x, (double)hx)),
                        __double2float_rn(__dsub_rn(p.y, (double)hy)));
    const double ax = fabs(p.x), ay = fabs(p.y);
    if (!(ax <= kSplitMaxCoord && ay <= kSplitMaxCoord)) big = 1;
    else bm = max(bm, __float_as_uint(__double2float_ru(__dadd_ru(ax, ay))));
  }
  for (int o = 16; o > 0; o >>= 1) {
    bm = max(bm, __shfl_xor_sync(0xffffffffu, bm, o));
    big |= __shfl_xor_sync(0xffffffffu, big, o);
  }
  if ((threadIdx.x & 31) == 0) {
    // non-negative floats order as their bit patterns
    if (bm) atomicMax(&mag[0], bm);
    if (big) atomicOr(&mag[1], big);
  }
}

// Whole-leaf decision from the leaf's f32 box (the union of its points'
// RN32 boxes): +1 when every point of the leaf is within d, -1 when every
// point is farther, 0 to test the points.  Per axis, the split difference of
// a box coordinate c (an exact f32) and the probe is within 2^-21 of itself
// plus 2^-46 |p| (the split analysis above, with no rounding of c), and a
// point lies within 2^-24 |RN32| of its RN32 copy inside the box (e); the
// bounds below add these to the farthest / nearest box offsets and decide
// with the same neighbours of d as the point test.  Points outside the
// probe's expanded box have no part in the result either way, so emitting a
// whole leaf in index order gives what the per-point loop gives.
__device__ __forceinline__ int leaf_class(float4 b, float hx, float hy, float lx, float ly,
                                          float cerr, float d_lo, float d_hi) {
  const float sx0 = __fsub_rn(__fsub_rn(b.x, hx), lx), sx1 = __fsub_rn(__fsub_rn(b.z, hx), lx);
  const float sy0 = __fsub_rn(__fsub_rn(b.y, hy), ly), sy1 = __fsub_rn(__fsub_rn(b.w, hy), ly);
  const float ex = __fadd_ru(__fmul_ru(fmaxf(fabsf(b.x), fabsf(b.z)), 5.9604645e-08f), cerr);
  const float ey = __fadd_ru(__fmul_ru(fmaxf(fabsf(b.y), fabsf(b.w)), 5.9604645e-08f), cerr);
  // farthest: |point - p| <= max(|s0|, |s1|) (1 + 2^-20) + e per axis
  const float fx = __fadd_ru(__fmul_ru(fmaxf(fabsf(sx0), fabsf(sx1)), kSplitUp), ex);
  const float fy = __fadd_ru(__fmul_ru(fmaxf(fabsf(sy0), fabsf(sy1)), kSplitUp), ey);
  const float up = __fmul_ru(__fsqrt_ru(__fadd_ru(__fmul_ru(fx, fx), __fmul_ru(fy, fy))), kSplitUp);
  if (up < d_lo) return 1;
  // nearest: the probe's offset outside the box, less the same errors
  const float nx = fmaxf(fmaxf(sx0, -sx1), 0.0f), ny = fmaxf(fmaxf(sy0, -sy1), 0.0f);
  const float nxl = fmaxf(__fsub_rd(__fmul_rd(nx, kSplitDown), ex), 0.0f);
  const float nyl = fmaxf(__fsub_rd(__fmul_rd(ny, kSplitDown), ey), 0.0f);
  const float lo =
      __fmul_rd(__fsqrt_rd(__fadd_rd(__fmul_rd(nxl, nxl), __fmul_rd(nyl, nyl))), kSplitDown);
  if (lo > d_hi) return -1;
  return 0;
}

// Appends one build id to the probe's arena chain (counting pass).
__device__ __forceinline__ void arena_put(const DwithinArena& A, uint32_t id, uint32_t& cur,
                                          uint32_t& first, uint32_t& fill, bool& failed) {
  if (failed) return;
  if (cur == kArenaEnd || fill == kArenaChunkWords - 1) {
    // one atomic per group of lanes that need a chunk at the same time (in
    // Morton order neighbouring lanes overflow together)
    const unsigned act = __activemask();
    const int lane = threadIdx.x & 31, leader = __ffs(act) - 1;
    unsigned long long b = 0;
    if (lane == leader) b = atomicAdd(A.cursor, (unsigned long long)__popc(act));
    b = __shfl_sync(act, b, leader);
    const unsigned long long nc64 = b + (unsigned)__popc(act & ((1u << lane) - 1u));
    if (nc64 >= A.chunks) {
      failed = true;
      return;
    }
    const uint32_t nc = (uint32_t)nc64;
    if (cur == kArenaEnd) first = nc;
    else A.words[(size_t)cur * kArenaChunkWords] = nc;
    cur = nc;
    fill = 0;
  }
  A.words[(size_t)cur * kArenaChunkWords + 1 + fill] = id;
  fill++;
}

template <bool kScatter, bool kArena>
__global__ void __launch_bounds__(kTravThreads)
    k_dwithin_fused(LbvhView t, const double2* __restrict__ bxy, const float4* __restrict__ bhl,
                    float bmag, int split_ok, const float4* __restrict__ probe_box,
                    const double2* __restrict__ probe_pt, uint32_t n, double d0, float d_lo0,
                    float d_hi0, const double* __restrict__ d_row,
                    const uint32_t* __restrict__ order, uint32_t* __restrict__ counts,
                    const uint64_t* __restrict__ offs, uint32_t probe_base,
                    uint32_t* __restrict__ out_build, uint32_t* __restrict__ out_probe,
                    uint64_t cap, DeviceStatus* st, uint32_t* __restrict__ slots, uint32_t K,
                    DwithinArena A) {
  __shared__ int stack[kTravStack * kTravThreads];
  // staged output runs: the scatter pass's pair run, the counting pass's
  // slot row (rows of K ids, so with K a multiple of kRunBuf its groups are
  // whole sectors)
  __shared__ uint32_t runbuf[kRunBuf * kTravThreads];
  const uint64_t max_steps = 2ull * t.nleaves + 2;
  uint32_t esc = 0, tested = 0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pi = order ? (int64_t)order[j] : j;
    if (pi < 0 || pi >= n) {
      traversal_fault(t, kBadProbe, (unsigned)pi);
      continue;
    }
    // the scatter pass only traverses the probes whose results did not all
    // fit in the counting pass's slots and arena
    if (kScatter && K > 0 && (counts[pi] <= K || (kArena && A.head[pi] != kArenaFailed)))
      continue;
    const float4 q = probe_box[pi];
    // the probe row's distance and its FP32 neighbours (the expanded box of
    // a row with a negative or NaN distance is empty: no traversal)
    double d = d0;
    float d_lo = d_lo0, d_hi = d_hi0;
    if (d_row) {
      d = d_row[pi];
      d_lo = __double2float_rn(d);
      d_hi = d_lo;
      if ((double)d_lo > d) d_lo = next_downf(d_lo);
      if ((double)d_hi < d) d_hi = next_upf(d_hi);
    }
    uint32_t cnt = 0;
    uint32_t a_cur = kArenaEnd, a_first = kArenaEnd, a_fill = 0;
    bool a_failed = false;
    uint64_t pos = kScatter ? offs[pi] : 0;
    // counting pass: the slot row [pi K, pi K + K)
    uint64_t spos = (uint64_t)pi * K;
    const uint64_t send = spos + K;
    int staged = 0;
    if (q.x <= q.z && q.y <= q.w && t.nprims > 0) {
      const double2 p = probe_pt[pi];
      const bool split =
          split_ok && fabs(p.x) <= kSplitMaxCoord && fabs(p.y) <= kSplitMaxCoord;
      float hx = 0, hy = 0, lx = 0, ly = 0, cerr = 0;
      if (split) {
        hx = __double2float_rn(p.x);
        hy = __double2float_rn(p.y);
        lx = __double2float_rn(__dsub_rn(p.x, (double)hx));
        ly = __double2float_rn(__dsub_rn(p.y, (double)hy));
        cerr = __fadd_ru(__fmul_ru(__fadd_ru(bmag, __fadd_ru(fabsf(hx), fabsf(hy))), kTwoM44),
                         kTwoM120);
      }
      int sp = 0;
      int node = t.nleaves > 1 ? 0 : ~0;
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
          // (both whole-leaf cases fall through to the pop below)
          const int cls = split ? leaf_class(t.leaf_box[c], hx, hy, lx, ly, cerr, d_lo, d_hi) : 0;
          if (cls > 0) {  // every point of the leaf is within d
            tested += b1 - b0;
            for (uint32_t k = b0; k < b1; k++) {
              if (kScatter) {
                run_put(out_build, cap, runbuf, pos, staged, t.sorted_id[k]);
              } else {
                if (cnt < K) run_put(slots, send, runbuf, spos, staged, t.sorted_id[k]);
                else if (kArena) arena_put(A, t.sorted_id[k], a_cur, a_first, a_fill, a_failed);
                cnt++;
              }
            }
          }
          // cls < 0: every point of the leaf is farther than d
          for (uint32_t k = b0; cls == 0 && k < b1; k++) {
            if (!box_overlap(t.sorted_box[k], q)) continue;
            tested++;
            int r = -1;
            if (split) {
              const float4 h = bhl[k];
              const float dx = __fadd_rn(__fsub_rn(h.x, hx), __fsub_rn(h.z, lx));
              const float dy = __fadd_rn(__fsub_rn(h.y, hy), __fsub_rn(h.w, ly));
              const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
              // D <= hi < d_lo <= d: RN(D) <= d.  D >= lo > d_hi >= d with lo
              // a float above d_hi, so D exceeds d by an FP32 ulp: RN(D) > d.
              if (__fadd_ru(__fmul_ru(__fsqrt_ru(d2), kSplitUp), cerr) < d_lo) r = 1;
              else if (__fsub_rd(__fmul_rd(__fsqrt_rd(d2), kSplitDown), cerr) > d_hi) r = 0;
            }
            if (r < 0) {
              esc++;
              r = exact::dwithin_exact(bxy[k], p, d) ? 1 : 0;
            }
            if (r) {
              if (kScatter) {
                // (probe ids: fill_probe_ids)
                run_put(out_build, cap, runbuf, pos, staged, t.sorted_id[k]);
              } else {
                if (cnt < K) run_put(slots, send, runbuf, spos, staged, t.sorted_id[k]);
                else if (kArena) arena_put(A, t.sorted_id[k], a_cur, a_first, a_fill, a_failed);
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
    if (staged) run_flush(kScatter ? out_build : slots, kScatter ? cap : send, runbuf,
                          kScatter ? pos : spos, staged);
    if (!kScatter) {
      counts[pi] = cnt;
      if (kArena) {
        if (a_cur != kArenaEnd) A.words[(size_t)a_cur * kArenaChunkWords] = kArenaEnd;
        A.head[pi] = a_failed ? kArenaFailed : a_first;
      }
    }
  }
  if (!kScatter) {
    for (int o = 16; o > 0; o >>= 1) {
      esc += __shfl_xor_sync(0xffffffffu, esc, o);
      tested += __shfl_xor_sync(0xffffffffu, tested, o);
    }
    if ((threadIdx.x & 31) == 0) {
      if (esc) atomicAdd(&st->counters[0], (unsigned long long)esc);
      if (tested) atomicAdd(&st->counters[1], (unsigned long long)tested);
    }
  }
}

// out_build over each row's run from its slots: all of a row with <= K
// results, the first K of a row whose rest is in the arena (warp per 32
// consecutive rows, coalesced stores; see fill_probe_ids)
__global__ void k_copy_slots(const uint64_t* __restrict__ offs, const uint32_t* __restrict__ counts,
                             const uint32_t* __restrict__ slots, uint32_t K, uint32_t n,
                             uint32_t* __restrict__ out, uint64_t cap,
                             const uint32_t* __restrict__ head) {
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
      const uint64_t r = w * 32 + L;
      const uint64_t sr = __shfl_sync(0xffffffffu, st, L);
      if (e < e1 && e < cap && r < n) {
        const uint64_t i = e - sr;
        const bool mine = counts[r] <= K || (head != nullptr && head[r] != kArenaFailed && i < K);
        if (mine) out[e] = slots[r * K + i];
      }
    }
  }
}

// out_build past the first K of each row whose overflow is in the arena: a
// warp per row, each chunk's ids copied by 31 lanes, the chain followed for
// at most the chunks the row's count needs.
__global__ void k_copy_arena(const uint64_t* __restrict__ offs, const uint32_t* __restrict__ counts,
                             uint32_t K, uint32_t n, DwithinArena A, uint32_t* __restrict__ out,
                             uint64_t cap) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; r < n; r += nw) {
    const uint32_t c = counts[r];
    if (c <= K) continue;
    uint32_t ch = A.head[r];
    if (ch == kArenaFailed) continue;
    const uint64_t end = offs[r] + c;
    uint64_t e = offs[r] + K;
    const uint32_t maxq = (c - K + kArenaChunkWords - 2) / (kArenaChunkWords - 1);
    for (uint32_t q = 0; q < maxq && ch < A.chunks && e < end; q++) {
      const uint64_t o = e + lane;
      if (lane < kArenaChunkWords - 1 && o < end && o < cap)
        out[o] = A.words[(size_t)ch * kArenaChunkWords + 1 + lane];
      e += kArenaChunkWords - 1;
      ch = A.words[(size_t)ch * kArenaChunkWords];
    }
  }
}

void float_neighbours(double d, float& lo, float& hi) {
  lo = (float)d;
  hi = (float)d;
  if ((double)lo > d) lo = next_downf(lo);
  if ((double)hi < d) hi = next_upf(hi);
}

}  // namespace

void build_point_split(const double2* pts, uint32_t npts, const Lbvh& bvh, PointSplit& out,
                       cudaStream_t s) {
  const uint32_t m = bvh.nprims;
  out.n = m;
  out.xy.reserve(((size_t)m + 1) * 16, s);
  out.hl.reserve(((size_t)m + 1) * 16, s);
  out.tmp.reserve(8, s);
  SPJ_CUDA(cudaMemsetAsync(out.tmp.get(), 0, 8, s));
  if (m)
    k_split_points<<<grid_for(m, 256), 256, 0, s>>>(pts, npts, bvh.sorted_id.as<uint32_t>(), m,
                                                    out.xy.as<double2>(), out.hl.as<float4>(),
                                                    out.tmp.as<unsigned>());
  SPJ_CUDA(cudaGetLastError());
  unsigned mag[2];
  SPJ_CUDA(cudaMemcpyAsync(mag, out.tmp.get(), 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  float b;
  std::memcpy(&b, &mag[0], 4);
  SPJ_CHECK((mag[1] & 2u) == 0, "point split: sorted id out of range");
  out.bmag = b;
  out.ok = mag[1] == 0;
}

void dwithin_count(const LbvhView& t, const PointSplit& bs, const float4* probe_box,
                   const double2* probe_pt, uint32_t n, double d, const uint32_t* order,
                   uint32_t* counts, DeviceStatus* st, cudaStream_t s, uint32_t* slots,
                   uint32_t K, DwithinArena arena, const double* d_row) {
  if (n == 0) return;
  float lo, hi;
  float_neighbours(d, lo, hi);
  const int g = grid_for(n, kTravThreads, kNumSMs * 16);
  if (slots && K > 0 && arena.words)
    k_dwithin_fused<false, true><<<g, kTravThreads, 0, s>>>(
        t, bs.xy.as<double2>(), bs.hl.as<float4>(), bs.bmag, bs.ok ? 1 : 0, probe_box, probe_pt,
        n, d, lo, hi, d_row, order, counts, nullptr, 0, nullptr, nullptr, 0, st, slots, K, arena);
  else
    k_dwithin_fused<false, false><<<g, kTravThreads, 0, s>>>(
        t, bs.xy.as<double2>(), bs.hl.as<float4>(), bs.bmag, bs.ok ? 1 : 0, probe_box, probe_pt,
        n, d, lo, hi, d_row, order, counts, nullptr, 0, nullptr, nullptr, 0, st, slots,
        slots ? K : 0, DwithinArena());
  SPJ_CUDA(cudaGetLastError());
}

void dwithin_scatter(const LbvhView& t, const PointSplit& bs, const float4* probe_box,
                     const double2* probe_pt, uint32_t n, double d, const uint32_t* order,
                     const uint64_t* offs, uint32_t probe_base, uint32_t* out_build,
                     uint32_t* out_probe, uint64_t capacity, cudaStream_t s,
                     const uint32_t* counts, const uint32_t* slots, uint32_t K,
                     DwithinArena arena, const double* d_row) {
  if (!(slots && K > 0)) arena = DwithinArena();
  if (n == 0) return;
  float lo, hi;
  float_neighbours(d, lo, hi);
  const int g = grid_for(n, kTravThreads, kNumSMs * 16);
  if (arena.words)
    k_dwithin_fused<true, true><<<g, kTravThreads, 0, s>>>(
        t, bs.xy.as<double2>(), bs.hl.as<float4>(), bs.bmag, bs.ok ? 1 : 0, probe_box, probe_pt,
        n, d, lo, hi, d_row, order, const_cast<uint32_t*>(counts), offs, probe_base, out_build,
        out_probe, capacity, nullptr, nullptr, slots ? K : 0, arena);
  else
    k_dwithin_fused<true, false><<<g, kTravThreads, 0, s>>>(
        t, bs.xy.as<double2>(), bs.hl.as<float4>(), bs.bmag, bs.ok ? 1 : 0, probe_box, probe_pt,
        n, d, lo, hi, d_row, order, const_cast<uint32_t*>(counts), offs, probe_base, out_build,
        out_probe, capacity, nullptr, nullptr, slots ? K : 0, arena);
  SPJ_CUDA(cudaGetLastError());
  if (slots && K > 0)
    k_copy_slots<<<grid_for((int64_t)n, 256), 256, 0, s>>>(offs, counts, slots, K, n, out_build,
                                                            capacity, arena.head);
  if (arena.words)
    k_copy_arena<<<grid_for((int64_t)n * 32, 256, kNumSMs * 32), 256, 0, s>>>(
        offs, counts, K, n, arena, out_build, capacity);
  fill_probe_ids(offs, n, probe_base, out_probe, capacity, s);
}

}  // namespace spj
