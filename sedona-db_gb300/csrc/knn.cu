// knn.cu — KNN join: LBVH over the build points, depth-first traversal
// nearest child first, a register-resident best list per probe thread,
// probes taken in Morton order of their coordinates.
//
// Ranking key: the exact squared distance dx^2 + dy^2 of the FP64 deltas
// dx = RN(b.x - p.x), dy = RN(b.y - p.y) (the deltas the reference's
// Euclidean distance forms), held as a normalized double-double (hi, lo) and
// compared lexicographically, then by build id.  Exact duplicates tie on the
// key and fall back to the build id, as in the reference ground truth.
//
// Chosen form (k <= 16): every coordinate is split into an FP32 pair
// hi = RN32(v), lo = RN32(v - hi), and the traversal ranks points by the FP32
// squared distance of (b.hi - q.hi) + (b.lo - q.lo), whose error is a few
// ulps of the distance itself plus 2^-44 of the coordinate magnitude (the
// bound is derived at kSplitRel below).  It keeps the k+1 best; when the
// (k+1)-th is provably farther than each of the first k (their error
// intervals are disjoint), the k-set is exact, and only those k points get
// the FP64 key that orders them.  Probes whose k-set is not proven this way
// (near ties at rank k, exact duplicates) are queued for the exact kernel.
// Plain form: every visited point gets the FP64 key.
#include "knn.cuh"
#include "prims.cuh"

#include <cmath>
#include <vector>

namespace spj {
namespace {

constexpr int kKnnThreads = 128;
constexpr int kKnnStack = 64;

// |true distance - sqrt(d2)| <= kSplitRel * sqrt(d2) + cerr, cerr =
// 2^-44 (max|b.x|+|b.y| + |q.x|+|q.y|) + 2^-120, for the split FP32 distance
// d2.  Per axis, with u = 2^-24: b = hi + lo + e, |e| <= 2^-48 |b|; the three
// FP32 roundings give |dx - (b - q).x| <= 2u |dx| (1 + 2u) + 3 * 2^-48 (|b.x| +
// |q.x|); the two axes add to <= 2^-22 * |d| + 2^-46 (..); squaring, summing
// and the square root add 2^-23 relative.  kSplitRel = 2^-20 covers the
// relative part twice over, 2^-44 the absolute part four times over, and
// 2^-120 the absolute error of FP32 results below the normal range.
constexpr float kSplitUp = 1.00000095367431640625f;    // 1 + 2^-20
constexpr float kSplitDown = 0.99999904632568359375f;  // 1 - 2^-20
constexpr float kTwoM44 = 5.684341886080801486968994140625e-14f;
constexpr float kTwoM120 = 7.5231638452626400509999138382223723380394595633413601376560e-37f;
// coordinates up to this magnitude keep every split FP32 square finite
constexpr double kSplitMaxCoord = 1e18;

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

// exact dx^2 + dy^2 as a normalized double-double
__device__ __forceinline__ void sq_dist_dd(double2 b, double2 p, double& hi, double& lo) {
  const double dx = __dsub_rn(b.x, p.x), dy = __dsub_rn(b.y, p.y);
  const double a1 = __dmul_rn(dx, dx), a2 = __fma_rn(dx, dx, -a1);
  const double b1 = __dmul_rn(dy, dy), b2 = __fma_rn(dy, dy, -b1);
  double s, e;
  two_sum(a1, b1, s, e);
  e = __dadd_rn(e, __dadd_rn(a2, b2));
  two_sum(s, e, hi, lo);
}

__device__ __forceinline__ bool key_less(double h1, double l1, uint32_t i1, double h2, double l2,
                                         uint32_t i2) {
  if (h1 != h2) return h1 < h2;
  if (l1 != l2) return l1 < l2;
  return i1 < i2;
}

// lower bound of the FP32 distance from q to box b (0 inside)
__device__ __forceinline__ float box_dist(float2 q, float4 b) {
  const float dx = fmaxf(fmaxf(b.x - q.x, q.x - b.z), 0.0f);
  const float dy = fmaxf(fmaxf(b.y - q.y, q.y - b.w), 0.0f);
  return __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
}

__device__ __forceinline__ void write_empty(uint32_t* out_idx, double* out_dist, uint64_t qi,
                                            uint32_t k) {
  for (uint32_t j = 0; j < k; j++) {
    out_idx[qi * k + j] = 0xFFFFFFFFu;
    out_dist[qi * k + j] = INFINITY;
  }
}

// Exact kernel.  With `order`, thread slot j serves probe order[j]; with
// n_dev, the slot count is read from device memory (the queue the split
// kernel filled).
template <int K, bool kFast>
__global__ void __launch_bounds__(kKnnThreads)
    k_knn(LbvhView t, const double2* __restrict__ bxy, const double2* __restrict__ probe,
          uint64_t n, const uint32_t* __restrict__ order, const uint32_t* __restrict__ n_dev,
          uint32_t k, float slack, uint32_t* __restrict__ out_idx, double* __restrict__ out_dist,
          unsigned long long* __restrict__ exact_evals) {
  __shared__ int stack[kKnnStack * kKnnThreads];
  const uint64_t max_steps = 2ull * t.nleaves + 2;
  uint32_t evals = 0;
  const uint64_t nn = n_dev ? (uint64_t)*n_dev : n;
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < nn;
       j += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t qi = order ? (uint64_t)order[j] : j;
    if (qi >= n) {
      traversal_fault(t, kBadProbe, (unsigned)qi);
      continue;
    }
    const double2 q = probe[qi];
    const float2 q32 = make_float2(__double2float_rn(q.x), __double2float_rn(q.y));
    // |q - q32| bound, plus the build-side bound
    const float qs = __fadd_ru(__fmul_ru(fabsf(q32.x) + fabsf(q32.y), 1.1920929e-07f), slack);
    double kh[K], kl[K];
    uint32_t ki[K];
#pragma unroll
    for (int c = 0; c < K; c++) {
      kh[c] = INFINITY;
      kl[c] = 0;
      ki[c] = 0xFFFFFFFFu;
    }
    uint32_t have = 0;
    float bound = INFINITY;  // FP32 upper bound of the k-th best distance
    const bool valid = !(isnan(q.x) || isnan(q.y)) && t.nprims > 0;
    int sp = 0;
    int node = valid ? (t.nleaves > 1 ? 0 : ~0) : 0;
    bool done = !valid;
    uint64_t steps = 0;
    while (!done) {
      if (++steps > max_steps) {  // each node is visited at most once
        traversal_fault(t, kTooLong, (unsigned)qi);
        break;
      }
      if (node < 0) {
        const uint32_t c = (uint32_t)(~node);
        if (c >= t.nleaves) {
          traversal_fault(t, kBadLeaf, c);
          break;
        }
        const uint32_t b0 = c * t.leaf_size, b1 = min(b0 + t.leaf_size, t.nprims);
        for (uint32_t pi = b0; pi < b1; pi++) {
          const double2 b = bxy[pi];
          if (kFast && have >= k) {
            const float4 pb = t.sorted_box[pi];  // RN32 of the point
            const float fx = __fsub_rn(pb.x, q32.x), fy = __fsub_rn(pb.y, q32.y);
            const float d32 = __fsqrt_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)));
            const float mag = fabsf(pb.x) + fabsf(q32.x) + fabsf(pb.y) + fabsf(q32.y) +
                              fabsf(fx) + fabsf(fy);
            const float err = __fadd_ru(__fmul_ru(mag, 2.384185791015625e-07f),
                                        __fmul_ru(d32, 4.76837158203125e-07f));
            if (__fsub_rd(d32, err) > bound) continue;  // provably farther than the k-th
          }
          double h, l;
          sq_dist_dd(b, q, h, l);
          evals++;
          const uint32_t id = t.sorted_id[pi];
          if (have >= k && !key_less(h, l, id, kh[K - 1], kl[K - 1], ki[K - 1])) continue;
          // insert into the sorted register list
          bool placed = false;
#pragma unroll
          for (int c2 = K - 1; c2 > 0; c2--) {
            if (!placed) {
              if (key_less(h, l, id, kh[c2 - 1], kl[c2 - 1], ki[c2 - 1])) {
                kh[c2] = kh[c2 - 1];
                kl[c2] = kl[c2 - 1];
                ki[c2] = ki[c2 - 1];
              } else {
                kh[c2] = h;
                kl[c2] = l;
                ki[c2] = id;
                placed = true;
              }
            }
          }
          if (!placed) {
            kh[0] = h;
            kl[0] = l;
            ki[0] = id;
          }
          if (have < k) have++;
          if (have >= k) {
            // k-th entry of the list sits at index k-1 (k <= K)
            double kth = kh[K - 1];
#pragma unroll
            for (int c2 = 0; c2 < K; c2++)
              if (c2 == (int)k - 1) kth = __dadd_rn(kh[c2], kl[c2]);
            bound = __double2float_ru(sqrt(kth) * (1.0 + 1e-12));
          }
        }
      } else {
        if ((uint32_t)node + 1 >= t.nleaves) {
          traversal_fault(t, kBadNode, (unsigned)node);
          break;
        }
        const float4 lb = t.node_box[2 * node], rb = t.node_box[2 * node + 1];
        const int2 ch = t.node_child[node];
        // conservative lower bounds of the true distance
        const float dl = __fsub_rd(__fmul_rd(box_dist(q32, lb), 0.99999905f), qs);
        const float dr = __fsub_rd(__fmul_rd(box_dist(q32, rb), 0.99999905f), qs);
        const bool vl = dl <= bound, vr = dr <= bound;
        if (vl && vr) {
          const int nearc = dl <= dr ? ch.x : ch.y;
          const int farc = dl <= dr ? ch.y : ch.x;
          if (sp >= kKnnStack) {  // deeper than any tree built here: record, stop
            traversal_fault(t, kStackOverflow, (unsigned)qi);
            break;
          }
          stack[sp * kKnnThreads + threadIdx.x] = farc;
          sp++;
          node = nearc;
          continue;
        }
        if (vl) {
          node = ch.x;
          continue;
        }
        if (vr) {
          node = ch.y;
          continue;
        }
      }
      // pop, skipping subtrees the bound now excludes is left to the next
      // visit (the node test re-checks the bound)
      if (sp == 0) break;
      sp--;
      node = stack[sp * kKnnThreads + threadIdx.x];
    }
    for (uint32_t c = 0; c < k; c++) {
      uint32_t id = 0xFFFFFFFFu;
      double d = INFINITY;
#pragma unroll
      for (int cc = 0; cc < K; cc++)
        if (cc == (int)c && cc < (int)have) {
          id = ki[cc];
          d = sqrt(__dadd_rn(kh[cc], kl[cc]));
        }
      out_idx[qi * k + c] = id;
      out_dist[qi * k + c] = d;
    }
  }
  for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
  if ((threadIdx.x & 31) == 0 && evals) atomicAdd(exact_evals, (unsigned long long)evals);
}

// Split-FP32 kernel (chosen form): see the file comment.  hl[pi] holds the
// sorted build point pi as (hi.x, hi.y, lo.x, lo.y); bmag bounds |b.x|+|b.y|
// over the build side.  Probes whose k-set is not proven are appended to
// redo[] (count in *nredo) and their outputs left to the exact kernel.
template <int K>
__global__ void __launch_bounds__(kKnnThreads)
    k_knn_split(LbvhView t, const float4* __restrict__ hl, const double2* __restrict__ bxy,
                const double2* __restrict__ probe, uint64_t n, const uint32_t* __restrict__ order,
                uint32_t k, float slack, float bmag, uint32_t* __restrict__ out_idx,
                double* __restrict__ out_dist, uint32_t* __restrict__ redo,
                uint32_t* __restrict__ nredo, unsigned long long* __restrict__ exact_evals) {
  __shared__ int stack[kKnnStack * kKnnThreads];
  const uint64_t max_steps = 2ull * t.nleaves + 2;
  uint32_t evals = 0;
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < n;
       j += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t qi = order ? (uint64_t)order[j] : j;
    if (qi >= n) {
      traversal_fault(t, kBadProbe, (unsigned)qi);
      continue;
    }
    const double2 q = probe[qi];
    if (isnan(q.x) || isnan(q.y) || t.nprims == 0) {
      write_empty(out_idx, out_dist, qi, k);
      continue;
    }
    if (!(fabs(q.x) <= kSplitMaxCoord && fabs(q.y) <= kSplitMaxCoord)) {
      redo[atomicAdd(nredo, 1u)] = (uint32_t)qi;
      continue;
    }
    const float qhx = __double2float_rn(q.x), qhy = __double2float_rn(q.y);
    // q - RN32(q) is exact in FP64
    const float qlx = __double2float_rn(__dsub_rn(q.x, (double)qhx));
    const float qly = __double2float_rn(__dsub_rn(q.y, (double)qhy));
    const float2 q32 = make_float2(qhx, qhy);
    const float qs = __fadd_ru(__fmul_ru(fabsf(qhx) + fabsf(qhy), 1.1920929e-07f), slack);
    const float cerr =
        __fadd_ru(__fmul_ru(__fadd_ru(bmag, __fadd_ru(fabsf(qhx), fabsf(qhy))), kTwoM44),
                  kTwoM120);
    // the K+1 smallest split distances seen, ascending
    float ld[K + 1];
    uint32_t lp[K + 1];
#pragma unroll
    for (int c = 0; c <= K; c++) {
      ld[c] = INFINITY;
      lp[c] = 0xFFFFFFFFu;
    }
    uint32_t have = 0;       // list entries, capped at k + 1
    float bound = INFINITY;  // upper bound of the true distance of the (k+1)-th entry
    int sp = 0;
    int node = t.nleaves > 1 ? 0 : ~0;
    uint64_t steps = 0;
    while (true) {
      if (++steps > max_steps) {  // each node is visited at most once
        traversal_fault(t, kTooLong, (unsigned)qi);
        break;
      }
      if (node < 0) {
        const uint32_t c = (uint32_t)(~node);
        if (c >= t.nleaves) {
          traversal_fault(t, kBadLeaf, c);
          break;
        }
        const uint32_t b0 = c * t.leaf_size, b1 = min(b0 + t.leaf_size, t.nprims);
        for (uint32_t pi = b0; pi < b1; pi++) {
          const float4 h = hl[pi];
          const float dx = __fadd_rn(__fsub_rn(h.x, qhx), __fsub_rn(h.z, qlx));
          const float dy = __fadd_rn(__fsub_rn(h.y, qhy), __fsub_rn(h.w, qly));
          const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
          if (!(d2 < ld[K])) continue;
          bool placed = false;
#pragma unroll
          for (int c2 = K; c2 > 0; c2--) {
            if (!placed) {
              if (d2 < ld[c2 - 1]) {
                ld[c2] = ld[c2 - 1];
                lp[c2] = lp[c2 - 1];
              } else {
                ld[c2] = d2;
                lp[c2] = pi;
                placed = true;
              }
            }
          }
          if (!placed) {
            ld[0] = d2;
            lp[0] = pi;
          }
          if (have <= k) have++;
          if (have > k) {
            float dk1 = ld[K];
#pragma unroll
            for (int c2 = 0; c2 <= K; c2++)
              if (c2 == (int)k) dk1 = ld[c2];
            bound = __fadd_ru(__fmul_ru(__fsqrt_ru(dk1), kSplitUp), cerr);
          }
        }
      } else {
        if ((uint32_t)node + 1 >= t.nleaves) {
          traversal_fault(t, kBadNode, (unsigned)node);
          break;
        }
        const float4 lb = t.node_box[2 * node], rb = t.node_box[2 * node + 1];
        const int2 ch = t.node_child[node];
        const float dl = __fsub_rd(__fmul_rd(box_dist(q32, lb), 0.99999905f), qs);
        const float dr = __fsub_rd(__fmul_rd(box_dist(q32, rb), 0.99999905f), qs);
        const bool vl = dl <= bound, vr = dr <= bound;
        if (vl && vr) {
          const int nearc = dl <= dr ? ch.x : ch.y;
          const int farc = dl <= dr ? ch.y : ch.x;
          if (sp >= kKnnStack) {  // deeper than any tree built here: record, stop
            traversal_fault(t, kStackOverflow, (unsigned)qi);
            break;
          }
          stack[sp * kKnnThreads + threadIdx.x] = farc;
          sp++;
          node = nearc;
          continue;
        }
        if (vl) {
          node = ch.x;
          continue;
        }
        if (vr) {
          node = ch.y;
          continue;
        }
      }
      if (sp == 0) break;
      sp--;
      node = stack[sp * kKnnThreads + threadIdx.x];
    }
    // With fewer than k+1 entries the bound never closed, so every build
    // point was visited and listed.  Otherwise the k-set is proven when the
    // (k+1)-th entry's lower bound exceeds the k-th entry's upper bound (the
    // list is ascending, so the k-th bounds the first k).
    if (have > k) {
      float dk = ld[0], dk1 = ld[0];
#pragma unroll
      for (int c = 0; c <= K; c++) {
        if (c == (int)k - 1) dk = ld[c];
        if (c == (int)k) dk1 = ld[c];
      }
      const float up = __fadd_ru(__fmul_ru(__fsqrt_ru(dk), kSplitUp), cerr);
      const float lo = __fsub_rd(__fmul_rd(__fsqrt_rd(dk1), kSplitDown), cerr);
      if (!(lo > up)) {
        redo[atomicAdd(nredo, 1u)] = (uint32_t)qi;
        continue;
      }
    }
    // Order of the proven set by (exact key, build id).  The list is already
    // ascending in the split distance; two neighbours whose error intervals
    // [lo, up] are disjoint are in exact order, and only neighbours whose
    // intervals overlap (near ties, duplicates) compare exact double-double
    // keys (computed on the spot: this is rare).  Odd-even transposition over
    // the K slots (static register indices); slots past kk stay last.
    const uint32_t kk = min(k, have);
    float lo[K], up[K];
    uint32_t ki[K];
#pragma unroll
    for (int c = 0; c < K; c++) {
      const bool v = c < (int)kk;
      ki[c] = v ? t.sorted_id[lp[c]] : 0xFFFFFFFFu;
      lo[c] = v ? __fsub_rd(__fmul_rd(__fsqrt_rd(ld[c]), kSplitDown), cerr) : INFINITY;
      up[c] = v ? __fadd_ru(__fmul_ru(__fsqrt_ru(ld[c]), kSplitUp), cerr) : INFINITY;
    }
#pragma unroll
    for (int r = 0; r < K; r++) {
#pragma unroll
      for (int c = r & 1; c + 1 < K; c += 2) {
        if (lo[c + 1] == INFINITY || up[c] < lo[c + 1]) continue;  // empty, or in order
        bool swap = up[c + 1] < lo[c];
        if (!swap) {
          double ha, la, hb, lb;
          sq_dist_dd(bxy[lp[c]], q, ha, la);
          sq_dist_dd(bxy[lp[c + 1]], q, hb, lb);
          evals += 2;
          swap = key_less(hb, lb, ki[c + 1], ha, la, ki[c]);
        }
        if (swap) {
          const float tl = lo[c], tu = up[c];
          const uint32_t tp = lp[c], ti = ki[c];
          lo[c] = lo[c + 1];
          up[c] = up[c + 1];
          lp[c] = lp[c + 1];
          ki[c] = ki[c + 1];
          lo[c + 1] = tl;
          up[c + 1] = tu;
          lp[c + 1] = tp;
          ki[c + 1] = ti;
        }
      }
    }
    // distances in FP64 from the reference's deltas (within a few ulps of
    // the exact value; the order above is exact)
    for (uint32_t c = 0; c < k; c++) {
      uint32_t id = 0xFFFFFFFFu;
      double dist = INFINITY;
#pragma unroll
      for (int cc = 0; cc < K; cc++)
        if (cc == (int)c && cc < (int)kk) {
          id = ki[cc];
          const double2 b = bxy[lp[cc]];
          const double dx = __dsub_rn(b.x, q.x), dy = __dsub_rn(b.y, q.y);
          dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
        }
      out_idx[qi * k + c] = id;
      out_dist[qi * k + c] = dist;
    }
  }
  for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
  if ((threadIdx.x & 31) == 0 && evals) atomicAdd(exact_evals, (unsigned long long)evals);
}

// Tie rows of include_tie_breakers (rust/sedona-spatial-join/src/index/
// default_spatial_index.rs:378-470): after a probe's k results come the
// build points outside them whose distance is within DISTANCE_TOLERANCE
// (1e-9, rust/sedona-spatial-join/src/index/spatial_index.rs:32) of the k-th
// distance, found as the reference finds them, by a box search around the
// probe.  A probe with fewer than k results has no ties.  The counting pass
// writes each probe's output length (its valid results plus its ties); the
// scatter pass writes the results, then the ties in traversal order.
constexpr double kTieTolerance = 1e-9;

template <bool kScatter>
__global__ void __launch_bounds__(kKnnThreads)
    k_knn_ties(LbvhView t, const double2* __restrict__ bxy, const double2* __restrict__ probe,
               uint64_t n, uint32_t k, bool ties, const uint32_t* __restrict__ kidx,
               const double* __restrict__ kdist, uint32_t* __restrict__ counts,
               const uint64_t* __restrict__ offs, uint32_t* __restrict__ out_idx,
               double* __restrict__ out_dist, uint64_t cap) {
  __shared__ int stack[kKnnStack * kKnnThreads];
  const uint64_t max_steps = 2ull * t.nleaves + 2;
  for (uint64_t qi = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; qi < n;
       qi += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t* ki = kidx + qi * k;
    uint32_t nvalid = 0;
    while (nvalid < k && ki[nvalid] != 0xFFFFFFFFu) nvalid++;
    uint64_t pos = kScatter ? offs[qi] : 0;
    if (kScatter) {
      for (uint32_t c = 0; c < nvalid; c++, pos++)
        if (pos < cap) {
          out_idx[pos] = ki[c];
          out_dist[pos] = kdist[qi * k + c];
        }
    }
    uint32_t cnt = 0;
    const double2 q = probe[qi];
    if (ties && nvalid == k && t.nprims > 0 && !(isnan(q.x) || isnan(q.y))) {
      const double kth = kdist[qi * k + k - 1];
      const double r = __dadd_ru(kth, kTieTolerance);
      // every build point within r of q has its RN32 box in this box
      const float4 qb = make_float4(__double2float_rd(__dsub_rd(q.x, r)),
                                    __double2float_rd(__dsub_rd(q.y, r)),
                                    __double2float_ru(__dadd_ru(q.x, r)),
                                    __double2float_ru(__dadd_ru(q.y, r)));
      int sp = 0;
      int node = t.nleaves > 1 ? 0 : ~0;
      uint64_t steps = 0;
      while (true) {
        if (++steps > max_steps) {
          traversal_fault(t, kTooLong, (unsigned)qi);
          break;
        }
        if (node < 0) {
          const uint32_t c = (uint32_t)(~node);
          if (c >= t.nleaves) {
            traversal_fault(t, kBadLeaf, c);
            break;
          }
          const uint32_t b0 = c * t.leaf_size, b1 = min(b0 + t.leaf_size, t.nprims);
          for (uint32_t kk = b0; kk < b1; kk++) {
            if (!box_overlap(t.sorted_box[kk], qb)) continue;
            const uint32_t id = t.sorted_id[kk];
            bool mine = false;
            for (uint32_t c2 = 0; c2 < k; c2++) mine |= ki[c2] == id;
            if (mine) continue;
            const double2 b = bxy[kk];
            const double dx = __dsub_rn(b.x, q.x), dy = __dsub_rn(b.y, q.y);
            const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
            if (!(__dsub_rn(dist, kth) <= kTieTolerance)) continue;
            if (kScatter) {
              if (pos < cap) {
                out_idx[pos] = id;
                out_dist[pos] = dist;
              }
              pos++;
            } else {
              cnt++;
            }
          }
        } else {
          if ((uint32_t)node + 1 >= t.nleaves) {
            traversal_fault(t, kBadNode, (unsigned)node);
            break;
          }
          const float4 lb = t.node_box[2 * node], rb = t.node_box[2 * node + 1];
          const int2 ch = t.node_child[node];
          const bool hl = box_overlap(lb, qb), hr = box_overlap(rb, qb);
          if (hl && hr) {
            if (sp >= kKnnStack) {  // deeper than any tree built here: record, stop
              traversal_fault(t, kStackOverflow, (unsigned)qi);
              break;
            }
            stack[sp * kKnnThreads + threadIdx.x] = ch.y;
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
        node = stack[sp * kKnnThreads + threadIdx.x];
      }
    }
    if (!kScatter) counts[qi] = nvalid + cnt;
  }
}

__global__ void k_points_to_boxes(const double2* __restrict__ xy, uint64_t n,
                                  float4* __restrict__ boxes) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const double2 p = xy[i];
    const float x = __double2float_rn(p.x), y = __double2float_rn(p.y);
    boxes[i] = make_float4(x, y, x, y);
  }
}

// sorted FP64 points and their (hi, lo) FP32 splits
__global__ void k_gather_xy(const double2* __restrict__ xy, const uint32_t* __restrict__ ids,
                            uint32_t m, double2* __restrict__ out, float4* __restrict__ hl) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const double2 p = xy[ids[i]];
    out[i] = p;
    const float hx = __double2float_rn(p.x), hy = __double2float_rn(p.y);
    hl[i] = make_float4(hx, hy, __double2float_rn(__dsub_rn(p.x, (double)hx)),
                        __double2float_rn(__dsub_rn(p.y, (double)hy)));
  }
}

}  // namespace

KnnIndex::KnnIndex(uint32_t leaf_size, int form) : leaf_size_(leaf_size), form_(form) {
  SPJ_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
}

KnnIndex::~KnnIndex() {
  if (stream_) {
    cudaStreamSynchronize(stream_);
    bvh_ = Lbvh();
    xy_sorted_.release();
    xy_split_.release();
    probe_.release();
    oidx_.release();
    odist_.release();
    counters_.release();
    redo_.release();
    tie_probe_.release();
    tie_kidx_.release();
    tie_kdist_.release();
    tie_counts_.release();
    tie_offs_.release();
    tie_tmp_.release();
    tie_out_idx_.release();
    tie_out_dist_.release();
    osc_ = ProbeScratch();
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
}

void KnnIndex::build(const double* xy_host, uint64_t n) {
  SPJ_CHECK(n < 0xFFFFFFFFull, "too many build points");
  SPJ_CHECK(n == 0 || xy_host != nullptr, "null build points");
  cudaStream_t s = stream_;
  n_ = n;
  DevBuf xy((n + 1) * 16, s), boxes((n + 1) * 16, s);
  if (n) SPJ_CUDA(cudaMemcpyAsync(xy.get(), xy_host, n * 16, cudaMemcpyHostToDevice, s));
  k_points_to_boxes<<<grid_for((int64_t)n, 256), 256, 0, s>>>(xy.as<double2>(), n,
                                                               boxes.as<float4>());
  build_lbvh(boxes.as<float4>(), (uint32_t)n, leaf_size_, bvh_, s);
  xy_sorted_.reserve(((size_t)bvh_.nprims + 1) * 16, s);
  xy_split_.reserve(((size_t)bvh_.nprims + 1) * 16, s);
  if (bvh_.nprims)
    k_gather_xy<<<grid_for(bvh_.nprims, 256), 256, 0, s>>>(
        xy.as<double2>(), bvh_.sorted_id.as<uint32_t>(), bvh_.nprims, xy_sorted_.as<double2>(),
        xy_split_.as<float4>());
  // |p - RN32(p)| <= 2^-24 (|x| + |y|) <= 2^-24 * 2 * max|coord|
  double mx = 0, l1 = 0;
  bool split_ok = true;
  for (uint64_t i = 0; i < n; i++) {
    const double x = xy_host[2 * i], y = xy_host[2 * i + 1];
    if (std::isnan(x) || std::isnan(y)) continue;  // left out of the tree
    const double ax = std::fabs(x), ay = std::fabs(y);
    if (!(ax <= kSplitMaxCoord && ay <= kSplitMaxCoord)) split_ok = false;
    if (std::isfinite(ax) && ax > mx) mx = ax;
    if (std::isfinite(ay) && ay > mx) mx = ay;
    if (std::isfinite(ax + ay) && ax + ay > l1) l1 = ax + ay;
  }
  slack_ = (float)(mx * 2.0 * std::ldexp(1.0, -23));
  split_ok_ = split_ok;
  // rounded up so that it bounds max(|x| + |y|)
  bmag_ = (float)l1;
  if ((double)bmag_ < l1) bmag_ = std::nextafter(bmag_, INFINITY);
  SPJ_CUDA(cudaStreamSynchronize(s));
}

uint64_t KnnIndex::query_ties(const double* probe_xy, uint64_t n, uint32_t k, bool device_ptrs,
                              uint64_t* offsets, uint32_t* out_idx, double* out_dist,
                              uint64_t capacity, bool ties) {
  SPJ_CHECK(offsets != nullptr, "null offsets");
  cudaStream_t s = stream_;
  const double2* dp;
  if (device_ptrs) {
    dp = reinterpret_cast<const double2*>(probe_xy);
  } else {
    tie_probe_.reserve((n + 1) * 16, s);
    if (n) SPJ_CUDA(cudaMemcpyAsync(tie_probe_.get(), probe_xy, n * 16, cudaMemcpyHostToDevice, s));
    dp = tie_probe_.as<double2>();
  }
  tie_kidx_.reserve((n * k + 1) * 4, s);
  tie_kdist_.reserve((n * k + 1) * 8, s);
  query(reinterpret_cast<const double*>(dp), n, k, tie_kidx_.as<uint32_t>(),
        tie_kdist_.as<double>(), true);  // syncs
  tie_counts_.reserve((n + 1) * 4, s);
  tie_offs_.reserve((n + 1) * 8, s);
  const LbvhView t = bvh_.view();
  const int g = grid_for((int64_t)n, kKnnThreads, kNumSMs * 16);
  if (n)
    k_knn_ties<false><<<g, kKnnThreads, 0, s>>>(t, xy_sorted_.as<double2>(), dp, n, k, ties,
                                                 tie_kidx_.as<uint32_t>(), tie_kdist_.as<double>(),
                                                 tie_counts_.as<uint32_t>(), nullptr, nullptr,
                                                 nullptr, 0);
  scan_u32_u64(tie_counts_.as<uint32_t>(), tie_offs_.as<uint64_t>(), (int64_t)n, tie_tmp_, s);
  SPJ_CUDA(cudaMemcpyAsync(offsets, tie_offs_.get(), (n + 1) * 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  check_traversal(t, s);
  const uint64_t total = offsets[n];
  if (total > capacity || n == 0) return total;
  SPJ_CHECK(out_idx && out_dist, "null outputs");
  tie_out_idx_.reserve((total + 1) * 4, s);
  tie_out_dist_.reserve((total + 1) * 8, s);
  k_knn_ties<true><<<g, kKnnThreads, 0, s>>>(t, xy_sorted_.as<double2>(), dp, n, k, ties,
                                              tie_kidx_.as<uint32_t>(), tie_kdist_.as<double>(),
                                              nullptr, tie_offs_.as<uint64_t>(),
                                              tie_out_idx_.as<uint32_t>(),
                                              tie_out_dist_.as<double>(), total);
  SPJ_CUDA(cudaGetLastError());
  if (total) {
    SPJ_CUDA(cudaMemcpyAsync(out_idx, tie_out_idx_.get(), total * 4, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaMemcpyAsync(out_dist, tie_out_dist_.get(), total * 8, cudaMemcpyDeviceToHost, s));
  }
  SPJ_CUDA(cudaStreamSynchronize(s));
  check_traversal(t, s);
  return total;
}

void KnnIndex::query(const double* probe_xy, uint64_t n, uint32_t k, uint32_t* out_idx,
                     double* out_dist, bool device_ptrs) {
  SPJ_CHECK(k >= 1 && k <= 32, "k must be in [1, 32]");
  SPJ_CHECK(n < 0xFFFFFFFFull, "too many probe points");
  cudaStream_t s = stream_;
  const double2* dp;
  uint32_t* di;
  double* dd;
  if (device_ptrs) {
    dp = reinterpret_cast<const double2*>(probe_xy);
    di = out_idx;
    dd = out_dist;
  } else {
    probe_.reserve((n + 1) * 16, s);
    oidx_.reserve((n * k + 1) * 4, s);
    odist_.reserve((n * k + 1) * 8, s);
    if (n) SPJ_CUDA(cudaMemcpyAsync(probe_.get(), probe_xy, n * 16, cudaMemcpyHostToDevice, s));
    dp = probe_.as<double2>();
    di = oidx_.as<uint32_t>();
    dd = odist_.as<double>();
  }
  counters_.reserve(16, s);
  SPJ_CUDA(cudaMemsetAsync(counters_.get(), 0, 16, s));
  if (n) {
    const LbvhView t = bvh_.view();
    const uint32_t* order = point_order(t, dp, (uint32_t)n, osc_, s);
    const int g = grid_for((int64_t)n, kKnnThreads, kNumSMs * 16);
    auto* ev = counters_.as<unsigned long long>();
    uint32_t* nredo = reinterpret_cast<uint32_t*>(ev + 1);
    if (form_ == 1 && k <= 16 && split_ok_) {
      redo_.reserve((n + 1) * 4, s);
      uint32_t* redo = redo_.as<uint32_t>();
      if (k <= 8)
        k_knn_split<8><<<g, kKnnThreads, 0, s>>>(t, xy_split_.as<float4>(),
                                                 xy_sorted_.as<double2>(), dp, n, order, k,
                                                 slack_, bmag_, di, dd, redo, nredo, ev);
      else
        k_knn_split<16><<<g, kKnnThreads, 0, s>>>(t, xy_split_.as<float4>(),
                                                  xy_sorted_.as<double2>(), dp, n, order, k,
                                                  slack_, bmag_, di, dd, redo, nredo, ev);
      // the queued probes through the exact kernel (slot count read on the device)
      const int gr = grid_for((int64_t)n, kKnnThreads, kNumSMs * 4);
      if (k <= 8)
        k_knn<8, false><<<gr, kKnnThreads, 0, s>>>(t, xy_sorted_.as<double2>(), dp, n, redo,
                                                   nredo, k, slack_, di, dd, ev);
      else
        k_knn<16, false><<<gr, kKnnThreads, 0, s>>>(t, xy_sorted_.as<double2>(), dp, n, redo,
                                                    nredo, k, slack_, di, dd, ev);
    } else {
#define SPJ_KNN_LAUNCH(KK)                                                                       \
  if (form_ == 1)                                                                                \
    k_knn<KK, true><<<g, kKnnThreads, 0, s>>>(t, xy_sorted_.as<double2>(), dp, n, order, nullptr, \
                                              k, slack_, di, dd, ev);                            \
  else                                                                                           \
    k_knn<KK, false><<<g, kKnnThreads, 0, s>>>(t, xy_sorted_.as<double2>(), dp, n, order,        \
                                               nullptr, k, slack_, di, dd, ev);
      if (k <= 8) {
        SPJ_KNN_LAUNCH(8)
      } else if (k <= 16) {
        SPJ_KNN_LAUNCH(16)
      } else {
        SPJ_KNN_LAUNCH(32)
      }
#undef SPJ_KNN_LAUNCH
    }
    SPJ_CUDA(cudaGetLastError());
  }
  if (!device_ptrs && n) {
    SPJ_CUDA(cudaMemcpyAsync(out_idx, di, n * k * 4, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaMemcpyAsync(out_dist, dd, n * k * 8, cudaMemcpyDeviceToHost, s));
  }
  unsigned long long cnt[2] = {0, 0};
  SPJ_CUDA(cudaMemcpyAsync(cnt, counters_.get(), 16, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  check_traversal(bvh_.view(), s);
  exact_evals_ += cnt[0];
  redone_ += (uint32_t)cnt[1];
  queries_ += n;
}

}  // namespace spj
