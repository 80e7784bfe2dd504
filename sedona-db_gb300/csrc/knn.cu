// knn.cu — KNN join: LBVH over the build points, depth-first traversal
// nearest child first, a register-resident k-best list per probe thread.
//
// Ranking key: the exact squared distance dx^2 + dy^2 of the FP64 deltas
// dx = RN(b.x - p.x), dy = RN(b.y - p.y) (the deltas the reference's
// Euclidean distance forms), held as a normalized double-double (hi, lo) and
// compared lexicographically, then by build id.  Exact duplicates tie on the
// key and fall back to the build id, as in the reference ground truth.
// Chosen form: node pruning and point rejection in FP32 with a static error
// bound; only points that may enter the k-best list get the FP64 key.
// Plain form: every visited point gets the FP64 key.
#include "knn.cuh"
#include "prims.cuh"

#include <cmath>
#include <vector>

namespace spj {
namespace {

constexpr int kKnnThreads = 128;
constexpr int kKnnStack = 64;

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

template <int K, bool kFast>
__global__ void __launch_bounds__(kKnnThreads)
    k_knn(LbvhView t, const double2* __restrict__ bxy, const double2* __restrict__ probe,
          uint64_t n, uint32_t k, float slack, uint32_t* __restrict__ out_idx,
          double* __restrict__ out_dist, unsigned long long* __restrict__ exact_evals) {
  __shared__ int stack[kKnnStack * kKnnThreads];
  uint32_t evals = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t start = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t trips = (n + stride - 1) / stride;
  for (uint64_t tr = 0; tr < trips; tr++) {
    const uint64_t qi = start + tr * stride;
    if (qi >= n) continue;
    const double2 q = probe[qi];
    const float2 q32 = make_float2(__double2float_rn(q.x), __double2float_rn(q.y));
    // |q - q32| bound, plus the build-side bound
    const float qs = __fadd_ru(__fmul_ru(fabsf(q32.x) + fabsf(q32.y), 1.1920929e-07f), slack);
    double kh[K], kl[K];
    uint32_t ki[K];
#pragma unroll
    for (int j = 0; j < K; j++) {
      kh[j] = INFINITY;
      kl[j] = 0;
      ki[j] = 0xFFFFFFFFu;
    }
    uint32_t have = 0;
    float bound = INFINITY;  // FP32 upper bound of the k-th best distance
    const bool valid = !(isnan(q.x) || isnan(q.y)) && t.nprims > 0;
    int sp = 0;
    int node = valid ? (t.nleaves > 1 ? 0 : ~0) : 0;
    bool done = !valid;
    while (!done) {
      if (node < 0) {
        const uint32_t c = (uint32_t)(~node);
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
          for (int j = K - 1; j > 0; j--) {
            if (!placed) {
              if (key_less(h, l, id, kh[j - 1], kl[j - 1], ki[j - 1])) {
                kh[j] = kh[j - 1];
                kl[j] = kl[j - 1];
                ki[j] = ki[j - 1];
              } else {
                kh[j] = h;
                kl[j] = l;
                ki[j] = id;
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
            for (int j = 0; j < K; j++)
              if (j == (int)k - 1) kth = __dadd_rn(kh[j], kl[j]);
            bound = __double2float_ru(sqrt(kth) * (1.0 + 1e-12));
          }
        }
      } else {
        const float4 lb = t.node_box[2 * node], rb = t.node_box[2 * node + 1];
        const int2 ch = t.node_child[node];
        // conservative lower bounds of the true distance
        const float dl = __fsub_rd(__fmul_rd(box_dist(q32, lb), 0.99999905f), qs);
        const float dr = __fsub_rd(__fmul_rd(box_dist(q32, rb), 0.99999905f), qs);
        const bool vl = dl <= bound, vr = dr <= bound;
        if (vl && vr) {
          const int nearc = dl <= dr ? ch.x : ch.y;
          const int farc = dl <= dr ? ch.y : ch.x;
          if (sp < kKnnStack) stack[sp * kKnnThreads + threadIdx.x] = farc;
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
      node = sp < kKnnStack ? stack[sp * kKnnThreads + threadIdx.x] : 0;
    }
    for (uint32_t j = 0; j < k; j++) {
      uint32_t id = 0xFFFFFFFFu;
      double d = INFINITY;
#pragma unroll
      for (int jj = 0; jj < K; jj++)
        if (jj == (int)j && jj < (int)have) {
          id = ki[jj];
          d = sqrt(__dadd_rn(kh[jj], kl[jj]));
        }
      out_idx[qi * k + j] = id;
      out_dist[qi * k + j] = d;
    }
  }
  for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
  if ((threadIdx.x & 31) == 0 && evals) atomicAdd(exact_evals, (unsigned long long)evals);
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

__global__ void k_gather_xy(const double2* __restrict__ xy, const uint32_t* __restrict__ ids,
                            uint32_t m, double2* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    out[i] = xy[ids[i]];
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
    probe_.release();
    oidx_.release();
    odist_.release();
    counters_.release();
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
  if (bvh_.nprims)
    k_gather_xy<<<grid_for(bvh_.nprims, 256), 256, 0, s>>>(
        xy.as<double2>(), bvh_.sorted_id.as<uint32_t>(), bvh_.nprims, xy_sorted_.as<double2>());
  // |p - RN32(p)| <= 2^-24 (|x| + |y|) <= 2^-24 * 2 * max|coord|
  double mx = 0;
  for (uint64_t i = 0; i < 2 * n; i++) {
    double v = std::fabs(xy_host[i]);
    if (v > mx && std::isfinite(v)) mx = v;
  }
  slack_ = (float)(mx * 2.0 * std::ldexp(1.0, -23));
  SPJ_CUDA(cudaStreamSynchronize(s));
}

void KnnIndex::query(const double* probe_xy, uint64_t n, uint32_t k, uint32_t* out_idx,
                     double* out_dist, bool device_ptrs) {
  SPJ_CHECK(k >= 1 && k <= 32, "k must be in [1, 32]");
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
  SPJ_CUDA(cudaMemsetAsync(counters_.get(), 0, 8, s));
  if (n) {
    const LbvhView t = bvh_.view();
    const int g = grid_for((int64_t)n, kKnnThreads, kNumSMs * 16);
    auto* ev = counters_.as<unsigned long long>();
#define SPJ_KNN_LAUNCH(KK)                                                                    \
  if (form_ == 1)                                                                             \
    k_knn<KK, true><<<g, kKnnThreads, 0, s>>>(t, xy_sorted_.as<double2>(), dp, n, k, slack_,  \
                                              di, dd, ev);                                    \
  else                                                                                        \
    k_knn<KK, false><<<g, kKnnThreads, 0, s>>>(t, xy_sorted_.as<double2>(), dp, n, k, slack_, \
                                               di, dd, ev);
    if (k <= 8) {
      SPJ_KNN_LAUNCH(8)
    } else if (k <= 16) {
      SPJ_KNN_LAUNCH(16)
    } else {
      SPJ_KNN_LAUNCH(32)
    }
#undef SPJ_KNN_LAUNCH
    SPJ_CUDA(cudaGetLastError());
  }
  if (!device_ptrs && n) {
    SPJ_CUDA(cudaMemcpyAsync(out_idx, di, n * k * 4, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaMemcpyAsync(out_dist, dd, n * k * 8, cudaMemcpyDeviceToHost, s));
  }
  unsigned long long ev = 0;
  SPJ_CUDA(cudaMemcpyAsync(&ev, counters_.get(), 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  exact_evals_ += ev;
}

}  // namespace spj
