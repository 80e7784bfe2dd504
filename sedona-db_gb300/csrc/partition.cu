// partition.cu — the partitioned (out-of-core) join: box passes over both
// columns in host memory, the KDB partitioner (built on the host from a
// sample, applied on the device), partition bounds, probe assignment, then
// one build + probe pass per partition.  See partition.cuh for the rules and
// the reference they follow.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>

#include "geoms.cuh"
#include "lbvh.cuh"
#include "materialize.cuh"
#include "partition.cuh"
#include "prims.cuh"

namespace spj {
namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kKdbStack = 64;  // the device walk's stack: trees up to 62 levels
constexpr uint32_t kMaxLeaves = 4096;

struct KdbDev {
  float4 ext;  // (min x, min y, max x, max y)
  int32_t child0, child1, leaf, pad;
};

// ---------------------------------------------------------------------------
// The KDB tree on the host, restating kdb.rs:116-459: a leaf takes items until
// it holds max_items (or sits at max_levels); then it splits at the median
// item's min coordinate along its longer side (the shorter one if that
// fails), keeping points on the line on the low side.

class Kdb {
 public:
  struct Node {
    float x0, y0, x1, y1;
    uint32_t level;
    int32_t child[2] = {-1, -1};
    int32_t leaf = -1;
    std::vector<float4> items;
  };
  std::vector<Node> nodes;
  size_t max_items;
  size_t max_levels;

  Kdb(size_t mi, size_t ml, float4 ext) : max_items(mi), max_levels(ml) {
    Node r;
    r.x0 = ext.x;
    r.y0 = ext.y;
    r.x1 = ext.z;
    r.y1 = ext.w;
    r.level = 0;
    nodes.push_back(std::move(r));
  }
  static bool contains(const Node& n, float x, float y) {
    return x >= n.x0 && x <= n.x1 && y >= n.y0 && y <= n.y1;
  }
  void insert(float4 r) {
    if (contains(nodes[0], r.x, r.y)) insert_rect(0, r);
  }
  void insert_rect(int i, float4 r) {
    if (nodes[i].child[0] < 0) {
      if (nodes[i].items.size() < max_items || nodes[i].level >= max_levels) {
        nodes[i].items.push_back(r);
        return;
      }
      const bool sx = (nodes[i].x1 - nodes[i].x0) > (nodes[i].y1 - nodes[i].y0);
      if (!split(i, sx) && !split(i, !sx)) {
        nodes[i].items.push_back(r);
        return;
      }
    }
    for (int c = 0; c < 2; c++) {
      const int ci = nodes[i].child[c];
      if (contains(nodes[ci], r.x, r.y)) {
        insert_rect(ci, r);
        break;
      }
    }
  }
  bool split(int i, bool sx) {
    std::vector<float4>& items = nodes[i].items;
    std::stable_sort(items.begin(), items.end(), [sx](const float4& a, const float4& b) {
      const float a1 = sx ? a.x : a.y, b1 = sx ? b.x : b.y;
      if (a1 != b1) return a1 < b1;
      const float a2 = sx ? a.y : a.x, b2 = sx ? b.y : b.x;
      return a2 < b2;
    });
    const float4 mid = items[items.size() / 2];
    const float c = sx ? mid.x : mid.y;
    const Node n = Node{nodes[i].x0, nodes[i].y0, nodes[i].x1, nodes[i].y1, nodes[i].level};
    if (sx ? (c <= n.x0 || c >= n.x1) : (c <= n.y0 || c >= n.y1)) return false;
    Node l, r;
    l.level = r.level = n.level + 1;
    if (sx) {
      l.x0 = n.x0, l.y0 = n.y0, l.x1 = c, l.y1 = n.y1;
      r.x0 = c, r.y0 = n.y0, r.x1 = n.x1, r.y1 = n.y1;
    } else {
      l.x0 = n.x0, l.y0 = n.y0, l.x1 = n.x1, l.y1 = c;
      r.x0 = n.x0, r.y0 = c, r.x1 = n.x1, r.y1 = n.y1;
    }
    std::vector<float4> moved;
    moved.swap(nodes[i].items);
    const int li = (int)nodes.size();
    nodes.push_back(std::move(l));
    nodes.push_back(std::move(r));
    nodes[i].child[0] = li;
    nodes[i].child[1] = li + 1;
    for (const float4& it : moved) insert_rect((sx ? it.x : it.y) <= c ? li : li + 1, it);
    return true;
  }
  // leaf ids in depth-first order, children[0] first (kdb.rs assign_leaf_ids)
  uint32_t assign_leaf_ids() {
    uint32_t next = 0;
    std::vector<int> st{0};
    while (!st.empty()) {
      const int i = st.back();
      st.pop_back();
      if (nodes[i].child[0] < 0) {
        nodes[i].leaf = (int)next++;
      } else {
        st.push_back(nodes[i].child[1]);
        st.push_back(nodes[i].child[0]);
      }
    }
    return next;
  }
  uint32_t depth() const {
    uint32_t d = 0;
    for (const Node& n : nodes) d = std::max(d, n.level);
    return d;
  }
};

// order-preserving float <-> uint32 (for atomic min / max)
__host__ __device__ __forceinline__ uint32_t f2o(float f) {
#ifdef __CUDA_ARCH__
  const uint32_t u = __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
#endif
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float o2f(uint32_t o) {
  const uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

__device__ __forceinline__ bool box_ok(float4 b) { return !isnan(b.x); }

__global__ void k_extent(const float4* __restrict__ box, uint64_t n, uint32_t* acc) {
  uint32_t mnx = 0xffffffffu, mny = 0xffffffffu, mxx = 0, mxy = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float4 b = box[i];
    if (!box_ok(b)) continue;
    mnx = min(mnx, f2o(b.x));
    mny = min(mny, f2o(b.y));
    mxx = max(mxx, f2o(b.z));
    mxy = max(mxy, f2o(b.w));
  }
  // warp, then block, then one global atomic per word and block (global
  // atomics on four words from every warp would serialise in L2)
  __shared__ uint32_t blk[4];
  if (threadIdx.x < 4) blk[threadIdx.x] = threadIdx.x < 2 ? 0xffffffffu : 0u;
  __syncthreads();
  mnx = __reduce_min_sync(0xffffffffu, mnx);
  mny = __reduce_min_sync(0xffffffffu, mny);
  mxx = __reduce_max_sync(0xffffffffu, mxx);
  mxy = __reduce_max_sync(0xffffffffu, mxy);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(blk + 0, mnx);
    atomicMin(blk + 1, mny);
    atomicMax(blk + 2, mxx);
    atomicMax(blk + 3, mxy);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicMin(acc + 0, blk[0]);
    atomicMin(acc + 1, blk[1]);
    atomicMax(acc + 2, blk[2]);
    atomicMax(acc + 3, blk[3]);
  }
}

__device__ __forceinline__ bool meets(float4 a, float4 b) {
  return a.x <= b.z && a.z >= b.x && a.y <= b.w && a.w >= b.y;
}

// partition_no_multi: the leaf the box overlaps most (kdb.rs rect_intersection_area;
// the first leaf in depth-first order wins a tie)
__global__ void k_kdb_assign(const float4* __restrict__ box, uint64_t n,
                             const KdbDev* __restrict__ nodes, uint32_t* __restrict__ part) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float4 b = box[i];
    uint32_t best = kNone;
    if (box_ok(b)) {
      float best_area = -1.f;
      int32_t st[kKdbStack];
      int sp = 0;
      st[sp++] = 0;
      while (sp > 0) {
        const KdbDev nd = nodes[st[--sp]];
        if (!meets(nd.ext, b)) continue;
        if (nd.leaf >= 0) {
          const float w = fmaxf(fminf(b.z, nd.ext.z) - fmaxf(b.x, nd.ext.x), 0.f);
          const float h = fmaxf(fminf(b.w, nd.ext.w) - fmaxf(b.y, nd.ext.y), 0.f);
          const float area = w * h;
          if (area > best_area) {
            best_area = area;
            best = (uint32_t)nd.leaf;
          }
        } else if (sp + 2 <= kKdbStack) {  // the host keeps trees within the stack
          st[sp++] = nd.child1;
          st[sp++] = nd.child0;
        }
      }
    }
    part[i] = best;
  }
}

// The union of each partition's build boxes (ordered-integer min / max).  A
// warp reduces its rows partition by partition (the distinct partitions of
// 32 rows), then the block accumulates in shared memory (nparts <=
// kBoundsSmemParts; dynamic shared memory of 16 * nparts bytes) and issues
// one global atomic per word it touched; with more partitions the warps'
// results go to global memory directly.  (Four global atomics per row on a
// few words serialise in L2.)
constexpr uint32_t kBoundsSmemParts = 1024;
__global__ void k_bounds(const float4* __restrict__ box, const uint32_t* __restrict__ part,
                         uint64_t n, uint32_t nparts, uint32_t* acc) {
  extern __shared__ uint32_t sacc[];
  const bool smem = nparts <= kBoundsSmemParts;
  if (smem) {
    for (uint32_t k = threadIdx.x; k < 4 * nparts; k += blockDim.x)
      sacc[k] = (k & 3) < 2 ? 0xffffffffu : 0u;
    __syncthreads();
  }
  uint32_t* dst = smem ? sacc : acc;
  const int lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t end = (n + 31) / 32 * 32;  // whole warps take every turn
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < end; i += stride) {
    uint32_t p = nparts;
    uint32_t x0 = 0xffffffffu, y0 = 0xffffffffu, x1 = 0u, y1 = 0u;
    if (i < n) {
      p = part[i];
      if (p < nparts) {
        const float4 b = box[i];
        x0 = f2o(b.x);
        y0 = f2o(b.y);
        x1 = f2o(b.z);
        y1 = f2o(b.w);
      }
    }
    unsigned todo = __ballot_sync(0xffffffffu, p < nparts);
    while (todo) {
      const int leader = __ffs(todo) - 1;
      const uint32_t pl = __shfl_sync(0xffffffffu, p, leader);
      const bool mine = p == pl;
      const uint32_t a = __reduce_min_sync(0xffffffffu, mine ? x0 : 0xffffffffu);
      const uint32_t b = __reduce_min_sync(0xffffffffu, mine ? y0 : 0xffffffffu);
      const uint32_t c = __reduce_max_sync(0xffffffffu, mine ? x1 : 0u);
      const uint32_t d = __reduce_max_sync(0xffffffffu, mine ? y1 : 0u);
      if (lane == leader) {
        atomicMin(dst + 4 * pl + 0, a);
        atomicMin(dst + 4 * pl + 1, b);
        atomicMax(dst + 4 * pl + 2, c);
        atomicMax(dst + 4 * pl + 3, d);
      }
      todo &= ~__ballot_sync(0xffffffffu, mine);
    }
  }
  if (smem) {
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < 4 * nparts; k += blockDim.x) {
      const uint32_t v = sacc[k];
      if ((k & 3) < 2) {
        if (v != 0xffffffffu) atomicMin(acc + k, v);
      } else if (v != 0u) {
        atomicMax(acc + k, v);
      }
    }
  }
}

// FlatPartitioner::partition over the partitions' bounds: the one partition
// met, nparts (Multi) for several, nparts + 1 (None) for none
__global__ void k_flat_assign(const float4* __restrict__ box, uint64_t n,
                              const float4* __restrict__ bounds, uint32_t nparts,
                              uint32_t* __restrict__ part) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float4 b = box[i];
    uint32_t r = nparts + 1;
    if (box_ok(b)) {
      for (uint32_t k = 0; k < nparts; k++) {
        if (!meets(bounds[k], b)) continue;
        if (r == nparts + 1) {
          r = k;
        } else {
          r = nparts;
          break;
        }
      }
    }
    part[i] = r;
  }
}

__global__ void k_iota(uint32_t* __restrict__ v, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    v[i] = (uint32_t)i;
}

// kNone -> nbins - 1 so that the keys sort into bins; one atomic per group
// of lanes with the same bin (most rows of a warp share one)
__global__ void k_hist(uint32_t* __restrict__ part, uint64_t n, uint32_t nbins,
                       uint32_t* __restrict__ count) {
  // the block's counts in shared memory (dynamic, 4 * nbins bytes), then one
  // global atomic per non-empty bin and block
  extern __shared__ uint32_t scount[];
  for (uint32_t k = threadIdx.x; k < nbins; k += blockDim.x) scount[k] = 0;
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t end = (n + 31) / 32 * 32;  // whole warps take every turn
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < end; i += stride) {
    uint32_t p = 0xFFFFFFFFu;
    if (i < n) {
      p = part[i];
      if (p >= nbins) p = nbins - 1;
      part[i] = p;
    }
    const unsigned grp = __match_any_sync(0xffffffffu, p);
    if (i < n && (threadIdx.x & 31) == (unsigned)(__ffs(grp) - 1))
      atomicAdd(scount + p, (uint32_t)__popc(grp));
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < nbins; k += blockDim.x)
    if (scount[k]) atomicAdd(count + k, scount[k]);
}

__global__ void k_map_pairs(const uint32_t* __restrict__ db, const uint32_t* __restrict__ dp,
                            uint64_t m, const uint32_t* __restrict__ brows,
                            const uint32_t* __restrict__ prows, uint32_t* __restrict__ ob,
                            uint32_t* __restrict__ op) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    ob[i] = brows[db[i]];
    op[i] = prows[dp[i]];
  }
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

uint64_t host_off(const HostWkbColumn& c, int64_t i) {
  return c.offsets64 ? (uint64_t) static_cast<const int64_t*>(c.offsets)[i]
                     : (uint64_t)(uint32_t) static_cast<const int32_t*>(c.offsets)[i];
}

// A host column as the device sees it: straight through when the device can
// read pageable host memory, else not at all (rows are then staged).
struct ColumnAccess {
  const HostWkbColumn& h;
  bool direct;
  WkbDeviceColumn whole() const {
    WkbDeviceColumn c;
    c.n = h.n;
    c.offsets = h.offsets;
    c.offsets64 = h.offsets64;
    c.data = h.data;
    c.data_len = h.n ? host_off(h, h.n) : 0;
    c.validity = h.validity;
    c.validity_offset = h.validity_offset;
    return c;
  }
};

// Rows [r0, r1) of a host column on the device, for the box pass: a view
// into host memory, or a copy of the rows' contiguous bytes.
struct RangeStage {
  DevBuf off, data, valid;
  std::vector<int64_t> hoff;
  WkbDeviceColumn view(const ColumnAccess& a, int64_t r0, int64_t r1, cudaStream_t s) {
    const HostWkbColumn& h = a.h;
    WkbDeviceColumn c;
    c.n = r1 - r0;
    if (a.direct) {
      c.offsets = static_cast<const uint8_t*>(h.offsets) + r0 * (h.offsets64 ? 8 : 4);
      c.offsets64 = h.offsets64;
      c.data = h.data;
      c.data_len = host_off(h, h.n);
      c.validity = h.validity;
      c.validity_offset = h.validity_offset + r0;
      return c;
    }
    const uint64_t b0 = host_off(h, r0), b1 = host_off(h, r1);
    hoff.resize((size_t)(r1 - r0) + 1);
    for (int64_t i = r0; i <= r1; i++) hoff[i - r0] = (int64_t)(host_off(h, i) - b0);
    off.reserve(hoff.size() * 8, s);
    data.reserve(b1 - b0 + 16, s);
    SPJ_CUDA(cudaMemcpyAsync(off.get(), hoff.data(), hoff.size() * 8, cudaMemcpyHostToDevice, s));
    if (b1 > b0)
      SPJ_CUDA(cudaMemcpyAsync(data.get(), h.data + b0, b1 - b0, cudaMemcpyHostToDevice, s));
    c.offsets = off.get();
    c.offsets64 = true;
    c.data = data.as<uint8_t>();
    c.data_len = b1 - b0;
    c.validity = nullptr;
    c.validity_offset = 0;
    if (h.validity) {
      const int64_t v0 = h.validity_offset + r0, v1 = h.validity_offset + r1;
      const int64_t byte0 = v0 >> 3, byte1 = (v1 + 7) >> 3;
      valid.reserve((size_t)(byte1 - byte0) + 16, s);
      SPJ_CUDA(cudaMemcpyAsync(valid.get(), h.validity + byte0, (size_t)(byte1 - byte0),
                               cudaMemcpyHostToDevice, s));
      c.validity = valid.as<uint8_t>();
      c.validity_offset = v0 & 7;
    }
    SPJ_CUDA(cudaStreamSynchronize(s));  // hoff is reused by the next range
    return c;
  }
};

// The f32 boxes of every row of a host column (NaN for null / empty rows),
// decoded in row ranges; probe boxes are expanded by the ST_DWithin distance.
void column_boxes(const ColumnAccess& a, DevBuf& boxes, bool expand, double distance,
                  const double* d_dist, cudaStream_t s) {
  const int64_t n = a.h.n;
  boxes.reserve((size_t)(n + 1) * sizeof(float4), s);
  RangeStage stage;
  DeviceGeoms g;
  DecodeScratch sc;
  const int64_t kRows = 1 << 22;
  const uint64_t kBytes = 1ull << 30;
  int64_t r0 = 0;
  while (r0 < n) {
    int64_t r1 = std::min(n, r0 + kRows);
    // keep a range's bytes bounded
    while (r1 - r0 > 1024 && host_off(a.h, r1) - host_off(a.h, r0) > kBytes) r1 = r0 + (r1 - r0) / 2;
    const WkbDeviceColumn c = stage.view(a, r0, r1, s);
    decode_wkb(c, g, sc, false, s);
    float4* out = boxes.as<float4>() + r0;
    if (expand)
      expand_boxes(g.view(), distance, d_dist ? d_dist + r0 : nullptr, out, s);
    else
      SPJ_CUDA(cudaMemcpyAsync(out, g.box.get(), (size_t)(r1 - r0) * sizeof(float4),
                               cudaMemcpyDeviceToDevice, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    r0 = r1;
  }
}

// Rows idx (device, n of them) of a host column into a device large_binary
// column: read by the device from host memory, or gathered by host threads
// into page-locked memory and copied.
struct RowGather {
  DevBuf off, data, len, pos, tmp;
  PinnedBuf hdata, hoff;
  size_t hdata_cap = 0, hoff_cap = 0;
  std::vector<uint32_t> hidx;
  WkbDeviceColumn gather(const ColumnAccess& a, const uint32_t* d_idx, uint64_t n,
                         cudaStream_t s) {
    WkbDeviceColumn c;
    c.n = (int64_t)n;
    c.offsets64 = true;
    if (a.direct) {
      c.data_len = gather_binary(a.whole(), d_idx, n, off, data, len, pos, tmp, s);
      c.offsets = off.get();
      c.data = data.as<uint8_t>();
      return c;
    }
    const HostWkbColumn& h = a.h;
    hidx.resize(n);
    if (n)
      SPJ_CUDA(cudaMemcpyAsync(hidx.data(), d_idx, n * 4, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    if ((n + 1) * 8 > hoff_cap) {
      hoff.reserve((n + 1) * 8);
      hoff_cap = (n + 1) * 8;
    }
    int64_t* o = hoff.as<int64_t>();
    o[0] = 0;
    for (uint64_t i = 0; i < n; i++)
      o[i + 1] = o[i] + (int64_t)(host_off(h, hidx[i] + 1) - host_off(h, hidx[i]));
    const uint64_t total = (uint64_t)o[n];
    if (total + 16 > hdata_cap) {
      hdata.reserve(total + 16);
      hdata_cap = total + 16;
    }
    uint8_t* d = hdata.as<uint8_t>();
    const size_t nt = std::min<size_t>({8, std::max(1u, std::thread::hardware_concurrency()),
                                        (size_t)(n / 4096) + 1});
    auto run = [&](size_t t) {
      for (uint64_t i = t * n / nt; i < (t + 1) * n / nt; i++)
        memcpy(d + o[i], h.data + host_off(h, hidx[i]), (size_t)(o[i + 1] - o[i]));
    };
    std::vector<std::thread> th;
    for (size_t t = 1; t < nt; t++) th.emplace_back(run, t);
    run(0);
    for (auto& t : th) t.join();
    off.reserve((n + 1) * 8, s);
    data.reserve(total + 16, s);
    SPJ_CUDA(cudaMemcpyAsync(off.get(), o, (n + 1) * 8, cudaMemcpyHostToDevice, s));
    if (total) SPJ_CUDA(cudaMemcpyAsync(data.get(), d, total, cudaMemcpyHostToDevice, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    c.offsets = off.get();
    c.data = data.as<uint8_t>();
    c.data_len = total;
    return c;
  }
};

}  // namespace

int run_partitioned(JoinEngine& eng, Workspace& ws, const HostWkbColumn& build,
                    const HostWkbColumn& probe, int predicate, double distance,
                    const double* d_dist, const PartitionOptions& opt, PartitionStats* stats,
                    PartitionLayout* layout, const PairSink& sink) {
  cudaStream_t s = ws.stream;
  PartitionStats st;
  int dev = 0, pageable = 0;
  SPJ_CUDA(cudaGetDevice(&dev));
  SPJ_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
  const bool direct = pageable && !opt.host_gather;
  st.direct_host_reads = direct;
  const ColumnAccess ba{build, direct}, pa{probe, direct};
  SPJ_CHECK(build.n < (int64_t)kNone && probe.n < (int64_t)kNone, "more than 2^32 - 1 rows");
  const bool dwithin = predicate == 100;

  // 1. boxes of both sides
  auto t0 = std::chrono::steady_clock::now();
  DevBuf bbox, pbox;
  column_boxes(ba, bbox, false, 0.0, nullptr, s);
  column_boxes(pa, pbox, dwithin, distance, d_dist, s);
  st.ms_boxes = ms_since(t0);

  // 2. the KDB tree from a sample of the build boxes
  t0 = std::chrono::steady_clock::now();
  const uint64_t nb = (uint64_t)build.n, np = (uint64_t)probe.n;
  DevBuf acc(16, s);
  const uint32_t init[4] = {0xffffffffu, 0xffffffffu, 0u, 0u};
  SPJ_CUDA(cudaMemcpyAsync(acc.get(), init, 16, cudaMemcpyHostToDevice, s));
  if (nb)
    k_extent<<<grid_for((int64_t)nb, 256, kNumSMs * 8), 256, 0, s>>>(bbox.as<float4>(), nb,
                                                                      acc.as<uint32_t>());
  uint32_t ext_o[4];
  SPJ_CUDA(cudaMemcpyAsync(ext_o, acc.get(), 16, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  const bool any_build = nb && ext_o[0] != 0xffffffffu;
  const float4 extent = any_build ? make_float4(o2f(ext_o[0]), o2f(ext_o[1]), o2f(ext_o[2]),
                                                o2f(ext_o[3]))
                                  : make_float4(0.f, 0.f, 0.f, 0.f);
  uint64_t build_bytes = nb ? host_off(build, build.n) - host_off(build, 0) : 0;
  uint32_t target = opt.num_partitions;
  if (target == 0)
    target = opt.build_budget_bytes
                 ? (uint32_t)std::min<uint64_t>(
                       kMaxLeaves, (build_bytes * 5 / 2 + opt.build_budget_bytes - 1) /
                                       opt.build_budget_bytes)
                 : 1;
  target = std::max(1u, std::min(target, kMaxLeaves));
  // the sample: distinct rows in a seeded order (splitmix64), valid boxes only
  const uint32_t want = opt.sample_rows ? opt.sample_rows : 10000;
  std::vector<float4> samples;
  if (any_build) {
    const uint64_t m = std::min<uint64_t>(nb, (uint64_t)want * 2);
    std::vector<uint32_t> pick(m);
    uint64_t x = opt.seed + 0x9e3779b97f4a7c15ull;
    for (uint64_t i = 0; i < m; i++) {
      // a random row per slot of an even stride: covers the column, no repeats
      x += 0x9e3779b97f4a7c15ull;
      uint64_t z = x;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      z ^= z >> 31;
      const uint64_t lo = i * nb / m, hi = (i + 1) * nb / m;
      pick[i] = (uint32_t)(lo + (hi > lo ? z % (hi - lo) : 0));
    }
    // the sampled boxes, as two 8-byte halves each through the 8-byte gather
    std::vector<uint32_t> i2(2 * m);
    for (uint64_t i = 0; i < m; i++) {
      i2[2 * i] = 2 * pick[i];
      i2[2 * i + 1] = 2 * pick[i] + 1;
    }
    std::vector<float4> all_s(m);
    DevBuf idx2(m * 8, s), tmpbox(m * 16, s);
    SPJ_CUDA(cudaMemcpyAsync(idx2.get(), i2.data(), m * 8, cudaMemcpyHostToDevice, s));
    gather_u64(reinterpret_cast<const uint64_t*>(bbox.get()), 2 * nb, idx2.as<uint32_t>(), 2 * m,
               tmpbox.as<uint64_t>(), s);
    SPJ_CUDA(cudaMemcpyAsync(all_s.data(), tmpbox.get(), m * 16, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    for (const float4& b : all_s)
      if (!std::isnan(b.x) && samples.size() < want) samples.push_back(b);
    // the reference shuffles its sample before building (prepare.rs:286)
    for (size_t i = samples.size(); i > 1; i--) {
      x += 0x9e3779b97f4a7c15ull;
      uint64_t z = x;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      z ^= z >> 31;
      std::swap(samples[i - 1], samples[z % i]);
    }
  }
  const size_t max_items = std::max<size_t>(1, samples.size() / target);
  Kdb kdb(max_items, target, extent);
  for (const float4& b : samples) kdb.insert(b);
  const uint32_t nleaves = kdb.assign_leaf_ids();
  SPJ_CHECK(kdb.depth() + 2 < (uint32_t)kKdbStack, "KDB tree deeper than 61 levels");
  SPJ_CHECK(nleaves <= kMaxLeaves, "more than 4096 partitions");
  std::vector<KdbDev> hn(kdb.nodes.size());
  std::vector<float4> leaf_ext(nleaves);
  for (size_t i = 0; i < kdb.nodes.size(); i++) {
    const Kdb::Node& nd = kdb.nodes[i];
    hn[i].ext = make_float4(nd.x0, nd.y0, nd.x1, nd.y1);
    hn[i].child0 = nd.child[0];
    hn[i].child1 = nd.child[1];
    hn[i].leaf = nd.leaf;
    if (nd.leaf >= 0) leaf_ext[nd.leaf] = hn[i].ext;
  }
  DevBuf dnodes(hn.size() * sizeof(KdbDev), s);
  SPJ_CUDA(cudaMemcpyAsync(dnodes.get(), hn.data(), hn.size() * sizeof(KdbDev),
                           cudaMemcpyHostToDevice, s));

  // 3. build rows to leaves, partition bounds, probe rows to partitions
  DevBuf bpart((nb + 1) * 4, s), ppart((np + 1) * 4, s);
  if (nb)
    k_kdb_assign<<<grid_for((int64_t)nb, 128, kNumSMs * 16), 128, 0, s>>>(
        bbox.as<float4>(), nb, dnodes.as<KdbDev>(), bpart.as<uint32_t>());
  DevBuf bacc(16 * (size_t)nleaves, s);
  {
    std::vector<uint32_t> ia(4 * (size_t)nleaves);
    for (uint32_t k = 0; k < nleaves; k++) {
      ia[4 * k] = ia[4 * k + 1] = 0xffffffffu;
      ia[4 * k + 2] = ia[4 * k + 3] = 0u;
    }
    SPJ_CUDA(cudaMemcpyAsync(bacc.get(), ia.data(), ia.size() * 4, cudaMemcpyHostToDevice, s));
    if (nb)
      k_bounds<<<grid_for((int64_t)nb, 256, kNumSMs * 16), 256,
                 nleaves <= kBoundsSmemParts ? 16 * (size_t)nleaves : 0, s>>>(
          bbox.as<float4>(), bpart.as<uint32_t>(), nb, nleaves, bacc.as<uint32_t>());
    SPJ_CUDA(cudaMemcpyAsync(ia.data(), bacc.get(), ia.size() * 4, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    std::vector<float4> bounds(nleaves);
    const float qnan = std::numeric_limits<float>::quiet_NaN();
    for (uint32_t k = 0; k < nleaves; k++)
      bounds[k] = ia[4 * k] == 0xffffffffu
                      ? make_float4(qnan, qnan, qnan, qnan)  // empty: meets nothing
                      : make_float4(o2f(ia[4 * k]), o2f(ia[4 * k + 1]), o2f(ia[4 * k + 2]),
                                    o2f(ia[4 * k + 3]));
    SPJ_CUDA(cudaMemcpyAsync(bacc.get(), bounds.data(), 16 * (size_t)nleaves,
                             cudaMemcpyHostToDevice, s));
    if (layout) layout->bounds = bounds;
  }
  if (np)
    k_flat_assign<<<grid_for((int64_t)np, 256, kNumSMs * 16), 256, 0, s>>>(
        pbox.as<float4>(), np, bacc.as<float4>(), nleaves, ppart.as<uint32_t>());
  SPJ_CUDA(cudaGetLastError());
  if (layout) {
    layout->samples = samples;
    layout->extent = extent;
    layout->max_items = (uint32_t)max_items;
    layout->max_levels = target;
    layout->leaves = leaf_ext;
    layout->build_part.clear();
    layout->probe_part.clear();
  }
  if (layout && opt.record_layout) {
    layout->build_part.resize(nb);
    layout->probe_part.resize(np);
    if (nb)
      SPJ_CUDA(cudaMemcpyAsync(layout->build_part.data(), bpart.get(), nb * 4,
                               cudaMemcpyDeviceToHost, s));
    if (np)
      SPJ_CUDA(cudaMemcpyAsync(layout->probe_part.data(), ppart.get(), np * 4,
                               cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
  }
  // group rows by partition: build bins 0..L-1 and L (none); probe bins
  // 0..L-1, L (Multi), L+1 (None)
  const uint32_t bbins = nleaves + 1, pbins = nleaves + 2;
  DevBuf bcnt(4 * (size_t)bbins, s), pcnt(4 * (size_t)pbins, s);
  SPJ_CUDA(cudaMemsetAsync(bcnt.get(), 0, 4 * (size_t)bbins, s));
  SPJ_CUDA(cudaMemsetAsync(pcnt.get(), 0, 4 * (size_t)pbins, s));
  if (nb)
    k_hist<<<grid_for((int64_t)nb, 256, kNumSMs * 16), 256, 4 * (size_t)bbins, s>>>(
        bpart.as<uint32_t>(), nb, bbins, bcnt.as<uint32_t>());
  if (np)
    k_hist<<<grid_for((int64_t)np, 256, kNumSMs * 16), 256, 4 * (size_t)pbins, s>>>(
        ppart.as<uint32_t>(), np, pbins, pcnt.as<uint32_t>());
  std::vector<uint32_t> hb(bbins), hp(pbins);
  SPJ_CUDA(cudaMemcpyAsync(hb.data(), bcnt.get(), 4 * (size_t)bbins, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaMemcpyAsync(hp.data(), pcnt.get(), 4 * (size_t)pbins, cudaMemcpyDeviceToHost, s));
  DevBuf brows((nb + 1) * 4, s), prows((np + 1) * 4, s), alt_k((std::max(nb, np) + 1) * 4, s),
      alt_v((std::max(nb, np) + 1) * 4, s), sort_tmp;
  int bits = 1;
  while ((1u << bits) < pbins) bits++;
  if (nb) {
    k_iota<<<grid_for((int64_t)nb, 256), 256, 0, s>>>(brows.as<uint32_t>(), nb);
    radix_sort_pairs(bpart.as<uint32_t>(), brows.as<uint32_t>(), alt_k.as<uint32_t>(),
                     alt_v.as<uint32_t>(), (int64_t)nb, bits, sort_tmp, s);
  }
  if (np) {
    k_iota<<<grid_for((int64_t)np, 256), 256, 0, s>>>(prows.as<uint32_t>(), np);
    radix_sort_pairs(ppart.as<uint32_t>(), prows.as<uint32_t>(), alt_k.as<uint32_t>(),
                     alt_v.as<uint32_t>(), (int64_t)np, bits, sort_tmp, s);
  }
  SPJ_CUDA(cudaStreamSynchronize(s));
  std::vector<uint64_t> bstart(bbins + 1, 0), pstart(pbins + 1, 0);
  for (uint32_t k = 0; k < bbins; k++) bstart[k + 1] = bstart[k] + hb[k];
  for (uint32_t k = 0; k < pbins; k++) pstart[k + 1] = pstart[k] + hp[k];
  const uint64_t n_multi = hp[nleaves];
  st.partitions = nleaves;
  st.probe_rows_multi = n_multi;
  st.probe_rows_none = hp[nleaves + 1];
  st.ms_partition = ms_since(t0);

  // 4. one pass per partition
  t0 = std::chrono::steady_clock::now();
  RowGather gb, gp;
  DevBuf qrows, qdist, ob, op;
  PinnedBuf hob, hop;
  size_t hcap = 0;
  int status = 0;
  for (uint32_t k = 0; k < nleaves && status == 0; k++) {
    const uint64_t nbk = bstart[k + 1] - bstart[k];
    const uint64_t nqk = (pstart[k + 1] - pstart[k]) + n_multi;
    if (nbk == 0 || nqk == 0) continue;
    st.passes++;
    st.build_rows_max = std::max(st.build_rows_max, nbk);
    st.probe_rows_probed += nqk;
    const WkbDeviceColumn bc = gb.gather(ba, brows.as<uint32_t>() + bstart[k], nbk, s);
    eng.build(bc);
    qrows.reserve((nqk + 1) * 4, s);
    const uint64_t nreg = pstart[k + 1] - pstart[k];
    if (nreg)
      SPJ_CUDA(cudaMemcpyAsync(qrows.get(), prows.as<uint32_t>() + pstart[k], nreg * 4,
                               cudaMemcpyDeviceToDevice, s));
    if (n_multi)
      SPJ_CUDA(cudaMemcpyAsync(qrows.as<uint32_t>() + nreg, prows.as<uint32_t>() + pstart[nleaves],
                               n_multi * 4, cudaMemcpyDeviceToDevice, s));
    const WkbDeviceColumn pc = gp.gather(pa, qrows.as<uint32_t>(), nqk, s);
    const double* drow = nullptr;
    if (d_dist) {
      qdist.reserve((nqk + 1) * 8, s);
      gather_u64(reinterpret_cast<const uint64_t*>(d_dist), np, qrows.as<uint32_t>(), nqk,
                 qdist.as<uint64_t>(), s);
      drow = qdist.as<double>();
    }
    const uint32_t *db, *dp;
    const uint64_t m = eng.probe(ws, pc, predicate, distance, 0, &db, &dp, drow);
    st.pairs += m;
    if (!m) continue;
    ob.reserve(m * 4, s);
    op.reserve(m * 4, s);
    k_map_pairs<<<grid_for((int64_t)m, 256, kNumSMs * 16), 256, 0, s>>>(
        db, dp, m, brows.as<uint32_t>() + bstart[k], qrows.as<uint32_t>(), ob.as<uint32_t>(),
        op.as<uint32_t>());
    if (m * 4 > hcap) {
      hob.reserve(m * 4);
      hop.reserve(m * 4);
      hcap = m * 4;
    }
    SPJ_CUDA(cudaMemcpyAsync(hob.as<uint32_t>(), ob.get(), m * 4, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaMemcpyAsync(hop.as<uint32_t>(), op.get(), m * 4, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    status = sink(hob.as<uint32_t>(), hop.as<uint32_t>(), m);
  }
  SPJ_CUDA(cudaStreamSynchronize(s));
  st.ms_passes = ms_since(t0);
  if (stats) *stats = st;
  return status;
}

}  // namespace spj
