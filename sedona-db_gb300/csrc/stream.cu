// stream.cu — the batched probe stream (see stream.cuh), its CUDA graph and
// its autotuner.
#include <chrono>
#include <cstdio>
#include <fstream>
#include <sstream>

#include "predicates.cuh"
#include "prims.cuh"
#include "stream.cuh"
#include "wkb_read.cuh"

namespace spj {
namespace {

using namespace pred;

struct BatchDesc {
  const void* offsets;
  const uint8_t* data;
  uint64_t data_len;
  const uint8_t* validity;
  int64_t validity_offset;
  uint32_t rows;
  uint32_t row_base;
  uint32_t off64;
  uint32_t aligned;
};

struct ChunkDesc {
  uint32_t batch, row0, rows, pad;
};

constexpr int kSStack = 64;

__device__ __forceinline__ bool overlap4(float4 a, float4 b) {
  return !(a.x > b.z || a.z < b.x || a.y > b.w || a.w < b.y);
}

// pred(build row b, probe point p) with the semantics of refine.cu's
// dispatch for a point probe (tg.c intersects/contains/covers/touches
// dispatch; within/coveredby/equals by argument swap).
template <bool kFast>
__device__ __forceinline__ int eval_point_probe(const GeomsView& B, uint32_t b, double2 p,
                                                float2 p32, int predicate, uint32_t& esc) {
  const uint8_t kb = B.kind[b];
  if (kb == kEmpty) return predicate == kDisjoint ? 1 : 0;
  if (kb == kPoint) {
    const bool eq = pteq(B.pt[b], p);
    if (predicate == kTouches) return 0;
    if (predicate == kDisjoint) return !eq;
    return eq;
  }
  const uint32_t q0 = B.row_part[b], q1 = B.row_part[b + 1];
  switch (predicate) {
    case kIntersects:
    case kCovers:
    case kDisjoint: {
      bool hit = false;
      for (uint32_t q = q0; q < q1 && !hit; q++)
        hit = poly_contains_point<kFast>(B, q, p, p32, true, esc);
      return predicate == kDisjoint ? !hit : hit;
    }
    case kContains:
      for (uint32_t q = q0; q < q1; q++)
        if (poly_contains_point<kFast>(B, q, p, p32, false, esc)) return 1;
      return 0;
    case kWithin:
    case kEquals:
      return 0;  // a point contains no polygon (tg.c:1157-1162)
    case kCoveredBy: {
      if (kb != kPolygon) return -1;
      const uint32_t r = B.part_ring[q0];
      if (ring_npts(B, r) < 3) return 0;
      const Rect64 R = B.ring_rect[r];
      return pteq(p, make_double2(R.x, R.y)) && pteq(p, make_double2(R.z, R.w));
    }
    case kTouches:
      if (kb != kPolygon) return -1;
      return poly_touches_point<kFast>(B, q0, p, p32, esc);
  }
  return -1;
}

template <int kThreads, int kPass>
__global__ void __launch_bounds__(kThreads)
    k_stream(GeomsView B, LbvhView t, const BatchDesc* __restrict__ batches,
             const ChunkDesc* __restrict__ chunks, uint32_t nchunks, unsigned* queue,
             int predicate, uint32_t* __restrict__ counts, const uint64_t* __restrict__ offs,
             uint64_t capacity, uint32_t* __restrict__ ob, uint32_t* __restrict__ op,
             DeviceStatus* st) {
  __shared__ int stack[kSStack * kThreads];
  __shared__ uint32_t s_chunk;
  uint32_t esc = 0;
  for (;;) {
    if (threadIdx.x == 0) s_chunk = atomicAdd(queue, 1u);
    __syncthreads();
    const uint32_t c = s_chunk;
    __syncthreads();
    if (c >= nchunks) break;  // block-uniform
    const ChunkDesc ch = chunks[c];
    const BatchDesc bt = batches[ch.batch];
    for (uint32_t r = threadIdx.x; r < ch.rows; r += kThreads) {
      const uint32_t row = ch.row0 + r;
      const uint32_t g = bt.row_base + row;
      bool have = false;
      double2 p = make_double2(0.0, 0.0);
      float2 p32 = make_float2(0.f, 0.f);
      if (wkb::row_valid(bt.validity, bt.validity_offset, row)) {
        uint64_t s, e;
        if (bt.off64) wkb::row_range<true>(bt.offsets, row, s, e);
        else wkb::row_range<false>(bt.offsets, row, s, e);
        if (e < s || e > bt.data_len || s + 21 > e) {
          status_fail(st, kWkbTruncated, g);
        } else if (bt.data[s] > 1) {
          status_fail(st, kWkbByteOrder, g);
        } else {
          const bool le = bt.data[s] == 1;
          const uint32_t type = wkb::read_u32(bt.data, s + 1, bt.data_len, bt.aligned, le);
          if (type != 1) {
            status_fail(st, kWkbType, g);  // the stream path takes point batches
          } else {
            uint32_t w[4];
            wkb::load_words<4>(bt.data, s + 5, bt.data_len, bt.aligned, w);
            const double x = wkb::wkb_f64(w[0], w[1], le), y = wkb::wkb_f64(w[2], w[3], le);
            if (!(isnan(x) && isnan(y))) {
              have = true;
              p = make_double2(x, y);
              p32 = make_float2(__double2float_rn(x), __double2float_rn(y));
            }
          }
        }
      }
      uint32_t cnt = 0;
      uint64_t pos = kPass ? offs[g] : 0;
      if (have && t.nprims > 0) {
        const float4 q = make_float4(p32.x, p32.y, p32.x, p32.y);
        int sp = 0;
        int node = t.nleaves > 1 ? 0 : ~0;
        while (true) {
          if (node < 0) {
            const uint32_t lc = (uint32_t)(~node);
            const uint32_t b0 = lc * t.leaf_size, b1 = min(b0 + t.leaf_size, t.nprims);
            for (uint32_t k = b0; k < b1; k++) {
              if (!overlap4(t.sorted_box[k], q)) continue;
              const uint32_t id = t.sorted_id[k];
              int rr = eval_point_probe<true>(B, id, p, p32, predicate, esc);
              if (rr < 0) {
                status_fail(st, kUnsupported, g);
                rr = 0;
              }
              if (rr) {
                if (kPass) {
                  if (pos < capacity) {
                    ob[pos] = id;
                    op[pos] = g;
                  }
                  pos++;
                } else {
                  cnt++;
                }
              }
            }
          } else {
            const float4 lb = t.node_box[2 * node], rb = t.node_box[2 * node + 1];
            const int2 chn = t.node_child[node];
            const bool hl = overlap4(lb, q), hr = overlap4(rb, q);
            if (hl && hr) {
              if (sp < kSStack) stack[sp * kThreads + threadIdx.x] = chn.y;
              sp++;
              node = chn.x;
              continue;
            }
            if (hl) {
              node = chn.x;
              continue;
            }
            if (hr) {
              node = chn.y;
              continue;
            }
          }
          if (sp == 0) break;
          sp--;
          node = sp < kSStack ? stack[sp * kThreads + threadIdx.x] : 0;
        }
      }
      if (!kPass) counts[g] = cnt;
    }
  }
  // every thread of the block leaves the loop together: warp-aggregate
  for (int o = 16; o > 0; o >>= 1) esc += __shfl_xor_sync(0xffffffffu, esc, o);
  if ((threadIdx.x & 31) == 0 && esc && kPass == 0)
    atomicAdd(&st->counters[0], (unsigned long long)esc);
}

template <int kThreads>
void launch_pass(int pass, int grid, cudaStream_t s, const GeomsView& B, const LbvhView& t,
                 const BatchDesc* batches, const ChunkDesc* chunks, uint32_t nchunks,
                 unsigned* queue, int predicate, uint32_t* counts, const uint64_t* offs,
                 uint64_t capacity, uint32_t* ob, uint32_t* op, DeviceStatus* st) {
  if (pass == 0)
    k_stream<kThreads, 0><<<grid, kThreads, 0, s>>>(B, t, batches, chunks, nchunks, queue,
                                                    predicate, counts, offs, capacity, ob, op, st);
  else
    k_stream<kThreads, 1><<<grid, kThreads, 0, s>>>(B, t, batches, chunks, nchunks, queue,
                                                    predicate, counts, offs, capacity, ob, op, st);
}

template <int kThreads>
int persistent_grid() {
  int dev = 0, sms = 0, per_sm = 0;
  SPJ_CUDA(cudaGetDevice(&dev));
  SPJ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  SPJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stream<kThreads, 0>,
                                                         kThreads, 0));
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace

StreamJoin::StreamJoin(JoinEngine& eng) : eng_(eng) {
  SPJ_CUDA(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
  SPJ_CUDA(cudaMallocHost(&h_total_, 4 * sizeof(uint64_t)));
  SPJ_CUDA(cudaEventCreate(&ev0_));
  SPJ_CUDA(cudaEventCreate(&ev1_));
  ctrl_.alloc(8 + sizeof(DeviceStatus), s_);
  params_.leaf_size = eng_.lbvh().leaf_size;
}

StreamJoin::~StreamJoin() {
  destroy_graph();
  cudaStreamSynchronize(s_);
  batches_.release();
  chunks_.release();
  counts_.release();
  offs_.release();
  sums_.release();
  out_b_.release();
  out_p_.release();
  ctrl_.release();
  cudaStreamSynchronize(s_);
  cudaStreamDestroy(s_);
  cudaFreeHost(h_total_);
  cudaEventDestroy(ev0_);
  cudaEventDestroy(ev1_);
}

void StreamJoin::destroy_graph() {
  if (exec_) cudaGraphExecDestroy(exec_);
  exec_ = nullptr;
  graph_pred_ = -1;
}

void StreamJoin::set_batches(const std::vector<WkbDeviceColumn>& cols) {
  destroy_graph();
  cols_ = cols;
  std::vector<BatchDesc> bd;
  std::vector<ChunkDesc> cd;
  uint64_t base = 0;
  for (size_t i = 0; i < cols.size(); i++) {
    const WkbDeviceColumn& c = cols[i];
    SPJ_CHECK(c.n >= 0 && base + (uint64_t)c.n < 0xFFFFFFFFull, "stream rows exceed 32 bits");
    BatchDesc b;
    b.offsets = c.offsets;
    b.data = c.data;
    b.data_len = c.data_len;
    b.validity = c.validity;
    b.validity_offset = c.validity_offset;
    b.rows = (uint32_t)c.n;
    b.row_base = (uint32_t)base;
    b.off64 = c.offsets64 ? 1 : 0;
    b.aligned = (((uintptr_t)c.data) & 3u) == 0 ? 1 : 0;
    bd.push_back(b);
    for (uint32_t r = 0; r < b.rows; r += params_.chunk_rows)
      cd.push_back(ChunkDesc{(uint32_t)i, r, std::min(params_.chunk_rows, b.rows - r), 0});
    base += (uint64_t)c.n;
  }
  nbatches_ = (uint32_t)bd.size();
  nrows_ = (uint32_t)base;
  nchunks_ = (uint32_t)cd.size();
  batches_.reserve((bd.size() + 1) * sizeof(BatchDesc), s_);
  chunks_.reserve((cd.size() + 1) * sizeof(ChunkDesc), s_);
  if (!bd.empty())
    SPJ_CUDA(cudaMemcpyAsync(batches_.get(), bd.data(), bd.size() * sizeof(BatchDesc),
                             cudaMemcpyHostToDevice, s_));
  if (!cd.empty())
    SPJ_CUDA(cudaMemcpyAsync(chunks_.get(), cd.data(), cd.size() * sizeof(ChunkDesc),
                             cudaMemcpyHostToDevice, s_));
  counts_.reserve(((size_t)nrows_ + 1) * 4, s_);
  offs_.reserve(((size_t)nrows_ + 1) * 8, s_);
  sums_.reserve(scan_tile_sums_bytes(nrows_), s_);
  if (capacity_ == 0) {
    capacity_ = (uint64_t)nrows_ * 4 + 1024;
    out_b_.reserve(capacity_ * 4, s_);
    out_p_.reserve(capacity_ * 4, s_);
  }
  SPJ_CUDA(cudaStreamSynchronize(s_));
  std::ostringstream sig;
  sig << eng_.build_geoms().n << "x" << eng_.build_geoms().nverts << "|" << nrows_ << "|"
      << nbatches_;
  signature_ = sig.str();
}

void StreamJoin::build_graph(int predicate) {
  destroy_graph();
  const GeomsView B = eng_.build_geoms().view();
  const LbvhView t = eng_.lbvh().view();
  unsigned* queue = ctrl_.as<unsigned>();
  DeviceStatus* st = reinterpret_cast<DeviceStatus*>(ctrl_.as<uint8_t>() + 8);
  const BatchDesc* bd = batches_.as<BatchDesc>();
  const ChunkDesc* cd = chunks_.as<ChunkDesc>();
  int grid = 0;
  switch (params_.block) {
    case 64: grid = persistent_grid<64>(); break;
    case 256: grid = persistent_grid<256>(); break;
    default: grid = persistent_grid<128>(); break;
  }
  auto pass = [&](int ps) {
    switch (params_.block) {
      case 64:
        launch_pass<64>(ps, grid, s_, B, t, bd, cd, nchunks_, queue + ps, predicate,
                        counts_.as<uint32_t>(), offs_.as<uint64_t>(), capacity_,
                        out_b_.as<uint32_t>(), out_p_.as<uint32_t>(), st);
        break;
      case 256:
        launch_pass<256>(ps, grid, s_, B, t, bd, cd, nchunks_, queue + ps, predicate,
                         counts_.as<uint32_t>(), offs_.as<uint64_t>(), capacity_,
                         out_b_.as<uint32_t>(), out_p_.as<uint32_t>(), st);
        break;
      default:
        launch_pass<128>(ps, grid, s_, B, t, bd, cd, nchunks_, queue + ps, predicate,
                         counts_.as<uint32_t>(), offs_.as<uint64_t>(), capacity_,
                         out_b_.as<uint32_t>(), out_p_.as<uint32_t>(), st);
        break;
    }
  };
  cudaGraph_t g = nullptr;
  SPJ_CUDA(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
  SPJ_CUDA(cudaMemsetAsync(ctrl_.get(), 0, 8 + sizeof(DeviceStatus), s_));
  SPJ_CUDA(cudaMemsetAsync(st, 0xFF, sizeof(unsigned long long), s_));
  pass(0);
  scan_u32_u64_into(counts_.as<uint32_t>(), offs_.as<uint64_t>(), nrows_, sums_.as<uint64_t>(),
                    s_);
  pass(1);
  SPJ_CUDA(cudaMemcpyAsync(h_total_, offs_.as<uint64_t>() + nrows_, 8, cudaMemcpyDeviceToHost,
                           s_));
  SPJ_CUDA(cudaMemcpyAsync(h_total_ + 1, &st->first_bad, 8, cudaMemcpyDeviceToHost, s_));
  SPJ_CUDA(cudaMemcpyAsync(h_total_ + 2, &st->counters[0], 8, cudaMemcpyDeviceToHost, s_));
  SPJ_CUDA(cudaStreamEndCapture(s_, &g));
  cudaError_t e = cudaGraphInstantiate(&exec_, g, 0);
  cudaGraphDestroy(g);
  SPJ_CUDA(e);
  graph_pred_ = predicate;
  stats_.launches_per_replay = 2 + 3 + 2;  // two passes, three scan kernels, two memsets
}

uint64_t StreamJoin::run(int predicate, const uint32_t** d_build, const uint32_t** d_probe) {
  SPJ_CHECK(eng_.built(), "stream run before the build side was finished");
  SPJ_CHECK(predicate >= 0 && predicate <= 7, "the stream path takes relation predicates");
  SPJ_CHECK(eng_.build_geoms().n == 0 || eng_.build_geoms().has_bands ||
                eng_.build_geoms().nrings == 0,
            "build side has no band index");
  uint64_t total = 0;
  for (int attempt = 0; attempt < 3; attempt++) {
    if (!exec_ || graph_pred_ != predicate) build_graph(predicate);
    SPJ_CUDA(cudaEventRecord(ev0_, s_));
    SPJ_CUDA(cudaGraphLaunch(exec_, s_));
    SPJ_CUDA(cudaEventRecord(ev1_, s_));
    SPJ_CUDA(cudaStreamSynchronize(s_));
    if (h_total_[1] != ~0ull) {
      const uint32_t code = (uint32_t)(h_total_[1] >> 40);
      throw Error("stream: row " + std::to_string(h_total_[1] & 0xFFFFFFFFFFull) + ": " +
                  status_message(code));
    }
    total = h_total_[0];
    if (total <= capacity_) break;
    // output too small: grow, re-capture (the pointers changed), replay
    capacity_ = total + total / 8 + 1024;
    out_b_.alloc(capacity_ * 4, s_);
    out_p_.alloc(capacity_ * 4, s_);
    destroy_graph();
  }
  float ms = 0;
  SPJ_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
  stats_.ms_last = ms;
  stats_.rows += nrows_;
  stats_.pairs += total;
  stats_.replays++;
  stats_.escalations += h_total_[2];
  *d_build = out_b_.as<uint32_t>();
  *d_probe = out_p_.as<uint32_t>();
  return total;
}

void StreamJoin::set_params(const StreamParams& p) {
  SPJ_CHECK(p.block == 64 || p.block == 128 || p.block == 256, "block must be 64, 128 or 256");
  SPJ_CHECK(p.chunk_rows >= 32 && p.chunk_rows <= (1u << 20), "chunk_rows out of range");
  SPJ_CHECK(p.leaf_size >= 1 && p.leaf_size <= 64, "leaf_size out of range");
  const bool chunk_changed = p.chunk_rows != params_.chunk_rows;
  if (p.leaf_size != eng_.lbvh().leaf_size) eng_.reindex(p.leaf_size);
  params_ = p;
  destroy_graph();
  if (chunk_changed && !cols_.empty()) {
    std::vector<WkbDeviceColumn> c = cols_;
    set_batches(c);
  }
}

StreamParams StreamJoin::autotune(int predicate, const std::string& cache_path) {
  char dev_name[256] = {0};
  {
    int dev = 0;
    cudaDeviceProp prop;
    SPJ_CUDA(cudaGetDevice(&dev));
    SPJ_CUDA(cudaGetDeviceProperties(&prop, dev));
    snprintf(dev_name, sizeof dev_name, "%s", prop.name);
  }
  const std::string key = std::string(dev_name) + "|" + signature_ + "|" + std::to_string(predicate);
  if (!cache_path.empty()) {
    std::ifstream in(cache_path);
    std::string line;
    while (std::getline(in, line)) {
      // key<TAB>block chunk leaf
      const size_t tab = line.find('\t');
      if (tab == std::string::npos || line.substr(0, tab) != key) continue;
      std::istringstream vs(line.substr(tab + 1));
      StreamParams p;
      if (vs >> p.block >> p.chunk_rows >> p.leaf_size) {
        set_params(p);
        return p;
      }
    }
  }
  const StreamParams start = params_;
  StreamParams best = start;
  double best_ms = 1e30;
  const int blocks[] = {64, 128, 256};
  const uint32_t chunks[] = {256, 1024, 4096};
  const uint32_t leaves[] = {2, 4, 8};
  const uint32_t *db, *dp;
  for (uint32_t leaf : leaves) {
    for (int blk : blocks) {
      for (uint32_t ck : chunks) {
        set_params(StreamParams{blk, ck, leaf});
        run(predicate, &db, &dp);  // warm-up (and capture)
        run(predicate, &db, &dp);
        const double ms = stats_.ms_last;
        if (ms < best_ms) {
          best_ms = ms;
          best = params_;
        }
      }
    }
  }
  set_params(best);
  if (!cache_path.empty()) {
    std::ofstream out(cache_path, std::ios::app);
    out << key << "\t" << best.block << " " << best.chunk_rows << " " << best.leaf_size << "\n";
  }
  return best;
}

}  // namespace spj
