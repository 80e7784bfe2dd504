// stream.cu — the batched probe stream (see stream.cuh), its CUDA graph and
// its autotuner.
#include <cstdio>
#include <fstream>
#include <sstream>

#include "prims.cuh"
#include "stream.cuh"
#include "wkb_read.cuh"

namespace spj {
namespace {

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

// Persistent decode: CTAs pull row chunks from the queue and decode each
// row's point (the decoder's point path: GPU-factory round-to-nearest box,
// POINT EMPTY and nulls give an empty row) into the stream-wide column.
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_stream_decode(const BatchDesc* __restrict__ batches, const ChunkDesc* __restrict__ chunks,
                    uint32_t nchunks, unsigned* queue, uint8_t* __restrict__ kind,
                    double2* __restrict__ pt, float4* __restrict__ box, DeviceStatus* st) {
  __shared__ uint32_t s_chunk;
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  const float fnan = __int_as_float(0x7fc00000);
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
      uint8_t k = kEmpty;
      double2 p = make_double2(qnan, qnan);
      float4 b = make_float4(fnan, fnan, fnan, fnan);
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
              k = kPoint;
              p = make_double2(x, y);
              const float fx = __double2float_rn(x), fy = __double2float_rn(y);
              b = make_float4(fx, fy, fx, fy);
            }
          }
        }
      }
      kind[g] = k;
      pt[g] = p;
      box[g] = b;
    }
  }
}

template <int kThreads>
int persistent_grid() {
  int dev = 0, sms = 0, per_sm = 0;
  SPJ_CUDA(cudaGetDevice(&dev));
  SPJ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  SPJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stream_decode<kThreads>,
                                                         kThreads, 0));
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace

StreamJoin::StreamJoin(JoinEngine& eng) : eng_(eng) {
  SPJ_CUDA(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
  SPJ_CUDA(cudaMallocHost(&h_tot_, 8 * sizeof(uint64_t)));
  g_allocations.fetch_add(1, std::memory_order_relaxed);
  SPJ_CUDA(cudaEventCreate(&ev0_));
  SPJ_CUDA(cudaEventCreate(&ev1_));
  ctrl_.alloc(16 + sizeof(DeviceStatus), s_);
  params_.leaf_size = eng_.lbvh().leaf_size;
}

StreamJoin::~StreamJoin() {
  destroy_graph();
  cudaStreamSynchronize(s_);
  for (DevBuf* b : {&batches_, &chunks_, &ctrl_, &kind_, &pt_, &box_, &counts_, &offs_, &sums_,
                    &cand_b_, &cand_p_, &flags_, &sums2_, &out_b_, &out_p_})
    b->release();
  psc_ = ProbeScratch();  // its buffers free on s_ too
  cudaStreamSynchronize(s_);
  cudaStreamDestroy(s_);
  cudaFreeHost(h_tot_);
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
  const size_t n1 = (size_t)nrows_ + 1;
  kind_.reserve(n1, s_);
  pt_.reserve(n1 * sizeof(double2), s_);
  box_.reserve(n1 * sizeof(float4), s_);
  counts_.reserve(n1 * 4, s_);
  offs_.reserve(n1 * 8, s_);
  sums_.reserve(scan_tile_sums_bytes(nrows_), s_);
  if (ccap_ == 0) {
    ccap_ = (uint64_t)nrows_ * 8 + 1024;
    ocap_ = (uint64_t)nrows_ * 4 + 1024;
  }
  SPJ_CUDA(cudaStreamSynchronize(s_));
  std::ostringstream sig;
  sig << eng_.build_geoms().n << "x" << eng_.build_geoms().nverts << "|" << nrows_ << "|"
      << nbatches_;
  signature_ = sig.str();
}

void StreamJoin::build_graph(int predicate) {
  destroy_graph();
  // capacity-sized buffers
  cand_b_.reserve((ccap_ + 1) * 4, s_);
  cand_p_.reserve((ccap_ + 1) * 4, s_);
  flags_.reserve(ccap_ + 1, s_);
  sums2_.reserve(compact_sums_bytes((int64_t)ccap_), s_);
  out_b_.reserve((ocap_ + 1) * 4, s_);
  out_p_.reserve((ocap_ + 1) * 4, s_);
  const EngineConfig cfg = eng_.config();
  // probes in Morton order (coherent traversals, and a refine that takes
  // neighbouring probes' candidates together); everything the ordering
  // uses is reserved here, so the capture allocates nothing
  const bool ordered = ccap_ < 0xFFFFFFFFull &&
                       (cfg.probe_order > 0 || (cfg.probe_order == 0 && nrows_ >= kOrderMinRows));
  if (ordered) {
    reserve_probe_order(nrows_, psc_, s_);
    reserve_candidate_order(nrows_, ccap_, psc_, s_);
  }
  SPJ_CUDA(cudaStreamSynchronize(s_));

  const GeomsView B = eng_.build_geoms().view();
  const LbvhView t = eng_.lbvh().view();
  GeomsView P;  // the stream-wide probe column: points only
  P.n = nrows_;
  P.kind = kind_.as<uint8_t>();
  P.pt = pt_.as<double2>();
  P.box = box_.as<float4>();
  unsigned* queue = ctrl_.as<unsigned>();
  DeviceStatus* st = reinterpret_cast<DeviceStatus*>(ctrl_.as<uint8_t>() + 16);
  const BatchDesc* bd = batches_.as<BatchDesc>();
  const ChunkDesc* cd = chunks_.as<ChunkDesc>();
  const int grid = params_.block == 128 ? persistent_grid<128>() : persistent_grid<256>();
  const uint64_t* d_m = offs_.as<uint64_t>() + nrows_;  // candidate count

  cudaGraph_t g = nullptr;
  SPJ_CUDA(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
  SPJ_CUDA(cudaMemsetAsync(ctrl_.get(), 0, 16 + sizeof(DeviceStatus), s_));
  SPJ_CUDA(cudaMemsetAsync(st, 0xFF, sizeof(unsigned long long), s_));
  if (params_.block == 128)
    k_stream_decode<128><<<grid, 128, 0, s_>>>(bd, cd, nchunks_, queue, kind_.as<uint8_t>(),
                                               pt_.as<double2>(), box_.as<float4>(), st);
  else
    k_stream_decode<256><<<grid, 256, 0, s_>>>(bd, cd, nchunks_, queue, kind_.as<uint8_t>(),
                                               pt_.as<double2>(), box_.as<float4>(), st);
  const uint32_t* order = ordered ? probe_order(t, box_.as<float4>(), nrows_, psc_, s_) : nullptr;
  probe_count_into(t, box_.as<float4>(), nrows_, counts_.as<uint32_t>(), s_, order);
  scan_u32_u64_into(counts_.as<uint32_t>(), offs_.as<uint64_t>(), nrows_, sums_.as<uint64_t>(),
                    s_);
  probe_scatter_from(t, box_.as<float4>(), nrows_, offs_.as<uint64_t>(), 0,
                     cand_b_.as<uint32_t>(), cand_p_.as<uint32_t>(), s_, ccap_, order);
  const uint32_t* cperm =
      order ? candidate_order_into(order, counts_.as<uint32_t>(), offs_.as<uint64_t>(), nrows_,
                                   ccap_, psc_, s_)
            : nullptr;
  // with a permutation the refine visits only the m candidates; the flags of
  // the rest of the capacity are cleared here for the flag scan
  if (cperm) SPJ_CUDA(cudaMemsetAsync(flags_.get(), 0, ccap_ + 1, s_));
  refine_relation(B, P, cand_b_.as<uint32_t>(), cand_p_.as<uint32_t>(), ccap_, 0, predicate,
                  cfg.refine_form, flags_.as<uint8_t>(), st, s_, d_m, cperm,
                  refine_blocks(cfg.refine_min_blocks, false));
  // compaction per 4096-flag tile (the flags past m are clear)
  compact_count(flags_.as<uint8_t>(), (int64_t)ccap_, sums2_.as<uint64_t>(), s_);
  compact_pairs_tiles(cand_b_.as<uint32_t>(), cand_p_.as<uint32_t>(), flags_.as<uint8_t>(),
                      (int64_t)ccap_, sums2_.as<uint64_t>(), out_b_.as<uint32_t>(),
                      out_p_.as<uint32_t>(), ocap_, s_);
  SPJ_CUDA(cudaMemcpyAsync(h_tot_, d_m, 8, cudaMemcpyDeviceToHost, s_));
  SPJ_CUDA(cudaMemcpyAsync(h_tot_ + 1, sums2_.as<uint64_t>() + compact_tiles((int64_t)ccap_), 8,
                           cudaMemcpyDeviceToHost, s_));
  SPJ_CUDA(cudaMemcpyAsync(h_tot_ + 2, &st->first_bad, 8, cudaMemcpyDeviceToHost, s_));
  SPJ_CUDA(cudaMemcpyAsync(h_tot_ + 3, &st->counters[0], 8, cudaMemcpyDeviceToHost, s_));
  SPJ_CUDA(cudaStreamEndCapture(s_, &g));
  cudaError_t e = cudaGraphInstantiate(&exec_, g, 0);
  cudaGraphDestroy(g);
  SPJ_CUDA(e);
  graph_pred_ = predicate;
  // memsets 2, decode 1, count 1, scan 3, scatter 1, refine 1, flag counts 2, compact 1;
  // ordered: keys 1 + 4 radix passes of 5, candidate order 5, flags memset 1
  stats_.launches_per_replay = 12 + (cperm ? 27 : (order ? 21 : 0));
}

uint64_t StreamJoin::run(int predicate, const uint32_t** d_build, const uint32_t** d_probe) {
  SPJ_CHECK(eng_.built(), "stream run before the build side was finished");
  SPJ_CHECK(predicate >= 0 && predicate <= 7, "the stream path takes relation predicates");
  uint64_t m = 0, total = 0;
  for (int attempt = 0; attempt < 4; attempt++) {
    if (!exec_ || graph_pred_ != predicate) build_graph(predicate);
    SPJ_CUDA(cudaEventRecord(ev0_, s_));
    SPJ_CUDA(cudaGraphLaunch(exec_, s_));
    SPJ_CUDA(cudaEventRecord(ev1_, s_));
    SPJ_CUDA(cudaStreamSynchronize(s_));
    check_traversal(eng_.lbvh().view(), s_);
    m = h_tot_[0];
    total = h_tot_[1];
    if (m > ccap_) {
      // candidates did not fit: grow, re-capture, replay (results discarded)
      ccap_ = m + m / 8 + 1024;
      destroy_graph();
      continue;
    }
    if (h_tot_[2] != ~0ull) {
      const uint32_t code = (uint32_t)(h_tot_[2] >> 40);
      throw Error("stream: row " + std::to_string(h_tot_[2] & 0xFFFFFFFFFFull) + ": " +
                  status_message(code));
    }
    if (total > ocap_) {
      ocap_ = total + total / 8 + 1024;
      destroy_graph();
      continue;
    }
    break;
  }
  SPJ_CHECK(m <= ccap_ && total <= ocap_, "stream: capacities did not settle");
  float ms = 0;
  SPJ_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
  stats_.ms_last = ms;
  stats_.rows += nrows_;
  stats_.pairs += total;
  stats_.candidates += m;
  stats_.replays++;
  stats_.escalations += h_tot_[3];
  *d_build = out_b_.as<uint32_t>();
  *d_probe = out_p_.as<uint32_t>();
  return total;
}

void StreamJoin::set_params(const StreamParams& p) {
  SPJ_CHECK(p.block == 128 || p.block == 256, "block must be 128 or 256");
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
  const std::string key =
      std::string(dev_name) + "|" + signature_ + "|" + std::to_string(predicate);
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
  // tune on a prefix of the batches (about 2M rows) to keep tuning short
  const std::vector<WkbDeviceColumn> all = cols_;
  std::vector<WkbDeviceColumn> prefix;
  int64_t rows = 0;
  for (const auto& c : all) {
    if (rows >= (2 << 20) && !prefix.empty()) break;
    prefix.push_back(c);
    rows += c.n;
  }
  set_batches(prefix);
  StreamParams best = params_;
  double best_ms = 1e30;
  const int blocks[] = {128, 256};
  const uint32_t chunks[] = {1024, 8192};
  const uint32_t leaves[] = {2, 4, 8};
  const uint32_t *db, *dp;
  for (uint32_t leaf : leaves) {
    for (int blk : blocks) {
      for (uint32_t ck : chunks) {
        set_params(StreamParams{blk, ck, leaf});
        run(predicate, &db, &dp);  // capture (and settle capacities)
        run(predicate, &db, &dp);
        if (stats_.ms_last < best_ms) {
          best_ms = stats_.ms_last;
          best = params_;
        }
      }
    }
  }
  set_params(best);
  set_batches(all);
  if (!cache_path.empty()) {
    std::ofstream out(cache_path, std::ios::app);
    out << key << "\t" << best.block << " " << best.chunk_rows << " " << best.leaf_size << "\n";
  }
  return best;
}

}  // namespace spj
