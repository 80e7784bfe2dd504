// stream.cuh — batched probe stream: many uneven Arrow record batches of
// point WKB probed in one CUDA-graph replay.
//
// The reference probes one DataFusion batch per FFI call
// (rust/sedona-spatial-join/src/stream.rs:1166-1200 -> query_batch), each call
// paying host round trips.  Here the batches of a stream are described in a
// device table and cut into fixed-size row chunks.  One replay of a CUDA graph
// runs:
//   1. a persistent decode kernel pulling chunks from a work queue (one atomic
//      per chunk) and decoding every row's point into one stream-wide column;
//   2. from 65,536 rows, the rows' Morton order (keys + radix sort), then the
//      LBVH count pass, a scan, and the scatter pass over that column in that
//      order (candidate pairs, bounded by the candidate capacity), and the
//      candidates' permutation into the same order;
//   3. the refine kernel over the candidates in that order (the pair count is
//      read on the device), a scan of its flags, and the compaction (bounded
//      by the output capacity);
//   4. the copy-out of the two totals.
// The host checks the totals after the replay; when a capacity was too small
// it grows the buffers, re-captures and replays (the buffers then stay large
// enough for later replays of the same stream).  Pairs come out grouped by
// probe row in ascending order.
#pragma once
#include <string>
#include <vector>

#include "engine.cuh"

namespace spj {

struct StreamParams {
  int block = 256;             // threads per CTA of the decode kernel: 128 or 256
  uint32_t chunk_rows = 4096;  // rows per work-queue item
  uint32_t leaf_size = 4;      // LBVH leaf size
  bool operator==(const StreamParams& o) const {
    return block == o.block && chunk_rows == o.chunk_rows && leaf_size == o.leaf_size;
  }
};

struct StreamStats {
  double ms_last = 0;  // device time of the last replay (CUDA events)
  uint64_t rows = 0, pairs = 0, candidates = 0, replays = 0, escalations = 0;
  uint64_t launches_per_replay = 0;
};

class StreamJoin {
 public:
  explicit StreamJoin(JoinEngine& eng);
  ~StreamJoin();
  // Describe the batches (device columns, point WKB); row ids are global:
  // batch i's rows start after the rows of batches 0..i-1.
  void set_batches(const std::vector<WkbDeviceColumn>& cols);
  // One graph replay over every batch; returns the pair count.  Device
  // pointers to the pairs stay valid until the next run / set_batches.
  uint64_t run(int predicate, const uint32_t** d_build, const uint32_t** d_probe);
  void set_params(const StreamParams& p);
  const StreamParams& params() const { return params_; }
  // Times the candidate parameter sets on (a prefix of) the current batches
  // and keeps the fastest; results are cached in `cache_path` (one line per
  // device / workload signature / predicate) when it is non-empty.
  StreamParams autotune(int predicate, const std::string& cache_path);
  cudaStream_t stream() const { return s_; }
  const StreamStats& stats() const { return stats_; }

 private:
  void build_graph(int predicate);
  void destroy_graph();
  JoinEngine& eng_;
  cudaStream_t s_ = nullptr;
  StreamParams params_;
  DevBuf batches_, chunks_, ctrl_;
  DevBuf kind_, pt_, box_, counts_, offs_, sums_;  // stream-wide decoded column
  DevBuf cand_b_, cand_p_, flags_, sums2_, out_b_, out_p_;
  ProbeScratch psc_;  // the probes' Morton order and the candidates' permutation
  uint64_t* h_tot_ = nullptr;  // pinned: candidates, pairs, status, escalations
  uint64_t ccap_ = 0, ocap_ = 0;
  uint32_t nrows_ = 0, nchunks_ = 0, nbatches_ = 0;
  std::vector<WkbDeviceColumn> cols_;
  cudaGraphExec_t exec_ = nullptr;
  int graph_pred_ = -1;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  StreamStats stats_;
  std::string signature_;
};

}  // namespace spj
