// stream.cuh — batched probe stream: many uneven Arrow record batches of
// point WKB probed in one CUDA-graph replay.
//
// The reference probes one DataFusion batch per FFI call
// (rust/sedona-spatial-join/src/stream.rs:1166-1200 -> query_batch), each call
// paying host round trips.  Here the batches of a stream are described in a
// device table and cut into fixed-size row chunks; a persistent kernel pulls
// chunks from a work queue (one atomic per chunk) and, per probe row, decodes
// the point from its WKB, walks the LBVH and refines each candidate inline.
// It runs twice — pass 0 counts each row's pairs, an exclusive scan turns the
// counts into offsets, pass 1 writes the pairs — so the output is grouped by
// probe row in ascending order and no candidate buffer exists.  Queue reset,
// both passes, the scan and the copy-out of the total are one CUDA graph.
#pragma once
#include <string>
#include <vector>

#include "engine.cuh"

namespace spj {

struct StreamParams {
  int block = 128;            // threads per CTA: 64, 128 or 256
  uint32_t chunk_rows = 1024;  // rows per work-queue item
  uint32_t leaf_size = 4;      // LBVH leaf size
  bool operator==(const StreamParams& o) const {
    return block == o.block && chunk_rows == o.chunk_rows && leaf_size == o.leaf_size;
  }
};

struct StreamStats {
  double ms_last = 0;         // device time of the last replay (CUDA events)
  uint64_t rows = 0, pairs = 0, replays = 0, escalations = 0, launches_per_replay = 0;
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
  // Times each candidate parameter set on the current batches and keeps the
  // fastest; results are cached in `cache_path` (JSON lines) when non-empty.
  StreamParams autotune(int predicate, const std::string& cache_path);
  cudaStream_t stream() const { return s_; }
  const StreamStats& stats() const { return stats_; }

 private:
  void build_graph(int predicate);
  void destroy_graph();
  JoinEngine& eng_;
  cudaStream_t s_ = nullptr;
  StreamParams params_;
  DevBuf batches_, chunks_, counts_, offs_, sums_, out_b_, out_p_, ctrl_;
  uint64_t* h_total_ = nullptr;  // pinned: total pairs + status word
  uint64_t capacity_ = 0;
  uint32_t nrows_ = 0, nchunks_ = 0, nbatches_ = 0;
  std::vector<WkbDeviceColumn> cols_;
  cudaGraphExec_t exec_ = nullptr;
  int graph_pred_ = -1;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  StreamStats stats_;
  std::string signature_;
};

}  // namespace spj
