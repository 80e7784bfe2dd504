// knn.cuh — KNN join over point columns: for each probe point the k build
// points with the smallest Euclidean distance, ties broken by build row id
// (the ground truth of rust/sedona-spatial-join/tests/spatial_join_integration.rs:1373-1414,
// the CPU query_knn of rust/sedona-spatial-join/src/index/default_spatial_index.rs:306-502).
#pragma once
#include "lbvh.cuh"

namespace spj {

class KnnIndex {
 public:
  KnnIndex(uint32_t leaf_size, int form);
  ~KnnIndex();
  void build(const double* xy_host, uint64_t n);
  // probe_xy: n (x, y) FP64 pairs; outputs n*k entries; host or device arrays
  void query(const double* probe_xy, uint64_t n, uint32_t k, uint32_t* out_idx, double* out_dist,
             bool device_ptrs);
  // Variable-length results: each probe's valid results (none for an empty
  // probe) and, with ties, the build points outside them whose distance is
  // within 1e-9 of the k-th (include_tie_breakers; the reference's
  // DISTANCE_TOLERANCE).  offsets (host, n+1) receive each probe's run in
  // out_idx / out_dist (host); returns the total; when it exceeds capacity
  // nothing else is written.
  uint64_t query_ties(const double* probe_xy, uint64_t n, uint32_t k, bool device_ptrs,
                      uint64_t* offsets, uint32_t* out_idx, double* out_dist, uint64_t capacity,
                      bool ties);
  cudaStream_t stream() const { return stream_; }
  uint64_t exact_evals() const { return exact_evals_; }
  // probes whose k-set the split FP32 pass did not prove (sent to the exact kernel)
  uint64_t redone() const { return redone_; }
  uint64_t queries() const { return queries_; }

 private:
  uint32_t leaf_size_;
  int form_;
  cudaStream_t stream_ = nullptr;
  uint64_t n_ = 0;
  Lbvh bvh_;
  DevBuf xy_sorted_;  // build points in LBVH order
  DevBuf xy_split_;   // the same as FP32 (hi.x, hi.y, lo.x, lo.y)
  float slack_ = 0;   // bound on |p - RN32(p)| over the build side
  float bmag_ = 0;    // max |x| + |y| over the build side (rounded up)
  bool split_ok_ = true;  // build coordinates within the split pass's range
  DevBuf probe_, oidx_, odist_, counters_, redo_;
  DevBuf tie_probe_, tie_kidx_, tie_kdist_, tie_counts_, tie_offs_, tie_tmp_, tie_out_idx_,
      tie_out_dist_;
  ProbeScratch osc_;  // Morton order of the probes
  uint64_t exact_evals_ = 0, redone_ = 0, queries_ = 0;
};

}  // namespace spj
