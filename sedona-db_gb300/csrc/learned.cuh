// learned.cuh — learned point index: the build points sorted by a 32-bit
// Hilbert key on a 2^16 x 2^16 grid over their extent, and a two-stage
// piecewise-linear model of key -> rank: stage one picks one of L
// equal-count leaves through a radix table over key prefixes (a radix spline
// over the leaves' first keys), stage two is one line per leaf.  A lookup evaluates
// the model and binary-searches only within the leaf's measured maximum
// error; the result is verified against the neighbouring keys, so a lookup
// is exact whatever the model's quality.  The LBVH over the same points is
// the fallback (leaves whose error exceeds the window, boxes covering too
// many grid cells) and the arbiter of the pair set (the regular join path on
// the same inputs must give the same pairs).
//
// Training runs on the GPU: per leaf, a forward pass evaluates the residuals
// of the line on (key, rank) pairs and a backward pass accumulates the
// gradient of the squared loss and its Hessian (one CTA per leaf,
// deterministic block reductions in FP64); one Newton step solves the
// per-leaf least squares exactly (the loss is quadratic).
#pragma once
#include <vector>

#include "geoms.cuh"
#include "lbvh.cuh"

namespace spj {

struct LearnedStats {
  uint32_t leaves = 0;
  uint64_t points = 0;
  uint32_t root_shift = 0, root_entries = 0;  // stage-one radix table
  uint32_t max_err = 0;   // over leaves
  double mean_err = 0;    // mean per-leaf max error (non-empty leaves)
  uint32_t leaves_over_window = 0;
  double grad_norm_after = 0;  // max |gradient| over leaves after the Newton step
  uint64_t lookups = 0, window_misses = 0, lbvh_fallbacks = 0;
  uint64_t search_steps = 0;  // binary-search steps over all lookups
  uint64_t ranges = 0;        // build-point ranges handed to the candidate phase
  double ms_order = 0, ms_ranges = 0, ms_eval = 0;  // query phases (CUDA events)
  uint64_t kernel_launches = 0;  // this library's kernels launched by queries
};

struct LearnedView;

class LearnedIndex {
 public:
  LearnedIndex(uint32_t leaves, uint32_t window);
  ~LearnedIndex();
  // Build over a decoded point column (non-point rows are left out) whose
  // LBVH `bvh` is the fallback; both must outlive the index.
  void build(const DeviceGeoms& pts, const Lbvh& bvh, cudaStream_t s);
  // trained = false keeps the untrained start (per leaf, the line through
  // its first and last key), to measure what training gains.
  void train(bool trained, cudaStream_t s);
  // Per-leaf squared loss and gradient (d/da, d/db) at host parameters.
  void loss_and_grad(const std::vector<double>& a, const std::vector<double>& b,
                     std::vector<double>& loss, std::vector<double>& ga, std::vector<double>& gb,
                     cudaStream_t s);
  // Probe with a decoded column: point rows are exact lookups
  // (pred(build pt, probe pt) is point equality), polygon rows range
  // queries (ST_Intersects / Within / CoveredBy(build pt, probe polygon)).
  // Two passes (count / scan / emit); pairs grouped by probe row.
  uint64_t query(const GeomsView& probe, uint32_t probe_base, int predicate, DevBuf& out_build,
                 DevBuf& out_probe, cudaStream_t s);
  const LearnedStats& stats() const { return stats_; }
  // Largest per-leaf error the model serves; leaves above it (and rows
  // touching them) take the LBVH.  Only queries read it.
  void set_window(uint32_t window);
  // separate windows for point lookups and for the cells of range rows
  void set_windows(uint32_t window, uint32_t window_box);
  uint32_t window() const { return window_; }
  uint32_t window_box() const { return window_box_; }
  void export_model(std::vector<uint32_t>& keys, std::vector<uint32_t>& leaf_start,
                    std::vector<uint32_t>& leaf_kc, std::vector<double>& a,
                    std::vector<double>& b, std::vector<uint32_t>& err, cudaStream_t s);

 private:
  void fit_root(cudaStream_t s);
  void measure_errors(cudaStream_t s);
  uint32_t L_, window_, window_box_ = 0;
  uint32_t n_ = 0;
  float x0_ = 0, y0_ = 0, sx_ = 0, sy_ = 0;  // grid map on RN32 coordinates
  GeomsView bv_;
  LbvhView tv_;
  DevBuf keys_, ids_, xy_, xy32_;  // sorted by key
  DevBuf leaf_start_, leaf_a_, leaf_b_, leaf_ab32_, leaf_kc_, leaf_err_, counters_, counts_, offs_, tmp_,
      scratch_;
  DevBuf root_tab_;
  DevBuf order_, okeys_, akeys_, avals_, ranges_, ccount_, coff_;  // query scratch
  DevBuf rcache_, cwords_, woff_, masks_;
  std::vector<uint32_t> host_err_, host_start_;  // per-leaf errors, leaf starts
  cudaEvent_t ev_[4] = {};
  uint32_t root_shift_ = 0, root_p_ = 1;
  uint32_t k0_ = 0;
  LearnedStats stats_;
};

}  // namespace spj
