// lbvh.cuh — linear BVH over f32 boxes, and the probe traversal.
//
// Replaces the reference's OptiX BVH build and ray-cast filter
// (c/sedona-libgpuspatial/libgpuspatial/src/rt_spatial_index.cu:289-613,
//  src/rt/shaders/{point_query,box_query_forward,box_query_backward}.cu):
// GB300 has no RT cores, so the filter is a Karras-style LBVH traversed by
// SIMT threads.  Layout in HBM:
//   sorted_box[m]        f32x4 primitive boxes in Morton order
//   sorted_id[m]         u32  original build row of each sorted primitive
//   node_box[2*(L-1)]    f32x4 the two child boxes of internal node i at 2i, 2i+1
//   node_child[L-1]      i32x2 child index; >= 0 internal node, < 0 leaf ~c
// where L = ceil(m / leaf_size) leaves, leaf c covering sorted primitives
// [c*leaf_size, min((c+1)*leaf_size, m)).  A traversal step is one 32-byte
// pair of child boxes (two 128-bit loads) plus one 8-byte child pair.
#pragma once
#include "common.cuh"

namespace spj {

struct LbvhView {
  uint32_t nprims = 0;
  uint32_t nleaves = 0;
  uint32_t leaf_size = 1;
  const float4* sorted_box = nullptr;
  const uint32_t* sorted_id = nullptr;
  const float4* node_box = nullptr;
  const int2* node_child = nullptr;
};

struct Lbvh {
  uint32_t nprims = 0, nleaves = 0, leaf_size = 4;
  DevBuf sorted_box, sorted_id, node_box, node_child;
  LbvhView view() const {
    LbvhView v;
    v.nprims = nprims;
    v.nleaves = nleaves;
    v.leaf_size = leaf_size;
    v.sorted_box = sorted_box.as<float4>();
    v.sorted_id = sorted_id.as<uint32_t>();
    v.node_box = node_box.as<float4>();
    v.node_child = node_child.as<int2>();
    return v;
  }
  size_t device_bytes() const {
    return sorted_box.size() + sorted_id.size() + node_box.size() + node_child.size();
  }
};

// Builds the LBVH over boxes[0..n); NaN / inverted boxes are left out.
void build_lbvh(const float4* boxes, uint32_t n, uint32_t leaf_size, Lbvh& out, cudaStream_t s);

// Two-pass filter: every (build, probe) pair whose boxes intersect (closed
// intervals).  Pass 1 counts per probe; an exclusive scan gives each probe
// its output offset; pass 2 writes build ids and probe ids.  Probe boxes with
// NaN are empty.  probe_base is added to the probe ids written.
struct ProbeScratch {
  DevBuf counts, offsets, tmp;
};
// returns the number of candidate pairs (syncs the stream once)
uint64_t probe_count(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                     ProbeScratch& sc, cudaStream_t s);
void probe_scatter(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                   const ProbeScratch& sc, uint32_t probe_base, uint32_t* out_build,
                   uint32_t* out_probe, cudaStream_t s);

// The two traversal passes with caller-owned count / offset arrays (no
// allocation): counts[nprobe] written by the first, offs[nprobe] read by the
// second.
void probe_count_into(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                      uint32_t* counts, cudaStream_t s);
void probe_scatter_from(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                        const uint64_t* offs, uint32_t probe_base, uint32_t* out_build,
                        uint32_t* out_probe, cudaStream_t s, uint64_t capacity = ~0ull);

// Expand point/box probes by a distance (f64), then round outward to f32
// (rust/sedona-spatial-join/src/operand_evaluator.rs:605-607).
void expand_boxes(const double2* pts, const float4* boxes, const uint8_t* kind, uint32_t n,
                  double distance, float4* out, cudaStream_t s);

}  // namespace spj
