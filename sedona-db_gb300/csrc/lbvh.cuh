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
#include "geoms.cuh"

namespace spj {

struct LbvhView {
  uint32_t nprims = 0;
  uint32_t nleaves = 0;
  uint32_t leaf_size = 1;
  const float4* sorted_box = nullptr;
  const uint32_t* sorted_id = nullptr;
  const float4* node_box = nullptr;
  const int2* node_child = nullptr;
  const float4* leaf_box = nullptr;  // [L] union of each leaf's primitive boxes
  // [code, value]: the first out-of-range index a traversal met (code 0 = none)
  unsigned* fault = nullptr;
};

struct Lbvh {
  uint32_t nprims = 0, nleaves = 0, leaf_size = 4;
  DevBuf sorted_box, sorted_id, node_box, node_child, leaf_box, fault;
  LbvhView view() const {
    LbvhView v;
    v.nprims = nprims;
    v.nleaves = nleaves;
    v.leaf_size = leaf_size;
    v.sorted_box = sorted_box.as<float4>();
    v.sorted_id = sorted_id.as<uint32_t>();
    v.node_box = node_box.as<float4>();
    v.node_child = node_child.as<int2>();
    v.leaf_box = leaf_box.as<float4>();
    v.fault = fault.as<unsigned>();
    return v;
  }
  size_t device_bytes() const {
    return sorted_box.size() + sorted_id.size() + node_box.size() + node_child.size() +
           leaf_box.size();
  }
};

namespace {

constexpr int kTravThreads = 128;  // traversal block size
constexpr int kTravStack = 64;     // per-thread stack depth (Karras depth <= 32 key bits + 32)

enum TraversalFault : unsigned {
  kBadLeaf = 1,
  kBadNode = 2,
  kBadProbe = 3,
  kTooLong = 4,
  kStackOverflow = 5,
};

// Records the first out-of-range index a traversal met (the traversal of
// that probe stops; the host turns the record into an error).
__device__ __forceinline__ void traversal_fault(const LbvhView& t, unsigned code, unsigned v) {
  if (t.fault && atomicCAS(&t.fault[0], 0u, code) == 0u) t.fault[1] = v;
}

__device__ __forceinline__ bool box_overlap(float4 a, float4 b) {
  return !(a.x > b.z || a.z < b.x || a.y > b.w || a.w < b.y);
}

// Staging of one thread's output run (a traversal writes its results to
// consecutive slots).  Ids collect in shared memory, laid out [slot][thread]
// over kTravThreads threads, and go out when the next destination reaches a
// multiple of kRunBuf: after a first partial group every group fills one
// 32-byte sector, written as two 16-byte stores (when the buffer allows).
// A traversal's lanes otherwise store 4 bytes at a time to 32 places.
constexpr int kRunBuf = 8;

__device__ __forceinline__ void run_flush(uint32_t* __restrict__ out, uint64_t cap,
                                          const uint32_t* sm, uint64_t end, int n) {
  const uint64_t start = end - (uint64_t)n;
  const int tid = threadIdx.x;
  if (n == kRunBuf && (start & (kRunBuf - 1)) == 0 && end <= cap &&
      (reinterpret_cast<uintptr_t>(out) & 15) == 0) {
    uint4* o = reinterpret_cast<uint4*>(out + start);
    o[0] = make_uint4(sm[0 * kTravThreads + tid], sm[1 * kTravThreads + tid],
                      sm[2 * kTravThreads + tid], sm[3 * kTravThreads + tid]);
    o[1] = make_uint4(sm[4 * kTravThreads + tid], sm[5 * kTravThreads + tid],
                      sm[6 * kTravThreads + tid], sm[7 * kTravThreads + tid]);
  } else {
    for (int i = 0; i < n; i++)
      if (start + i < cap) out[start + i] = sm[i * kTravThreads + tid];
  }
}

// Appends id at out[pos] (pos advances); n ids are staged.
__device__ __forceinline__ void run_put(uint32_t* __restrict__ out, uint64_t cap, uint32_t* sm,
                                        uint64_t& pos, int& n, uint32_t id) {
  sm[n * kTravThreads + threadIdx.x] = id;
  n++;
  pos++;
  if ((pos & (kRunBuf - 1)) == 0 || n == kRunBuf) {
    run_flush(out, cap, sm, pos, n);
    n = 0;
  }
}

}  // namespace

// Builds the LBVH over boxes[0..n); NaN / inverted boxes are left out.
void build_lbvh(const float4* boxes, uint32_t n, uint32_t leaf_size, Lbvh& out, cudaStream_t s);

// Two-pass filter: every (build, probe) pair whose boxes intersect (closed
// intervals).  Pass 1 counts per probe; an exclusive scan gives each probe
// its output offset; pass 2 writes build ids and probe ids.  Probe boxes with
// NaN are empty.  probe_base is added to the probe ids written.
// `order` (optional, a permutation of the probe rows) sets the order in which
// traversal threads take probes; it changes neither the pairs nor where they
// are written.
struct ProbeScratch {
  DevBuf counts, offsets, tmp;
  DevBuf order, okeys, akeys, avals;  // probe_order
  DevBuf ocount, opos, cperm;         // candidate_order
  DevBuf ckeys, ckeys_alt, cvals_alt, rank;  // build_major_order
};
// Throws if a traversal over t recorded an out-of-range index (syncs s).
void check_traversal(const LbvhView& t, cudaStream_t s);
// returns the number of candidate pairs (syncs the stream once)
uint64_t probe_count(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                     ProbeScratch& sc, cudaStream_t s, const uint32_t* order = nullptr);
void probe_scatter(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                   const ProbeScratch& sc, uint32_t probe_base, uint32_t* out_build,
                   uint32_t* out_probe, cudaStream_t s, const uint32_t* order = nullptr);

// Reserves what probe_order needs for nprobe rows (so that a call inside a
// stream capture allocates nothing).
void reserve_probe_order(uint32_t nprobe, ProbeScratch& sc, cudaStream_t s);
// The probe rows sorted by the Morton key of their box centre over the tree's
// extent (sc.order); nullptr when there is nothing to order.
const uint32_t* probe_order(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                            ProbeScratch& sc, cudaStream_t s);
// out[e] = row + probe_base over each row's output run [offs[row], offs[row+1])
// (offs: n+1 entries), writes bounded by cap; coalesced.  The scatter passes
// write build ids and leave the probe ids to this kernel.
void fill_probe_ids(const uint64_t* offs, uint32_t n, uint32_t probe_base, uint32_t* out,
                    uint64_t cap, cudaStream_t s);

// After the two traversal passes (sc.counts / sc.offsets by probe row): the
// m candidate indices listed probe by probe in `order` (sc.cperm), so that a
// refine in that order takes spatially neighbouring probes together.  With
// keys (m entries), keys[j] = cb[cperm[j]] is written in the same pass.
const uint32_t* candidate_order(const uint32_t* order, uint32_t nprobe, uint64_t m,
                                ProbeScratch& sc, cudaStream_t s, const uint32_t* cb = nullptr,
                                uint32_t* keys = nullptr);
// The same from caller-owned per-row counts / offsets, for a candidate
// buffer of capacity mcap whose fill count lives on the device (graph
// replays): cperm[0, m) is the permutation of the m candidates, its entries
// past m are unspecified.  reserve_candidate_order first, outside a capture.
void reserve_candidate_order(uint32_t nprobe, uint64_t mcap, ProbeScratch& sc, cudaStream_t s);
const uint32_t* candidate_order_into(const uint32_t* order, const uint32_t* counts,
                                     const uint64_t* offs, uint32_t nprobe, uint64_t mcap,
                                     ProbeScratch& sc, cudaStream_t s);

// The m candidates (cb, cp) ordered by build row, then by the probe's Morton
// rank (order, when given) - a refine in that order takes one build
// geometry with neighbouring probes together (sc.cperm).  With an order the
// candidates are first listed in the probes' Morton order and that list is
// sorted stably by build row (full rank resolution, one radix pass per 8
// build-row bits); without one, by a 32-bit key of build row and row id.
// tiles > 1 (with an order): the Morton list is cut into that many tiles of
// about equal length (whole radix-sort tiles of 2048 items) and the
// build-row order holds within each tile, so the refine reads one tile's
// probe rows at a time.
const uint32_t* build_major_order(const uint32_t* cb, const uint32_t* cp, uint64_t m,
                                  uint32_t probe_base, uint32_t nbuild, const uint32_t* order,
                                  uint32_t nprobe, uint64_t tiles, ProbeScratch& sc,
                                  cudaStream_t s);

// Sorts caller-made candidate keys: sc.ckeys holds m keys and sc.cperm the
// candidate indices 0..m-1 (both reserved by reserve_candidate_keys); the
// stable sort by key_bits bits returns the permutation (sc.cperm).
void reserve_candidate_keys(uint64_t m, ProbeScratch& sc, cudaStream_t s);
const uint32_t* sort_candidate_keys(uint64_t m, int key_bits, ProbeScratch& sc, cudaStream_t s);

// The same for FP64 points (KNN queries).
const uint32_t* point_order(const LbvhView& t, const double2* xy, uint32_t n, ProbeScratch& sc,
                            cudaStream_t s);

// The two traversal passes with caller-owned count / offset arrays (no
// allocation): counts[nprobe] written by the first, offs[nprobe] read by the
// second.
void probe_count_into(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                      uint32_t* counts, cudaStream_t s, const uint32_t* order = nullptr);
void probe_scatter_from(const LbvhView& t, const float4* probe_box, uint32_t nprobe,
                        const uint64_t* offs, uint32_t probe_base, uint32_t* out_build,
                        uint32_t* out_probe, cudaStream_t s, uint64_t capacity = ~0ull,
                        const uint32_t* order = nullptr);

// Each row's exact bounds expanded by a distance (f64: one value, or d_row,
// one per row, on the device), then rounded outward to f32
// (rust/sedona-spatial-join/src/operand_evaluator.rs:556-627, 605-607); empty
// rows and negative or NaN distances give an empty (NaN) box.
void expand_boxes(const GeomsView& g, double distance, const double* d_row, float4* out,
                  cudaStream_t s);

}  // namespace spj
