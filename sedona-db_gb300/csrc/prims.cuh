// prims.cuh — device-wide scan and radix sort used by the decode, LBVH and
// two-pass count/scatter stages.  Written for sm_103a: 256-thread blocks,
// warp-shuffle block scans, 8-bit LSD radix passes with block-local stable
// ranking (warp match) and a reorder in shared memory.
#pragma once
#include "common.cuh"

namespace spj {

// out[0..n] = exclusive prefix sums of in[0..n), out[n] = total.
void scan_u32_u64(const uint32_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s);
void scan_u8_u64(const uint8_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s);
void scan_u32_u32(const uint32_t* in, uint32_t* out, int64_t n, DevBuf& tmp, cudaStream_t s);
// Same scan with caller-owned tile-sum scratch of scan_tile_sums_bytes(n) bytes.
size_t scan_tile_sums_bytes(int64_t n);
void scan_u32_u64_into(const uint32_t* in, uint64_t* out, int64_t n, uint64_t* tile_sums,
                       cudaStream_t s);

// Stream compaction of n candidate pairs (cb, cp) by 0/1 flags, in order,
// without a per-element position array.  compact_count writes the exclusive
// offsets of the 4096-flag tiles to sums (compact_sums_bytes(n) bytes) and the
// survivor count to sums[tiles]; compact_pairs_tiles then writes the
// survivors (at most out_cap of them) to ob / op.
size_t compact_sums_bytes(int64_t n);
void compact_count(const uint8_t* flags, int64_t n, uint64_t* sums, cudaStream_t s);
inline int64_t compact_tiles(int64_t n) { return n > 0 ? (n + 4095) / 4096 : 0; }
void compact_pairs_tiles(const uint32_t* cb, const uint32_t* cp, const uint8_t* flags, int64_t n,
                         const uint64_t* sums, uint32_t* ob, uint32_t* op, uint64_t out_cap,
                         cudaStream_t s);

// Stable LSD sort of (keys, vals) by key bits [0, key_bits).  keys/vals are
// replaced by the sorted sequences; alt_keys/alt_vals are scratch of size n.
// segments > 1: the sequence is cut into that many consecutive segments of
// whole 2048-item sort tiles (ceil(tiles / segments) tiles each, the last
// shorter) and each segment is sorted in place, with the same passes.
// keys_out false: only vals are sorted on return (the last pass writes no
// keys, and keys is left undefined).
void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* alt_keys, uint32_t* alt_vals,
                      int64_t n, int key_bits, DevBuf& tmp, cudaStream_t s,
                      int64_t segments = 0, bool keys_out = true);
// Bytes of tmp that radix_sort_pairs uses for n keys (reserve them before a
// stream capture so that the sort allocates nothing inside it).
size_t radix_sort_tmp_bytes(int64_t n);

// Warp/block helpers usable from other kernels.
template <class T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T o = __shfl_up_sync(0xffffffffu, v, d);
    if ((threadIdx.x & 31) >= d) v += o;
  }
  return v;
}

// Block-wide exclusive scan for blockDim.x == 256; smem must hold 8 T.
template <class T>
__device__ __forceinline__ T block_exclusive_scan_256(T v, T* smem, T* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T inc = warp_inclusive_scan(v);
  if (lane == 31) smem[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = lane < 8 ? smem[lane] : T(0);
    T wi = warp_inclusive_scan(w);
    if (lane < 8) smem[lane] = wi - w;
    if (lane == 7) smem[8] = wi;
  }
  __syncthreads();
  T r = smem[warp] + inc - v;
  if (total) *total = smem[8];
  __syncthreads();
  return r;
}

// Copies l bytes from src to dst with the G lanes (G >= 4) of a lane group,
// gl = the lane's place in the group.  The destination is written as whole
// 4-byte words between a head and a tail of under 4 bytes each; each word is
// assembled from the two aligned source words it straddles (a funnel shift),
// whatever the two alignments.  A lane issues up to 8 word loads before its
// stores, so a value of up to G * 32 bytes costs one memory latency.  (An
// aligned source word that holds a byte of the value lies in the value's
// allocation.)
template <int G>
__device__ __forceinline__ void group_copy(const uint8_t* __restrict__ src,
                                           uint8_t* __restrict__ dst, uint64_t l, int gl) {
  static_assert(G >= 4, "head and tail bytes take one lane each");
  const uintptr_t da = reinterpret_cast<uintptr_t>(dst);
  const uint64_t head = min(l, (uint64_t)((4 - (da & 3)) & 3));
  if ((uint64_t)gl < head) dst[gl] = src[gl];
  const uint64_t words = (l - head) >> 2;
  const uintptr_t sa = reinterpret_cast<uintptr_t>(src + head);
  const uint32_t sh = (uint32_t)(sa & 3) * 8;
  const uint32_t* sw = reinterpret_cast<const uint32_t*>(sa & ~uintptr_t(3));
  uint32_t* dw = reinterpret_cast<uint32_t*>(dst + head);
  constexpr int kU = 8;
  for (uint64_t w0 = 0; w0 < words; w0 += (uint64_t)G * kU) {
    uint32_t lo[kU], hi[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const uint64_t w = w0 + (uint64_t)(u * G + gl);
      lo[u] = w < words ? sw[w] : 0u;
      hi[u] = w < words && sh ? sw[w + 1] : 0u;
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const uint64_t w = w0 + (uint64_t)(u * G + gl);
      if (w < words) dw[w] = __funnelshift_r(lo[u], hi[u], sh);
    }
  }
  const uint64_t t0 = head + words * 4;
  if (t0 + gl < l) dst[t0 + gl] = src[t0 + gl];
}

}  // namespace spj
