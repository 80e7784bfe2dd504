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

// Stable LSD sort of (keys, vals) by key bits [0, key_bits).  keys/vals are
// replaced by the sorted sequences; alt_keys/alt_vals are scratch of size n.
// segments > 1: the sequence is cut into that many consecutive segments of
// whole 2048-item sort tiles (ceil(tiles / segments) tiles each, the last
// shorter) and each segment is sorted in place, with the same passes.
void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* alt_keys, uint32_t* alt_vals,
                      int64_t n, int key_bits, DevBuf& tmp, cudaStream_t s,
                      int64_t segments = 0);
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

}  // namespace spj
