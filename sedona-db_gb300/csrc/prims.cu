// prims.cu — device-wide scans and an 8-bit LSD radix sort.
//
// Scan: reduce-then-scan over 4096-element tiles (256 threads x 16 items);
// the tile sums are scanned by one 1024-thread block that walks them in
// chunks, then each tile is rescanned with its prefix.  Two reads of the
// input plus one write of the output: the scan is HBM-bound.
//
// Radix sort: per 8-bit digit, (1) a per-tile 256-bin histogram, (2) a scan of
// the digit-major histogram table, (3) a stable block-local ranking of the
// tile by digit (warp match + per-warp digit counters), a reorder in shared
// memory, then a scatter whose runs of equal digits land on consecutive
// addresses.  With segments, the table is segment-major, so the same passes
// sort each segment of consecutive tiles in place.
//
// Compaction of candidate pairs by 0/1 flags: per-tile counts and their
// scan, then each tile gathers its survivors in shared memory and writes
// them as one run (no per-element position array).
#include "prims.cuh"

namespace spj {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
static_assert(kScanTile == 4096, "compact_tiles (prims.cuh) counts tiles of 4096 flags");

template <class Tin, class Tout>
__global__ void k_tile_reduce(const Tin* __restrict__ in, int64_t n, Tout* __restrict__ sums) {
  __shared__ Tout sm[9];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  Tout acc = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    int64_t i = base + j * kScanThreads + threadIdx.x;
    if (i < n) acc += (Tout)in[i];
  }
  Tout total;
  block_exclusive_scan_256<Tout>(acc, sm, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <class T>
__global__ void k_scan_sums(T* __restrict__ sums, int64_t nt, T* __restrict__ total_out) {
  // one block of 1024 threads scans all tile sums in place (exclusive)
  __shared__ T warp_tot[32];
  __shared__ T carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t b = 0; b < nt; b += blockDim.x) {
    int64_t i = b + threadIdx.x;
    T v = i < nt ? sums[i] : T(0);
    T inc = warp_inclusive_scan(v);
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      T w = warp_tot[lane];
      T wi = warp_inclusive_scan(w);
      warp_tot[lane] = wi - w;
    }
    __syncthreads();
    T ex = carry + warp_tot[warp] + inc - v;
    if (i < nt) sums[i] = ex;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = ex + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total_out = carry;
}

template <class Tin, class Tout>
__global__ void k_tile_scan(const Tin* __restrict__ in, int64_t n, const Tout* __restrict__ sums,
                            Tout* __restrict__ out) {
  __shared__ Tout sm[9];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  // blocked arrangement: thread t owns items [t*16, t*16+16) of the tile
  Tout v[kScanItems];
  Tout acc = 0;
  const int64_t mybase = base + (int64_t)threadIdx.x * kScanItems;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    int64_t i = mybase + j;
    v[j] = i < n ? (Tout)in[i] : Tout(0);
    acc += v[j];
  }
  Tout ex = block_exclusive_scan_256<Tout>(acc, sm, nullptr) + sums[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    int64_t i = mybase + j;
    if (i < n) out[i] = ex;
    ex += v[j];
  }
}

// Stream compaction of candidate pairs by 0/1 flags, per 4096-flag tile:
// the tile's flags (16 per thread, one 16-byte load when aligned), a block
// scan of their counts, the survivors gathered in shared memory, then
// written as one coalesced run at the tile's offset (sums: exclusive tile
// offsets).  No per-element position array is written or read.
__global__ void __launch_bounds__(kScanThreads)
    k_compact_tile(const uint32_t* __restrict__ cb, const uint32_t* __restrict__ cp,
                   const uint8_t* __restrict__ flags, int64_t n,
                   const uint64_t* __restrict__ sums, uint32_t* __restrict__ ob,
                   uint32_t* __restrict__ op, uint64_t out_cap) {
  __shared__ uint32_t sb[kScanTile], sp[kScanTile];
  __shared__ uint32_t sm[9];
  const int64_t mybase = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t f = 0;  // bit j: flag of item mybase + j
  if (mybase + kScanItems <= n && (reinterpret_cast<uintptr_t>(flags + mybase) & 15) == 0) {
    const uint4 v = *reinterpret_cast<const uint4*>(flags + mybase);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < kScanItems; j++)
      f |= (uint32_t)(((w[j >> 2] >> (8 * (j & 3))) & 0xffu) != 0) << j;
  } else {
#pragma unroll
    for (int j = 0; j < kScanItems; j++)
      if (mybase + j < n && flags[mybase + j]) f |= 1u << j;
  }
  uint32_t total;
  uint32_t lo = block_exclusive_scan_256<uint32_t>((uint32_t)__popc(f), sm, &total);
#pragma unroll
  for (int j = 0; j < kScanItems; j++)
    if ((f >> j) & 1u) {
      sb[lo] = cb[mybase + j];
      sp[lo] = cp[mybase + j];
      lo++;
    }
  __syncthreads();
  const uint64_t tb = sums[blockIdx.x];
  for (uint32_t k = threadIdx.x; k < total; k += kScanThreads) {
    const uint64_t o = tb + k;
    if (o < out_cap) {  // bounded by the output capacity
      ob[o] = sb[k];
      op[o] = sp[k];
    }
  }
}

// Scan with caller-owned tile sums ((tiles + 1) entries of Tout).
template <class Tin, class Tout>
void scan_into_impl(const Tin* in, Tout* out, int64_t n, Tout* sums, cudaStream_t s) {
  if (n == 0) {
    SPJ_CUDA(cudaMemsetAsync(out, 0, sizeof(Tout), s));
    return;
  }
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  k_tile_reduce<Tin, Tout><<<(unsigned)nt, kScanThreads, 0, s>>>(in, n, sums);
  k_scan_sums<Tout><<<1, 1024, 0, s>>>(sums, nt, out + n);
  k_tile_scan<Tin, Tout><<<(unsigned)nt, kScanThreads, 0, s>>>(in, n, sums, out);
  SPJ_CUDA(cudaGetLastError());
}

template <class Tin, class Tout>
void scan_impl(const Tin* in, Tout* out, int64_t n, DevBuf& tmp, cudaStream_t s) {
  int64_t nt = (n + kScanTile - 1) / kScanTile;
  if (nt < 1) nt = 1;
  tmp.reserve((size_t)(nt + 1) * sizeof(Tout), s);
  Tout* sums = tmp.as<Tout>();
  if (n == 0) {
    SPJ_CUDA(cudaMemsetAsync(out, 0, sizeof(Tout), s));
    return;
  }
  k_tile_reduce<Tin, Tout><<<(unsigned)nt, kScanThreads, 0, s>>>(in, n, sums);
  k_scan_sums<Tout><<<1, 1024, 0, s>>>(sums, nt, out + n);
  k_tile_scan<Tin, Tout><<<(unsigned)nt, kScanThreads, 0, s>>>(in, n, sums, out);
  SPJ_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// radix sort

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

// Place of (digit d, tile b) in the histogram table.  The tiles form
// segments of seg_tiles consecutive tiles (the last may be shorter); the
// table is segment-major, then digit-major, so its scan gives every item a
// place inside its own segment's range and a pass sorts each segment alone.
// seg_tiles = ntiles: one segment, the plain digit-major table.
__device__ __forceinline__ int64_t hist_slot(uint32_t d, int64_t b, int64_t ntiles,
                                             int64_t seg_tiles) {
  const int64_t b0 = b / seg_tiles * seg_tiles;
  const int64_t nb = min(seg_tiles, ntiles - b0);
  return b0 * 256 + (int64_t)d * nb + (b - b0);
}

__global__ void k_digit_hist(const uint32_t* __restrict__ keys, int64_t n, int shift,
                             uint32_t* __restrict__ hist, int64_t ntiles, int64_t seg_tiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
#pragma unroll
  for (int j = 0; j < kSortItems; j++) {
    int64_t i = base + j * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xFF], 1u);
  }
  __syncthreads();
  hist[hist_slot(threadIdx.x, blockIdx.x, ntiles, seg_tiles)] = h[threadIdx.x];
}

// One 8-bit LSD pass over a tile of kSortTile items: stable local ranking by
// digit (warp w ranks its 256 items in 8 rounds of 32 with __match_any_sync
// and per-warp digit counters; a scan over warps and digits gives each item
// its place in the tile's digit-sorted order), a reorder in shared memory,
// and a write of each digit run to its global offset (scan of the tile
// histograms, hist_slot).  Pads (past n) carry key 0xFFFFFFFF, so they rank
// last in digit 255 and land past the tile's valid items, which are all
// written.
__global__ void __launch_bounds__(kSortThreads)
    k_digit_scatter(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                    int64_t n, int shift, const uint32_t* __restrict__ offs, int64_t ntiles,
                    int64_t seg_tiles, uint32_t* __restrict__ okeys,
                    uint32_t* __restrict__ ovals) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ uint32_t sk[kSortTile];
  __shared__ uint32_t sv[kSortTile];
  __shared__ uint32_t wcnt[kWarps][256];
  __shared__ uint32_t doff[256];
  __shared__ uint32_t gbase[256];
  __shared__ uint32_t scan_sm[9];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int t = threadIdx.x; t < kWarps * 256; t += kSortThreads) (&wcnt[0][0])[t] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  const int cnt = (int)min((int64_t)kSortTile, n - base);
  uint32_t k[kSortItems], v[kSortItems], pos[kSortItems];
#pragma unroll
  for (int j = 0; j < kSortItems; j++) {
    const int li = w * (32 * kSortItems) + j * 32 + lane;  // warp-contiguous chunk
    const bool valid = li < cnt;
    k[j] = valid ? keys[base + li] : 0xFFFFFFFFu;
    v[j] = valid ? vals[base + li] : 0u;
    const uint32_t d = (k[j] >> shift) & 0xFFu;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    uint32_t b = 0;
    if (lane == leader) {
      b = wcnt[w][d];
      wcnt[w][d] = b + (uint32_t)__popc(peers);
    }
    b = __shfl_sync(peers, b, leader);
    pos[j] = b + (uint32_t)__popc(peers & ((1u << lane) - 1u));
    __syncwarp();  // the counters' updates before the next round reads them
  }
  __syncthreads();
  {
    // thread t owns digit t: offsets of each warp's run inside the digit,
    // then the digit's offset inside the tile
    const int d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int ww = 0; ww < kWarps; ww++) {
      const uint32_t c = wcnt[ww][d];
      wcnt[ww][d] = run;
      run += c;
    }
    uint32_t total;
    doff[d] = block_exclusive_scan_256<uint32_t>(run, scan_sm, &total);
    gbase[d] = offs[hist_slot(d, blockIdx.x, ntiles, seg_tiles)];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kSortItems; j++) {
    const uint32_t d = (k[j] >> shift) & 0xFFu;
    const uint32_t lp = doff[d] + wcnt[w][d] + pos[j];
    sk[lp] = k[j];
    sv[lp] = v[j];
  }
  __syncthreads();
  for (int li = threadIdx.x; li < cnt; li += kSortThreads) {
    const uint32_t key = sk[li];
    const uint32_t d = (key >> shift) & 0xFFu;
    const uint64_t dst = (uint64_t)gbase[d] + (uint32_t)(li - doff[d]);
    if (okeys) okeys[dst] = key;  // (null: the last pass of a sort whose keys are not kept)
    ovals[dst] = sv[li];
  }
}

}  // namespace

void scan_u32_u64(const uint32_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s) {
  scan_impl<uint32_t, uint64_t>(in, out, n, tmp, s);
}
void scan_u8_u64(const uint8_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s) {
  scan_impl<uint8_t, uint64_t>(in, out, n, tmp, s);
}
size_t scan_tile_sums_bytes(int64_t n) {
  int64_t nt = (n + kScanTile - 1) / kScanTile;
  return (size_t)((nt < 1 ? 1 : nt) + 1) * sizeof(uint64_t);
}

void scan_u32_u64_into(const uint32_t* in, uint64_t* out, int64_t n, uint64_t* sums,
                       cudaStream_t s) {
  if (n == 0) {
    SPJ_CUDA(cudaMemsetAsync(out, 0, sizeof(uint64_t), s));
    return;
  }
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  k_tile_reduce<uint32_t, uint64_t><<<(unsigned)nt, kScanThreads, 0, s>>>(in, n, sums);
  k_scan_sums<uint64_t><<<1, 1024, 0, s>>>(sums, nt, out + n);
  k_tile_scan<uint32_t, uint64_t><<<(unsigned)nt, kScanThreads, 0, s>>>(in, n, sums, out);
  SPJ_CUDA(cudaGetLastError());
}

void scan_u32_u32(const uint32_t* in, uint32_t* out, int64_t n, DevBuf& tmp, cudaStream_t s) {
  scan_impl<uint32_t, uint32_t>(in, out, n, tmp, s);
}

size_t compact_sums_bytes(int64_t n) {
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  return (size_t)((nt < 1 ? 1 : nt) + 1) * sizeof(uint64_t);
}

void compact_count(const uint8_t* flags, int64_t n, uint64_t* sums, cudaStream_t s) {
  if (n <= 0) {
    SPJ_CUDA(cudaMemsetAsync(sums, 0, sizeof(uint64_t), s));
    return;
  }
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  k_tile_reduce<uint8_t, uint64_t><<<(unsigned)nt, kScanThreads, 0, s>>>(flags, n, sums);
  k_scan_sums<uint64_t><<<1, 1024, 0, s>>>(sums, nt, sums + nt);
  SPJ_CUDA(cudaGetLastError());
}

void compact_pairs_tiles(const uint32_t* cb, const uint32_t* cp, const uint8_t* flags, int64_t n,
                         const uint64_t* sums, uint32_t* ob, uint32_t* op, uint64_t out_cap,
                         cudaStream_t s) {
  if (n <= 0) return;
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  k_compact_tile<<<(unsigned)nt, kScanThreads, 0, s>>>(cb, cp, flags, n, sums, ob, op, out_cap);
  SPJ_CUDA(cudaGetLastError());
}

size_t radix_sort_tmp_bytes(int64_t n) {
  const int64_t ntiles = (n + kSortTile - 1) / kSortTile;
  const int64_t nh = 256 * (ntiles < 1 ? 1 : ntiles);
  const int64_t nt = (nh + kScanTile - 1) / kScanTile;
  return (size_t)(2 * nh + 1 + nt + 1) * sizeof(uint32_t);
}

void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* alt_keys, uint32_t* alt_vals,
                      int64_t n, int key_bits, DevBuf& tmp, cudaStream_t s, int64_t segments,
                      bool keys_out) {
  if (n <= 1) return;
  SPJ_CHECK(n < (int64_t)0xFFFFFFFF, "radix sort: too many keys");
  const int64_t ntiles = (n + kSortTile - 1) / kSortTile;
  const int64_t seg_tiles =
      segments > 1 ? (ntiles + segments - 1) / segments : ntiles;
  const int64_t nh = 256 * ntiles;
  // histogram table, its scan, and the scan's tile sums, all in tmp (no
  // allocation when tmp already holds radix_sort_tmp_bytes(n): graph capture)
  tmp.reserve(radix_sort_tmp_bytes(n), s);
  uint32_t* hist = tmp.as<uint32_t>();
  uint32_t* offs = hist + nh;
  uint32_t* sums = offs + nh + 1;
  uint32_t *ik = keys, *iv = vals, *ok = alt_keys, *ov = alt_vals;
  int passes = 0;
  for (int shift = 0; shift < key_bits; shift += 8) {
    const bool last = shift + 8 >= key_bits;
    k_digit_hist<<<(unsigned)ntiles, kSortThreads, 0, s>>>(ik, n, shift, hist, ntiles,
                                                           seg_tiles);
    scan_into_impl<uint32_t, uint32_t>(hist, offs, nh, sums, s);
    k_digit_scatter<<<(unsigned)ntiles, kSortThreads, 0, s>>>(
        ik, iv, n, shift, offs, ntiles, seg_tiles, last && !keys_out ? nullptr : ok, ov);
    SPJ_CUDA(cudaGetLastError());
    std::swap(ik, ok);
    std::swap(iv, ov);
    passes++;
  }
  if (passes & 1) {
    if (keys_out) SPJ_CUDA(cudaMemcpyAsync(keys, ik, n * 4, cudaMemcpyDeviceToDevice, s));
    SPJ_CUDA(cudaMemcpyAsync(vals, iv, n * 4, cudaMemcpyDeviceToDevice, s));
  }
}

const char* status_message(uint32_t code) {
  switch (code) {
    case kOk: return "ok";
    case kWkbTruncated: return "invalid WKB (truncated)";
    case kWkbByteOrder: return "invalid WKB (byte order)";
    case kWkbType: return "unsupported WKB geometry type";
    case kWkbDims: return "only 2D WKB geometries are supported";
    case kWkbCount: return "invalid WKB (count)";
    case kOverflow: return "output capacity exceeded";
    case kUnsupported: return "predicate not supported for these geometry types";
  }
  return "unknown device error";
}

}  // namespace spj
