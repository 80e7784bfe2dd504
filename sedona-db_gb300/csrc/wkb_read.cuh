// wkb_read.cuh — device helpers that read little- or big-endian WKB fields
// at arbitrary byte offsets of an Arrow binary column's data buffer.
// Aligned 32-bit loads + funnel shifts when the buffer is 4-byte aligned and
// the words are in bounds; byte loads otherwise.
#pragma once
#include "geoms.cuh"

namespace spj {
namespace wkb {

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

// NW little-endian words covering bytes [o, o + 4*NW) of d (length len).
template <int NW>
__device__ __forceinline__ void load_words(const uint8_t* __restrict__ d, uint64_t o,
                                           uint64_t len, bool aligned_ok, uint32_t (&w)[NW]) {
  const uint64_t a = o & ~3ull;
  const uint32_t sh = (uint32_t)(o & 3u) * 8u;
  if (aligned_ok && a + 4 * (NW + 1) <= len) {
    const uint32_t* p = reinterpret_cast<const uint32_t*>(d + a);
    uint32_t r[NW + 1];
#pragma unroll
    for (int i = 0; i <= NW; i++) r[i] = __ldg(p + i);
#pragma unroll
    for (int i = 0; i < NW; i++) w[i] = __funnelshift_r(r[i], r[i + 1], sh);
  } else {
#pragma unroll
    for (int i = 0; i < NW; i++) {
      const uint8_t* b = d + o + 4 * i;
      w[i] = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) |
             ((uint32_t)b[3] << 24);
    }
  }
}

__device__ __forceinline__ uint32_t wkb_u32(uint32_t w, bool le) { return le ? w : bswap32(w); }

__device__ __forceinline__ double wkb_f64(uint32_t lo, uint32_t hi, bool le) {
  uint64_t bits = le ? (((uint64_t)hi << 32) | lo) : (((uint64_t)bswap32(lo) << 32) | bswap32(hi));
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ uint32_t read_u32(const uint8_t* d, uint64_t o, uint64_t len, bool al,
                                             bool le) {
  uint32_t w[1];
  load_words<1>(d, o, len, al, w);
  return wkb_u32(w[0], le);
}

template <bool kOff64>
__device__ __forceinline__ void row_range(const void* offsets, int64_t i, uint64_t& s, uint64_t& e) {
  if (kOff64) {
    const int64_t* o = reinterpret_cast<const int64_t*>(offsets);
    s = (uint64_t)o[i];
    e = (uint64_t)o[i + 1];
  } else {
    const int32_t* o = reinterpret_cast<const int32_t*>(offsets);
    s = (uint64_t)(uint32_t)o[i];
    e = (uint64_t)(uint32_t)o[i + 1];
  }
}

__device__ __forceinline__ bool row_valid(const uint8_t* validity, int64_t voff, int64_t i) {
  if (!validity) return true;
  int64_t b = voff + i;
  return (validity[b >> 3] >> (b & 7)) & 1;
}

}  // namespace wkb
}  // namespace spj
