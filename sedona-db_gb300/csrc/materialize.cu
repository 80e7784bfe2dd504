// materialize.cu — result materialisation on the device: the column gathers
// that build the joined batch from the refined pairs (the reference's
// build_batch_from_indices / assemble_partial_build_batch on the host,
// rust/sedona-spatial-join/src/stream.rs:1466-1580, an Arrow take per
// column), and the build side's visited bitmap of outer, semi and anti joins
// (rust/sedona-spatial-join/src/utils/join_utils.rs:53-62,
// SpatialIndex::visited_build_side).  Indices equal to SPJ_NULL_INDEX
// produce a null row (the unmatched side of an outer join).
//
// All HBM-bound: a gathered fixed-width value reads its width once and writes
// it once (the index 4 B); a binary value reads and writes its bytes once,
// with a length pass, a scan and a copy pass (8 lanes per value, the
// destination written as whole 4-byte words whatever the alignments).
#include <errno.h>

#include <string>

#include "../../include/spj_gb300.h"
#include "common.cuh"
#include "materialize.cuh"
#include "prims.cuh"

namespace spj {
namespace {

thread_local std::string g_error;

int fail(const std::exception& e) {
  g_error = e.what();
  return EINVAL;
}

template <class T>
__global__ void k_gather_fixed(const T* __restrict__ src, const uint32_t* __restrict__ idx,
                               uint64_t n, uint64_t nsrc, T* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t j = idx[i];
    T v{};
    if (j != SPJ_NULL_INDEX && j < nsrc) v = src[j];
    out[i] = v;
  }
}

// validity bits of the gathered rows: 32 rows per thread, one word out
__global__ void k_gather_valid(const uint8_t* __restrict__ valid, int64_t voff,
                               const uint32_t* __restrict__ idx, uint64_t n, uint64_t nsrc,
                               uint32_t* __restrict__ out, unsigned long long* __restrict__ nulls) {
  uint32_t cnt = 0;
  const uint64_t nw = (n + 31) / 32;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw;
       w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t bits = 0;
    for (int b = 0; b < 32; b++) {
      const uint64_t i = w * 32 + b;
      if (i >= n) break;
      const uint32_t j = idx[i];
      bool ok = j != SPJ_NULL_INDEX && j < nsrc;
      if (ok && valid) {
        const uint64_t bit = (uint64_t)voff + j;
        ok = (valid[bit >> 3] >> (bit & 7)) & 1;
      }
      if (ok) bits |= 1u << b;
      else cnt++;
    }
    out[w] = bits;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(nulls, (unsigned long long)cnt);
}

template <bool kOff64>
__device__ __forceinline__ void bin_range(const void* off, uint32_t j, uint64_t& s, uint64_t& e) {
  if (kOff64) {
    const int64_t* o = static_cast<const int64_t*>(off);
    s = (uint64_t)o[j];
    e = (uint64_t)o[j + 1];
  } else {
    const int32_t* o = static_cast<const int32_t*>(off);
    s = (uint64_t)(uint32_t)o[j];
    e = (uint64_t)(uint32_t)o[j + 1];
  }
}

template <bool kOff64>
__global__ void k_bin_lengths(const void* __restrict__ off, const uint32_t* __restrict__ idx,
                              uint64_t n, uint64_t nsrc, uint32_t* __restrict__ len) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t j = idx[i];
    uint32_t l = 0;
    if (j != SPJ_NULL_INDEX && j < nsrc) {
      uint64_t s, e;
      bin_range<kOff64>(off, j, s, e);
      l = e > s ? (uint32_t)(e - s) : 0;
    }
    len[i] = l;
  }
}

// A warp takes 32 values: lane k reads value k's index, source range and
// output position (one memory latency for all 32), then lane groups of 8
// copy 4 values at a time (group_copy: whole destination words, any
// alignment).
template <bool kOff64>
__global__ void k_bin_copy(const void* __restrict__ off, const uint8_t* __restrict__ data,
                           const uint32_t* __restrict__ idx, uint64_t n, uint64_t nsrc,
                           const uint64_t* __restrict__ pos, uint8_t* __restrict__ out,
                           uint64_t cap) {
  constexpr int G = 8;
  const int lane = threadIdx.x & 31, grp = lane / G, gl = lane % G;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t i0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; i0 < n;
       i0 += nwarps * 32) {
    const uint64_t i = i0 + lane;
    uint64_t s = 0, d = 0, l = 0;
    if (i < n) {
      const uint32_t j = idx[i];
      if (j != SPJ_NULL_INDEX && j < nsrc) {
        uint64_t e;
        bin_range<kOff64>(off, j, s, e);
        d = pos[i];
        l = e > s ? e - s : 0;
        if (d + l > cap) l = 0;  // bounded by the output buffer
      }
    }
    for (int v = 0; v < 32; v += 32 / G) {
      const uint64_t vs = __shfl_sync(0xffffffffu, s, v + grp);
      const uint64_t vd = __shfl_sync(0xffffffffu, d, v + grp);
      const uint64_t vl = __shfl_sync(0xffffffffu, l, v + grp);
      if (vl) group_copy<G>(data + vs, out + vd, vl, gl);
    }
  }
}

__global__ void k_u64_to_i64_offsets(const uint64_t* __restrict__ pos, uint64_t n,
                                     int64_t* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (int64_t)pos[i];
}

__global__ void k_mark(uint32_t* __restrict__ bits, uint64_t nbuild,
                       const uint32_t* __restrict__ ids, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t b = ids[i];
    if (b >= nbuild) continue;
    const uint32_t w = b >> 5, m = 1u << (b & 31);
    if (!(bits[w] & m)) atomicOr(&bits[w], m);  // read first: most marks repeat
  }
}

// rows whose bit equals want, in ascending order: per 32-row word a count,
// a scan, then the rows
__global__ void k_bits_count(const uint32_t* __restrict__ bits, uint64_t nbuild, uint32_t want,
                             uint32_t* __restrict__ cnt) {
  const uint64_t nw = (nbuild + 31) / 32;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw;
       w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t v = want ? bits[w] : ~bits[w];
    const uint64_t rem = nbuild - w * 32;
    if (rem < 32) v &= (1u << rem) - 1u;
    cnt[w] = __popc(v);
  }
}

__global__ void k_bits_rows(const uint32_t* __restrict__ bits, uint64_t nbuild, uint32_t want,
                            const uint64_t* __restrict__ pos, uint32_t* __restrict__ out,
                            uint64_t cap) {
  const uint64_t nw = (nbuild + 31) / 32;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw;
       w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t v = want ? bits[w] : ~bits[w];
    const uint64_t rem = nbuild - w * 32;
    if (rem < 32) v &= (1u << rem) - 1u;
    uint64_t p = pos[w];
    while (v) {
      const int b = __ffs(v) - 1;
      v &= v - 1;
      if (p < cap) out[p] = (uint32_t)(w * 32 + b);
      p++;
    }
  }
}

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

bool aligned(const void* p, size_t a) { return reinterpret_cast<uintptr_t>(p) % a == 0; }

}  // namespace

uint64_t gather_binary(const WkbDeviceColumn& col, const uint32_t* d_idx, uint64_t n,
                       DevBuf& out_off, DevBuf& out_data, DevBuf& scratch_len,
                       DevBuf& scratch_pos, DevBuf& scan_tmp, cudaStream_t s) {
  scratch_len.reserve(((size_t)n + 1) * 4, s);
  scratch_pos.reserve(((size_t)n + 1) * 8, s);
  out_off.reserve(((size_t)n + 1) * 8, s);
  const int g = grid_for((int64_t)n, 256, kNumSMs * 16);
  if (n) {
    if (col.offsets64)
      k_bin_lengths<true><<<g, 256, 0, s>>>(col.offsets, d_idx, n, (uint64_t)col.n,
                                            scratch_len.as<uint32_t>());
    else
      k_bin_lengths<false><<<g, 256, 0, s>>>(col.offsets, d_idx, n, (uint64_t)col.n,
                                             scratch_len.as<uint32_t>());
  }
  scan_u32_u64(scratch_len.as<uint32_t>(), scratch_pos.as<uint64_t>(), (int64_t)n, scan_tmp, s);
  uint64_t total = 0;
  SPJ_CUDA(cudaMemcpyAsync(&total, scratch_pos.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  k_u64_to_i64_offsets<<<grid_for((int64_t)n + 1, 256), 256, 0, s>>>(
      scratch_pos.as<uint64_t>(), n, out_off.as<int64_t>());
  out_data.reserve(total + 16, s);
  if (n && total) {
    const int gw = grid_for((int64_t)n * 32, 256, kNumSMs * 32);
    if (col.offsets64)
      k_bin_copy<true><<<gw, 256, 0, s>>>(col.offsets, col.data, d_idx, n, (uint64_t)col.n,
                                          scratch_pos.as<uint64_t>(), out_data.as<uint8_t>(),
                                          total);
    else
      k_bin_copy<false><<<gw, 256, 0, s>>>(col.offsets, col.data, d_idx, n, (uint64_t)col.n,
                                           scratch_pos.as<uint64_t>(), out_data.as<uint8_t>(),
                                           total);
  }
  SPJ_CUDA(cudaGetLastError());
  SPJ_CUDA(cudaStreamSynchronize(s));
  return total;
}

void gather_u64(const uint64_t* values, uint64_t n_values, const uint32_t* d_idx, uint64_t n,
                uint64_t* out, cudaStream_t s) {
  if (!n) return;
  k_gather_fixed<uint64_t><<<grid_for((int64_t)n, 256, kNumSMs * 16), 256, 0, s>>>(
      values, d_idx, n, n_values, out);
  SPJ_CUDA(cudaGetLastError());
}

}  // namespace spj

using namespace spj;

extern "C" const char* SpjMaterializeLastError(void) { return g_error.c_str(); }

extern "C" int SpjGatherFixed(const void* d_values, uint32_t width, uint64_t n_values,
                              const uint32_t* d_idx, uint64_t n, void* d_out, void* stream) {
  try {
    SPJ_CHECK(n == 0 || (d_idx && d_out && (d_values || n_values == 0)), "null buffer");
    SPJ_CHECK(width == 1 || width == 2 || width == 4 || width == 8 || width == 16,
              "width must be 1, 2, 4, 8 or 16 bytes");
    SPJ_CHECK(aligned(d_values, width) && aligned(d_out, width) && aligned(d_idx, 4),
              "values and output must be aligned to the width, indices to 4 bytes");
    const cudaStream_t s = as_stream(stream);
    if (n_values == 0) d_values = nullptr;
    if (n) {
      const int g = grid_for((int64_t)n, 256, kNumSMs * 16);
#define SPJ_GF(T)                                                                          \
  k_gather_fixed<T><<<g, 256, 0, s>>>(static_cast<const T*>(d_values), d_idx, n, n_values, \
                                       static_cast<T*>(d_out))
      switch (width) {
        case 1: SPJ_GF(uint8_t); break;
        case 2: SPJ_GF(uint16_t); break;
        case 4: SPJ_GF(uint32_t); break;
        case 8: SPJ_GF(uint64_t); break;
        case 16: SPJ_GF(uint4); break;
        default: throw Error("width must be 1, 2, 4, 8 or 16 bytes");
      }
#undef SPJ_GF
      SPJ_CUDA(cudaGetLastError());
    }
    SPJ_CUDA(cudaStreamSynchronize(s));
    g_error.clear();
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

extern "C" int SpjGatherValidity(const uint8_t* d_validity, int64_t validity_offset,
                                 uint64_t n_values, const uint32_t* d_idx, uint64_t n,
                                 uint8_t* d_out_bitmap, uint64_t* null_count, void* stream) {
  try {
    SPJ_CHECK(null_count != nullptr, "null null_count");
    SPJ_CHECK(n == 0 || (d_idx && d_out_bitmap), "null buffer");
    SPJ_CHECK(aligned(d_out_bitmap, 4) && aligned(d_idx, 4),
              "the output bitmap (written as 32-bit words) and the indices must be 4-byte "
              "aligned");
    const cudaStream_t s = as_stream(stream);
    DevBuf cnt(8, s);
    SPJ_CUDA(cudaMemsetAsync(cnt.get(), 0, 8, s));
    if (n) {
      const uint64_t nw = (n + 31) / 32;
      k_gather_valid<<<grid_for((int64_t)nw, 256, kNumSMs * 16), 256, 0, s>>>(
          d_validity, validity_offset, d_idx, n, n_values,
          reinterpret_cast<uint32_t*>(d_out_bitmap), cnt.as<unsigned long long>());
      SPJ_CUDA(cudaGetLastError());
    }
    unsigned long long h = 0;
    SPJ_CUDA(cudaMemcpyAsync(&h, cnt.get(), 8, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    *null_count = h;
    g_error.clear();
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

extern "C" int SpjGatherBinary(const void* d_offsets, int32_t offsets_are_64bit,
                               const uint8_t* d_data, uint64_t n_values, const uint32_t* d_idx,
                               uint64_t n, int64_t* d_out_offsets, uint8_t* d_out_data,
                               uint64_t capacity, uint64_t* out_bytes, void* stream) {
  try {
    SPJ_CHECK(out_bytes != nullptr, "null out_bytes");
    SPJ_CHECK(d_out_offsets != nullptr && d_offsets != nullptr && (n == 0 || d_idx),
              "null buffer");
    SPJ_CHECK(aligned(d_offsets, offsets_are_64bit ? 8 : 4) && aligned(d_out_offsets, 8) &&
                  aligned(d_idx, 4),
              "offsets and indices must be aligned to their element size");
    const cudaStream_t s = as_stream(stream);
    DevBuf len(((size_t)n + 1) * 4, s), pos(((size_t)n + 1) * 8, s), tmp;
    const int g = grid_for((int64_t)n, 256, kNumSMs * 16);
    if (n) {
      if (offsets_are_64bit)
        k_bin_lengths<true><<<g, 256, 0, s>>>(d_offsets, d_idx, n, n_values, len.as<uint32_t>());
      else
        k_bin_lengths<false><<<g, 256, 0, s>>>(d_offsets, d_idx, n, n_values, len.as<uint32_t>());
    }
    scan_u32_u64(len.as<uint32_t>(), pos.as<uint64_t>(), (int64_t)n, tmp, s);
    uint64_t total = 0;
    SPJ_CUDA(cudaMemcpyAsync(&total, pos.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    *out_bytes = total;
    k_u64_to_i64_offsets<<<grid_for((int64_t)n + 1, 256), 256, 0, s>>>(pos.as<uint64_t>(), n,
                                                                       d_out_offsets);
    if (total > capacity) {
      SPJ_CUDA(cudaStreamSynchronize(s));
      g_error = "output capacity " + std::to_string(capacity) + " < " + std::to_string(total) +
                " bytes";
      return ENOSPC;
    }
    if (n && total) {
      SPJ_CHECK(d_out_data != nullptr && d_data != nullptr, "null data buffer");
      const int gw = grid_for((int64_t)n * 32, 256, kNumSMs * 32);
      if (offsets_are_64bit)
        k_bin_copy<true><<<gw, 256, 0, s>>>(d_offsets, d_data, d_idx, n, n_values,
                                            pos.as<uint64_t>(), d_out_data, capacity);
      else
        k_bin_copy<false><<<gw, 256, 0, s>>>(d_offsets, d_data, d_idx, n, n_values,
                                             pos.as<uint64_t>(), d_out_data, capacity);
    }
    SPJ_CUDA(cudaGetLastError());
    SPJ_CUDA(cudaStreamSynchronize(s));
    g_error.clear();
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

extern "C" int SpjVisitedMark(uint32_t* d_bitmap, uint64_t n_build, const uint32_t* d_build_idx,
                              uint64_t n, void* stream) {
  try {
    SPJ_CHECK(n == 0 || n_build == 0 || (d_bitmap && d_build_idx), "null buffer");
    SPJ_CHECK(aligned(d_bitmap, 4) && aligned(d_build_idx, 4), "buffers must be 4-byte aligned");
    const cudaStream_t s = as_stream(stream);
    if (n && n_build)
      k_mark<<<grid_for((int64_t)n, 256, kNumSMs * 16), 256, 0, s>>>(d_bitmap, n_build,
                                                                      d_build_idx, n);
    SPJ_CUDA(cudaGetLastError());
    SPJ_CUDA(cudaStreamSynchronize(s));
    g_error.clear();
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

extern "C" int SpjVisitedCollect(const uint32_t* d_bitmap, uint64_t n_build, int32_t visited,
                                 uint32_t* d_out_idx, uint64_t capacity, uint64_t* count,
                                 void* stream) {
  try {
    SPJ_CHECK(count != nullptr, "null count");
    SPJ_CHECK(aligned(d_bitmap, 4) && aligned(d_out_idx, 4), "buffers must be 4-byte aligned");
    const cudaStream_t s = as_stream(stream);
    const uint64_t nw = (n_build + 31) / 32;
    DevBuf cnt((nw + 1) * 4, s), pos((nw + 1) * 8, s), tmp;
    const int g = grid_for((int64_t)nw, 256, kNumSMs * 16);
    if (nw) {
      SPJ_CHECK(d_bitmap != nullptr, "null bitmap");
      k_bits_count<<<g, 256, 0, s>>>(d_bitmap, n_build, visited ? 1u : 0u, cnt.as<uint32_t>());
    }
    scan_u32_u64(cnt.as<uint32_t>(), pos.as<uint64_t>(), (int64_t)nw, tmp, s);
    uint64_t total = 0;
    SPJ_CUDA(cudaMemcpyAsync(&total, pos.as<uint64_t>() + nw, 8, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    *count = total;
    if (total > capacity) {
      g_error = "output capacity " + std::to_string(capacity) + " < " + std::to_string(total) +
                " rows";
      return ENOSPC;
    }
    if (nw && total) {
      SPJ_CHECK(d_out_idx != nullptr, "null output");
      k_bits_rows<<<g, 256, 0, s>>>(d_bitmap, n_build, visited ? 1u : 0u, pos.as<uint64_t>(),
                                    d_out_idx, capacity);
    }
    SPJ_CUDA(cudaGetLastError());
    SPJ_CUDA(cudaStreamSynchronize(s));
    g_error.clear();
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}
