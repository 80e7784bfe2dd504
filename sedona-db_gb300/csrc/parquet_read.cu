// parquet_read.cu — GeoParquet WKB column chunks decoded on the device, and
// the SpjParquet* entry points.
//
// One read (all on the handle's stream, one H2D copy of the chunk bytes):
//   host           footer (parsed at open); page headers read from the file
//                  -> page table; chunk bytes -> page-locked buffer in
//                  groups of whole pages on host threads, each of which
//                  builds the Snappy block index of the pages it read
//                  (snappy_block_index: a chain of element headers) while
//                  they are in cache.  A header longer than the read
//                  window: all chunk bytes first, the index while they are
//                  copied
//   k_snappy_frags warp per 64 KiB output block: each element's bytes moved
//                  by the 32 lanes (a back-reference shorter than its length
//                  repeats its pattern, so every lane's byte is known without
//                  waiting); k_snappy_pages: warp per page for pages whose
//                  elements cross block ends
//   k_dict_pages   warp per dictionary page: PLAIN byte arrays -> entries
//   k_data_pages   warp per data page: RLE / bit-packed definition levels ->
//                  per-row validity; PLAIN values (equal-length values are
//                  located in parallel after a parallel check of every length
//                  word, others by a walk) or dictionary indices -> per-row
//                  (address, length)
//   scan           lengths -> int64 offsets
//   k_copy_values  8 lanes per row, 4 rows at a time per warp: value bytes ->
//                  the output data buffer
//   k_pack_valid   validity bytes -> an Arrow bitmap (only with nulls)
// Every read of page bytes is bounded by its page; a malformed page sets a
// status word (first error: code, page) that the host turns into a message.
#include <errno.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <exception>
#include <memory>
#include <thread>

#include "../../include/spj_gb300.h"
#include "parquet.cuh"
#include "prims.cuh"

namespace spj {
namespace pq {
namespace {

enum PqError : uint32_t {
  kErrSnappy = 1,
  kErrLevels = 2,
  kErrPlain = 3,
  kErrDictIndex = 4,
  kErrDictPage = 5,
  kErrPageShort = 6,
};

__device__ __forceinline__ void set_error(uint32_t* status, uint32_t code, uint32_t page) {
  if (atomicCAS(status, 0u, code) == 0u) status[1] = page;
}

__device__ __forceinline__ uint32_t ld_le32(const uint8_t* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

__device__ __forceinline__ bool rd_varint(const uint8_t*& p, const uint8_t* end, uint64_t& v) {
  v = 0;
  for (int sh = 0; sh < 64; sh += 7) {
    if (p >= end) return false;
    const uint8_t b = *p++;
    v |= (uint64_t)(b & 0x7f) << sh;
    if (!(b & 0x80)) return true;
  }
  return false;
}

// Snappy block decompression by one warp (every lane runs the same element
// loop); false on malformed input.
__device__ bool unsnap_warp(const uint8_t* in, uint32_t in_n, uint8_t* out, uint32_t out_n) {
  const int lane = threadIdx.x & 31;
  const uint8_t* ip = in;
  const uint8_t* end = in + in_n;
  uint64_t ulen;
  if (!rd_varint(ip, end, ulen) || ulen != out_n) return false;
  uint32_t op = 0;
  while (ip < end) {
    const uint8_t tag = *ip++;
    uint32_t len, off = 0;
    const int kind = tag & 3;
    if (kind == 0) {
      len = (uint32_t)(tag >> 2) + 1;
      if (len > 60) {
        const int nb = (int)len - 60;
        if (end - ip < nb) return false;
        uint32_t v = 0;
        for (int b = 0; b < nb; b++) v |= (uint32_t)ip[b] << (8 * b);
        ip += nb;
        if (v == 0xffffffffu) return false;
        len = v + 1;
      }
      if ((uint64_t)(end - ip) < len || (uint64_t)op + len > out_n) return false;
      for (uint32_t i = lane; i < len; i += 32) out[op + i] = ip[i];
      ip += len;
    } else {
      if (kind == 1) {
        if (end - ip < 1) return false;
        len = ((tag >> 2) & 7) + 4;
        off = ((uint32_t)(tag >> 5) << 8) | ip[0];
        ip += 1;
      } else if (kind == 2) {
        if (end - ip < 2) return false;
        len = (uint32_t)(tag >> 2) + 1;
        off = (uint32_t)ip[0] | ((uint32_t)ip[1] << 8);
        ip += 2;
      } else {
        if (end - ip < 4) return false;
        len = (uint32_t)(tag >> 2) + 1;
        off = ld_le32(ip);
        ip += 4;
      }
      if (off == 0 || off > op || (uint64_t)op + len > out_n) return false;
      const uint8_t* from = out + op - off;
      if (off >= len) {
        for (uint32_t i = lane; i < len; i += 32) out[op + i] = from[i];
      } else {
        for (uint32_t i = lane; i < len; i += 32) out[op + i] = from[i % off];
      }
    }
    op += len;
    __syncwarp();  // the bytes just written may be the next element's source
  }
  return op == out_n;
}

// ---------------------------------------------------------------------------
// A warp's window on a byte range [base, base + n), staged in shared memory
// with 16-byte loads; positions are 32-bit offsets from base.  Every lane
// keeps the same walk position, so the reloads are warp-uniform.  A stage
// starts at the 16-byte boundary at or below the position and may end up to
// 15 bytes past the range: every device buffer these kernels read starts
// 256-byte aligned and keeps 16 bytes of slack after its last page, so those
// loads stay inside the allocation, and bytes outside the range are never
// used.  The shared buffer has 16 bytes beyond `cap` for win_u32's second
// word.
struct Win {
  const uint8_t* base;
  uint32_t n;
  uint8_t* buf;
  uint32_t cap;
  int32_t p0;  // position of buf[0]
  int32_t hi;  // end of the staged positions
};

__device__ __forceinline__ void win_init(Win& w, const uint8_t* base, uint32_t n, uint8_t* buf,
                                         uint32_t cap) {
  w.base = base;
  w.n = n;
  w.buf = buf;
  w.cap = cap;
  w.p0 = 0;
  w.hi = 0;
}

__device__ __forceinline__ void win_stage(Win& w, uint32_t pos) {
  const int lane = threadIdx.x & 31;
  __syncwarp();  // every lane is done with the previous stage
  const uintptr_t a = reinterpret_cast<uintptr_t>(w.base) + pos;
  const uintptr_t a0 = a & ~uintptr_t(15);
  const uintptr_t e = (reinterpret_cast<uintptr_t>(w.base) + w.n + 15) & ~uintptr_t(15);
  const uint32_t bytes = e - a0 < w.cap ? (uint32_t)(e - a0) : w.cap;
  // asynchronous 16-byte copies: every lane's loads are in flight at once
  // (plain loads and stores through generic pointers would wait for each
  // load before the next, as the two may alias), then one wait
  const uint4* s = reinterpret_cast<const uint4*>(a0);
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(w.buf);
  for (uint32_t i = lane; i < (bytes >> 4); i += 32)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d + i * 16), "l"(s + i)
                 : "memory");
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncwarp();
  w.p0 = (int32_t)pos - (int32_t)(a - a0);
  w.hi = w.p0 + (int32_t)bytes;
}

// positions [pos, pos + k) staged (k <= cap - 16, and pos + k <= n)
__device__ __forceinline__ void win_need(Win& w, uint32_t pos, uint32_t k) {
  if ((int32_t)pos < w.p0 || (int32_t)(pos + k) > w.hi) win_stage(w, pos);
}
__device__ __forceinline__ uint32_t win_u8(const Win& w, uint32_t pos) {
  return w.buf[pos - w.p0];
}
// four bytes at pos, little-endian: two aligned shared loads and a funnel shift
__device__ __forceinline__ uint32_t win_u32(const Win& w, uint32_t pos) {
  const uint32_t o = pos - (uint32_t)w.p0;
  const uint32_t* q = reinterpret_cast<const uint32_t*>(w.buf + (o & ~3u));
  return __funnelshift_r(q[0], q[1], (o & 3) * 8);
}

constexpr uint32_t kFragBytes = 1u << 16;  // Snappy's compression block
constexpr uint64_t kHeaderWindow = 4096;   // bytes read per page header from the file
constexpr uint64_t kReadGroup = 4ull << 20;  // bytes of whole pages per reader-thread read
constexpr uint32_t kFragWin = 2048;        // per warp, k_snappy_frags (headers, literals)
constexpr uint32_t kWalkWin = 16384;       // per warp, PLAIN walks
constexpr int kWalkThreads = 128;          // 4 walking warps per block
enum PageMode : uint8_t { kModeStored = 0, kModeFragments = 1, kModeSequential = 2, kModeBad = 3 };

// One Snappy element header at position ip of the window's range: output
// length, copy offset (0 for a literal; a copy's offset is never 0), and
// input bytes to the next element (header plus a literal's bytes).  false
// when it runs past the range or is a copy with offset 0.
__device__ __forceinline__ bool snappy_header(Win& w, uint32_t ip, uint32_t& len, uint32_t& off,
                                              uint32_t& adv, uint32_t& hdr) {
  win_need(w, ip, 5);
  const uint32_t tag = win_u8(w, ip);
  const uint32_t kind = tag & 3;
  const uint32_t room = w.n - ip;  // >= 1
  if (kind == 0) {
    off = 0;
    len = (tag >> 2) + 1;
    hdr = 1;
    if (len > 60) {
      const uint32_t nb = len - 60;
      if (nb + 1 > room) return false;
      const uint32_t v = win_u32(w, ip + 1) & (nb == 4 ? 0xffffffffu : ((1u << (8 * nb)) - 1));
      if (v == 0xffffffffu) return false;
      len = v + 1;
      hdr = 1 + nb;
    }
    if ((uint64_t)hdr + len > room) return false;
    adv = hdr + len;
    return true;
  }
  hdr = kind == 1 ? 2 : kind == 2 ? 3 : 5;
  if (hdr > room) return false;
  if (kind == 1) {
    len = ((tag >> 2) & 7) + 4;
    off = ((tag >> 5) << 8) | win_u8(w, ip + 1);
  } else {
    len = (tag >> 2) + 1;
    const uint32_t v = win_u32(w, ip + 1);
    off = kind == 2 ? (v & 0xffffu) : v;
  }
  adv = hdr;
  return off != 0;
}

// Warp per 64 KiB output block of a block-independent page: element
// headers and literal bytes through a shared-memory window of the input
// (restaged a window at a time, so an element does not wait on a global
// load), copies from the block's own output, all by the 32 lanes.  A copy
// that reaches before its block sends the page to k_snappy_pages.  Work item
// (page, block 0) also copies a v2 page's level bytes.
__global__ void __launch_bounds__(128) k_snappy_frags(
    const PageInfo* __restrict__ pages, const uint2* __restrict__ work, uint32_t nwork,
    const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
    const uint64_t* __restrict__ frag_base, const uint32_t* __restrict__ frag_ip,
    uint8_t* __restrict__ mode, uint32_t* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  Win w;
  for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nwork; t += nwarps) {
    const uint2 wk = work[t];
    const uint32_t p = wk.x, k = wk.y;
    const PageInfo pg = pages[p];
    if (mode[p] != kModeFragments) continue;
    const uint8_t* in0 = src + pg.src;
    uint8_t* out0 = dst + pg.dst;
    if (k == 0)
      for (uint32_t i = lane; i < pg.lvl_bytes; i += 32) out0[i] = in0[i];
    const uint32_t out_n = pg.raw_size - pg.lvl_bytes;
    const uint32_t f0 = k * kFragBytes;
    if (f0 >= out_n) continue;
    const uint32_t fl = min(kFragBytes, out_n - f0);
    const uint8_t* in = in0 + pg.lvl_bytes;
    uint8_t* out = out0 + pg.lvl_bytes + f0;
    win_init(w, in, pg.src_size - pg.lvl_bytes, smem + (threadIdx.x >> 5) * (kFragWin + 16),
             kFragWin);
    uint32_t ip = frag_ip[frag_base[p] + k], op = 0;
    bool ok = true, local = true;
    while (op < fl) {
      uint32_t len, off, adv, hdr;
      if (ip >= w.n || !snappy_header(w, ip, len, off, adv, hdr) || len > fl - op) {
        ok = false;
        break;
      }
      if (off == 0) {
        // in pieces that fit the window (snappy_header checked that the
        // literal lies inside the input)
        for (uint32_t done = 0; done < len;) {
          const uint32_t piece = min(len - done, kFragWin - 16);
          win_need(w, ip + hdr + done, piece);
          const uint8_t* s = w.buf + (ip + hdr + done - w.p0);
          for (uint32_t i = lane; i < piece; i += 32) out[op + done + i] = s[i];
          done += piece;
        }
      } else {
        if (off > op) {  // reaches into an earlier block (or before the stream)
          local = false;
          break;
        }
        const uint8_t* s = out + op - off;
        if (off >= len) {
          for (uint32_t i = lane; i < len; i += 32) out[op + i] = s[i];
        } else {
          for (uint32_t i = lane; i < len; i += 32) out[op + i] = s[i % off];
        }
      }
      __syncwarp();  // the bytes just written may be the next copy's source
      ip += adv;
      op += len;
    }
    if (lane == 0) {
      if (!local) mode[p] = kModeSequential;
      else if (!ok) set_error(status, kErrSnappy, p);
    }
  }
}

// Warp per page that the block index or the block pass found not
// block-independent: the whole page by one warp.
__global__ void k_snappy_pages(const PageInfo* __restrict__ pages, uint32_t np,
                               const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                               const uint8_t* __restrict__ mode, uint32_t* status) {
  const int lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < np; p += nwarps) {
    if (mode[p] != kModeSequential) continue;
    const PageInfo pg = pages[p];
    const uint8_t* in0 = src + pg.src;
    uint8_t* out0 = dst + pg.dst;
    for (uint32_t i = lane; i < pg.lvl_bytes; i += 32) out0[i] = in0[i];
    const bool ok = unsnap_warp(in0 + pg.lvl_bytes, pg.src_size - pg.lvl_bytes,
                                out0 + pg.lvl_bytes, pg.raw_size - pg.lvl_bytes);
    if (!ok && lane == 0) set_error(status, kErrSnappy, p);
  }
}

__device__ __forceinline__ const uint8_t* page_bytes(const PageInfo& pg, const uint8_t* src,
                                                     const uint8_t* dst) {
  return pg.in_src ? src + pg.src : dst + pg.dst;
}

// Dictionary pages: every lane walks the PLAIN values through the warp's
// shared-memory window; lane k % 32 writes entry k.
__global__ void k_dict_pages(const PageInfo* __restrict__ pages, uint32_t np,
                             const uint8_t* __restrict__ src, const uint8_t* __restrict__ dst,
                             const uint64_t* __restrict__ dict_base,
                             uint64_t* __restrict__ dict_ptr, uint32_t* __restrict__ dict_len,
                             uint32_t* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  Win w;
  for (uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < np; p += nwarps) {
    const PageInfo pg = pages[p];
    if (pg.kind != 0) continue;
    const uint8_t* page = page_bytes(pg, src, dst);
    win_init(w, page, pg.raw_size, smem + (threadIdx.x >> 5) * (kWalkWin + 16), kWalkWin);
    const uint64_t base = dict_base[pg.dict];
    uint32_t q = 0;
    for (uint32_t k = 0; k < pg.num_values; k++) {
      if (pg.raw_size - q < 4) {
        if (lane == 0) set_error(status, kErrDictPage, p);
        break;
      }
      win_need(w, q, 4);
      const uint32_t l = win_u32(w, q);
      if (pg.raw_size - q - 4 < l) {
        if (lane == 0) set_error(status, kErrDictPage, p);
        break;
      }
      if ((k & 31) == (uint32_t)lane) {
        dict_ptr[base + k] = reinterpret_cast<uint64_t>(page + q + 4);
        dict_len[base + k] = l;
      }
      q += 4 + l;
    }
  }
}

// RLE / bit-packed hybrid decode of `count` values of width bw (<= 32) by a
// warp: run headers are read by every lane (the same address), each run's
// values are written by the lanes in parallel.  false on malformed input.
template <class W>
__device__ bool rle_hybrid_warp(const uint8_t* p, const uint8_t* end, int bw, uint32_t count,
                                W&& write) {
  const int lane = threadIdx.x & 31;
  const int vbytes = (bw + 7) >> 3;
  const uint64_t mask = bw == 32 ? 0xffffffffull : ((1ull << bw) - 1);
  uint32_t i = 0;
  while (i < count) {
    uint64_t h;
    if (!rd_varint(p, end, h)) return false;
    if (h & 1) {
      const uint64_t groups = h >> 1;
      if (groups == 0 || groups > (1ull << 32)) return false;
      const uint64_t take = min(groups * 8, (uint64_t)(count - i));
      const uint64_t need = (take * (uint64_t)bw + 7) >> 3;
      if ((uint64_t)(end - p) < need) return false;
      for (uint64_t k = lane; k < take; k += 32) {
        uint32_t v = 0;
        if (bw) {
          const uint64_t bit = k * (uint64_t)bw;
          const uint8_t* b = p + (bit >> 3);
          const int sh = (int)(bit & 7);
          const uint64_t last = ((bit + (uint64_t)bw - 1) >> 3) - (bit >> 3);  // < 5
          uint64_t w = 0;
          for (uint64_t j = 0; j <= last; j++) w |= (uint64_t)b[j] << (8 * j);
          v = (uint32_t)((w >> sh) & mask);
        }
        write(i + (uint32_t)k, v);
      }
      const uint64_t run_bytes = groups * (uint64_t)bw;
      p = (uint64_t)(end - p) < run_bytes ? end : p + run_bytes;
      i += (uint32_t)take;
    } else {
      const uint64_t run = h >> 1;
      if (run == 0) return false;
      if (end - p < vbytes) return false;
      uint32_t v = 0;
      for (int j = 0; j < vbytes; j++) v |= (uint32_t)p[j] << (8 * j);
      p += vbytes;
      const uint64_t take = min(run, (uint64_t)(count - i));
      for (uint64_t k = lane; k < take; k += 32) write(i + (uint32_t)k, v);
      i += (uint32_t)take;
    }
  }
  return true;
}

struct RowArrays {
  uint8_t* valid;     // per row: 1 valid
  uint64_t* tmp_ptr;  // per non-null value of a page, at first_row + rank
  uint32_t* tmp_len;
  uint64_t* vptr;     // per row: value address (0 for null)
  uint32_t* vlen;     // per row: value length (0 for null)
  unsigned long long* nulls;
};

__global__ void k_data_pages(const PageInfo* __restrict__ pages, uint32_t np,
                             const uint8_t* __restrict__ src, const uint8_t* __restrict__ dst,
                             const uint64_t* __restrict__ dict_base,
                             const uint32_t* __restrict__ dict_n,
                             const uint64_t* __restrict__ dict_ptr,
                             const uint32_t* __restrict__ dict_len, RowArrays ra,
                             uint32_t* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < np; p += nwarps) {
    const PageInfo pg = pages[p];
    if (pg.kind == 0) continue;
    const uint8_t* raw = page_bytes(pg, src, dst);
    const uint8_t* end = raw + pg.raw_size;
    const uint64_t fr = pg.first_row;
    const uint32_t nv = pg.num_values;
    uint8_t* valid = ra.valid + fr;
    // definition levels, counting the non-null values as they are written
    const uint8_t* vp = raw;
    uint32_t ones = 0;
    if (pg.max_def == 0) {
      for (uint32_t i = lane; i < nv; i += 32) valid[i] = 1;
      ones = lane == 0 ? nv : 0;
    } else {
      bool ok = true;
      const uint8_t* lv = raw;
      const uint8_t* lend = raw;
      if (pg.kind == 1) {
        if (pg.raw_size < 4 || ld_le32(raw) > pg.raw_size - 4) {
          ok = false;
        } else {
          lv = raw + 4;
          lend = lv + ld_le32(raw);
          vp = lend;
        }
      } else {
        lend = raw + pg.def_len;
        vp = raw + pg.lvl_bytes;
      }
      if (ok)
        ok = rle_hybrid_warp(lv, lend, 1, nv, [&](uint32_t i, uint32_t v) {
          valid[i] = (uint8_t)(v & 1);
          ones += v & 1;
        });
      if (!ok) {
        if (lane == 0) set_error(status, kErrLevels, p);
        continue;
      }
    }
    const uint32_t m = __reduce_add_sync(0xffffffffu, ones);  // non-null values
    // values, by non-null rank; a page without nulls writes its rows' spans
    // directly (rank = row)
    const bool all_valid = m == nv;
    uint64_t* tptr = all_valid ? ra.vptr + fr : ra.tmp_ptr + fr;
    uint32_t* tlen = all_valid ? ra.vlen + fr : ra.tmp_len + fr;
    if (pg.encoding == kPlain) {
      const uint64_t avail = (uint64_t)(end - vp);
      bool fixed = false;
      if (m > 0 && avail >= 4) {
        const uint32_t L0 = ld_le32(vp);
        const uint64_t stride = (uint64_t)L0 + 4;
        if (stride * m == avail) {
          bool same = true;
          for (uint32_t k = lane; k < m; k += 32) same &= ld_le32(vp + k * stride) == L0;
          fixed = __all_sync(0xffffffffu, same);
          if (fixed)
            for (uint32_t k = lane; k < m; k += 32) {
              tptr[k] = reinterpret_cast<uint64_t>(vp + k * stride + 4);
              tlen[k] = L0;
            }
        }
      }
      if (!fixed) {
        // every lane walks the length words through the warp's window
        Win w;
        const uint32_t avail32 = (uint32_t)avail;
        win_init(w, vp, avail32, smem + (threadIdx.x >> 5) * (kWalkWin + 16), kWalkWin);
        // lane j keeps the span of value k0 + j of each group of 32 and the
        // warp stores a group at once (no per-value divergent store)
        bool good = true;
        uint32_t q = 0, my_q = 0, my_l = 0;
        for (uint32_t k = 0; k < m; k++) {
          if (avail32 - q < 4) {
            good = false;
            break;
          }
          win_need(w, q, 4);
          const uint32_t l = win_u32(w, q);
          if (avail32 - q - 4 < l) {
            good = false;
            break;
          }
          const bool mine = (k & 31) == (uint32_t)lane;
          my_q = mine ? q + 4 : my_q;
          my_l = mine ? l : my_l;
          if ((k & 31) == 31 || k + 1 == m) {
            const uint32_t k0 = k & ~31u;
            if (k0 + lane <= k) {
              tptr[k0 + lane] = reinterpret_cast<uint64_t>(vp + my_q);
              tlen[k0 + lane] = my_l;
            }
          }
          q += 4 + l;
        }
        if (!good) {
          if (lane == 0) set_error(status, kErrPlain, p);
          continue;
        }
      }
    } else {
      // dictionary indices: a bit-width byte, then the hybrid runs
      const uint32_t dn = dict_n[pg.dict];
      const uint64_t db = dict_base[pg.dict];
      bool good = m == 0 || (end - vp >= 1 && vp[0] <= 32);
      if (good && m > 0)
        good = rle_hybrid_warp(vp + 1, end, vp[0], m, [&](uint32_t k, uint32_t v) { tlen[k] = v; });
      if (!good) {
        if (lane == 0) set_error(status, kErrLevels, p);
        continue;
      }
      __syncwarp();
      bool inb = true;
      for (uint32_t k = lane; k < m; k += 32) {
        const uint32_t d = tlen[k];
        if (d >= dn) {
          inb = false;
          continue;
        }
        tptr[k] = dict_ptr[db + d];
        tlen[k] = dict_len[db + d];
      }
      if (!__all_sync(0xffffffffu, inb)) {
        if (lane == 0) set_error(status, kErrDictIndex, p);
        continue;
      }
    }
    if (all_valid) continue;
    __syncwarp();
    // rows: the rank of each valid row among the page's valid rows
    uint32_t base = 0, nnull = 0;
    for (uint32_t i0 = 0; i0 < nv; i0 += 32) {
      const uint32_t i = i0 + lane;
      const bool v = i < nv && valid[i];
      const unsigned b = __ballot_sync(0xffffffffu, v);
      if (i < nv) {
        if (v) {
          const uint32_t r = base + __popc(b & lt);
          ra.vptr[fr + i] = tptr[r];
          ra.vlen[fr + i] = tlen[r];
        } else {
          ra.vptr[fr + i] = 0;
          ra.vlen[fr + i] = 0;
        }
      }
      base += __popc(b);
      nnull += __popc(__ballot_sync(0xffffffffu, i < nv && !v));
    }
    if (lane == 0 && nnull) atomicAdd(ra.nulls, (unsigned long long)nnull);
  }
}

// A warp takes 32 rows: lane k reads row k's span and output position, then
// lane groups of 8 copy 4 values at a time (group_copy: whole destination
// words, any alignment).
__global__ void k_copy_values(const uint64_t* __restrict__ vptr,
                              const uint32_t* __restrict__ vlen,
                              const uint64_t* __restrict__ pos, uint64_t n,
                              uint8_t* __restrict__ out) {
  constexpr int G = 8;
  const int lane = threadIdx.x & 31, grp = lane / G, gl = lane % G;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; r0 < n;
       r0 += nwarps * 32) {
    const uint64_t r = r0 + lane;
    uint64_t sp = 0, d = 0;
    uint32_t l = 0;
    if (r < n) {
      l = vlen[r];
      sp = vptr[r];
      d = pos[r];
    }
    for (int v = 0; v < 32; v += 32 / G) {
      const uint64_t vs = __shfl_sync(0xffffffffu, sp, v + grp);
      const uint64_t vd = __shfl_sync(0xffffffffu, d, v + grp);
      const uint32_t vl = __shfl_sync(0xffffffffu, l, v + grp);
      if (vl) group_copy<G>(reinterpret_cast<const uint8_t*>(vs), out + vd, vl, gl);
    }
  }
}

__global__ void k_offsets64(const uint64_t* __restrict__ pos, uint64_t n,
                            int64_t* __restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (int64_t)pos[i];
}

__global__ void k_pack_valid(const uint8_t* __restrict__ valid, uint64_t n,
                             uint32_t* __restrict__ bits) {
  const uint64_t nw = (n + 31) / 32;
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw;
       w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t v = 0;
    for (int b = 0; b < 32; b++) {
      const uint64_t i = w * 32 + b;
      if (i < n && valid[i]) v |= 1u << b;
    }
    bits[w] = v;
  }
}

const char* error_name(uint32_t code) {
  switch (code) {
    case kErrSnappy: return "malformed Snappy data";
    case kErrLevels: return "malformed RLE / bit-packed run";
    case kErrPlain: return "PLAIN byte array values run past the page";
    case kErrDictIndex: return "dictionary index out of range";
    case kErrDictPage: return "malformed dictionary page";
    case kErrPageShort: return "page shorter than its level bytes";
    default: return "unknown error";
  }
}

// The Snappy block index of one compressed page, on the host: the input
// position of every 64 KiB output block.  Snappy writers compress 64 KiB
// blocks on their own, so when no element straddles a block end the blocks
// decode in parallel on the device (kModeFragments); otherwise the page is
// decoded by one warp (kModeSequential).  The walk over element headers is a
// chain (each header gives the next one's position; literal bytes are
// skipped) that a CPU core runs several times faster than one GPU warp, so
// the host walks the pages, on several threads, while the chunk bytes are
// copied to the device.  Malformed headers give kModeBad.
uint8_t snappy_block_index(const uint8_t* in, uint32_t n_in, uint32_t out_n,
                           uint32_t* frag_ip) {
  uint64_t ulen = 0;
  uint32_t pos = 0;
  for (;; pos++) {
    if (pos >= n_in || pos >= 5) return kModeBad;
    ulen |= (uint64_t)(in[pos] & 0x7f) << (7 * pos);
    if (!(in[pos] & 0x80)) break;
  }
  pos++;
  if (ulen != out_n) return kModeBad;
  frag_ip[0] = pos;
  uint32_t op = 0, fk = 0;
  uint64_t fe = kFragBytes;
  bool indep = true;
  while (pos < n_in) {
    const uint32_t tag = in[pos];
    const uint32_t room = n_in - pos;
    uint64_t len, adv;
    if ((tag & 3) == 0) {
      len = (tag >> 2) + 1;
      uint32_t hdr = 1;
      if (len > 60) {
        const uint32_t nb = (uint32_t)len - 60;
        if (nb + 1 > room) return kModeBad;
        uint64_t v = 0;
        for (uint32_t b = 0; b < nb; b++) v |= (uint64_t)in[pos + 1 + b] << (8 * b);
        len = v + 1;
        hdr = 1 + nb;
      }
      adv = hdr + len;
    } else {
      const uint32_t kind = tag & 3;
      adv = kind == 1 ? 2 : kind == 2 ? 3 : 5;
      if (adv > room) return kModeBad;
      len = kind == 1 ? ((tag >> 2) & 7) + 4 : (tag >> 2) + 1;
      uint32_t off = 0;
      if (kind == 1)
        off = ((tag >> 5) << 8) | in[pos + 1];
      else
        for (uint32_t b = 0; b + 1 < adv; b++) off |= (uint32_t)in[pos + 1 + b] << (8 * b);
      if (off == 0 || off > op) return kModeBad;
    }
    if (adv > room || len > out_n - op) return kModeBad;
    pos += (uint32_t)adv;
    op += (uint32_t)len;
    if (indep && op >= fe) {
      if (op > fe) {
        indep = false;  // an element straddles a block end
      } else if (op < out_n) {
        frag_ip[++fk] = pos;
        fe += kFragBytes;
      }
    }
  }
  if (op != out_n) return kModeBad;
  return indep ? kModeFragments : kModeSequential;
}

}  // namespace
}  // namespace pq
}  // namespace spj

using namespace spj;

struct SpjParquet {
  std::string path;
  int fd = -1;
  uint64_t file_len = 0;
  pq::FileMeta meta;
  std::string last_error;
  int device = -1;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[6] = {};  // start, after H2D, after Snappy, after decode, values start, end
  PinnedBuf stage_h;
  uint64_t stage_h_cap = 0;
  DevBuf stage, pages, pagebuf, dict_base, dict_n, dict_ptr, dict_len, valid, tmp_ptr, tmp_len,
      vptr, vlen, pos, scan_tmp, out_off, out_data, out_valid, status, nulls, frag_base, frag_ip,
      mode, work;
  double ms = 0, ms_phase[4] = {};  // H2D, decompress, decode, values
  uint64_t file_bytes = 0, page_bytes = 0, value_bytes = 0;

  // device buffers go before the stream they are freed on
  void release_device() {
    for (DevBuf* b : {&stage, &pages, &pagebuf, &dict_base, &dict_n, &dict_ptr, &dict_len,
                      &valid, &tmp_ptr, &tmp_len, &vptr, &vlen, &pos, &scan_tmp, &out_off,
                      &out_data, &out_valid, &status, &nulls, &frag_base, &frag_ip, &mode,
                      &work})
      b->release();
    if (stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
      stream = nullptr;
    }
    for (auto& e : ev) {
      if (e) cudaEventDestroy(e);
      e = nullptr;
    }
  }
  ~SpjParquet() {
    if (device >= 0) {
      cudaSetDevice(device);
      release_device();
    }
    if (fd >= 0) ::close(fd);
  }
  void read_at(uint64_t off, uint64_t n, uint8_t* out) const {
    while (n) {
      const ssize_t r = ::pread(fd, out, n, (off_t)off);
      if (r <= 0) throw Error("parquet: read failed at byte " + std::to_string(off));
      out += r;
      off += (uint64_t)r;
      n -= (uint64_t)r;
    }
  }
  // The byte ranges (file offset, length, destination) in 8 MiB pieces on
  // up to 16 host threads: one thread's copy out of the page cache runs far
  // below the memory bandwidth of the host.
  struct ReadPiece {
    uint64_t off, len;
    uint8_t* out;
  };
  void read_parallel(const std::vector<ReadPiece>& ranges) const {
    constexpr uint64_t kPiece = 8ull << 20;
    std::vector<ReadPiece> pieces;
    for (const ReadPiece& r : ranges)
      for (uint64_t d = 0; d < r.len; d += kPiece)
        pieces.push_back({r.off + d, std::min(kPiece, r.len - d), r.out + d});
    const size_t nt = std::min<size_t>(
        {16, std::max(1u, std::thread::hardware_concurrency()), pieces.size()});
    if (nt <= 1) {
      for (const ReadPiece& q : pieces) read_at(q.off, q.len, q.out);
      return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::exception_ptr> err(nt);
    auto run = [&](size_t t) {
      try {
        for (size_t i = next++; i < pieces.size(); i = next++)
          read_at(pieces[i].off, pieces[i].len, pieces[i].out);
      } catch (...) {
        err[t] = std::current_exception();
      }
    };
    std::vector<std::thread> th;
    for (size_t t = 1; t < nt; t++) th.emplace_back(run, t);
    run(0);
    for (auto& t : th) t.join();
    for (auto& e : err)
      if (e) std::rethrow_exception(e);
  }
};

namespace {

thread_local std::string g_pq_error;  // SpjParquetOpen and writer failures

int pq_fail(SpjParquet* p, const std::exception& e) {
  if (p) p->last_error = e.what();
  else g_pq_error = e.what();
  return EINVAL;
}

int find_leaf(const pq::FileMeta& m, const std::string& name) {
  for (size_t i = 0; i < m.leaves.size(); i++)
    if (m.leaves[i].name == name) return (int)i;
  return -1;
}

}  // namespace

extern "C" int SpjParquetOpen(const char* path, SpjParquet** out) {
  try {
    SPJ_CHECK(path != nullptr && out != nullptr, "null path or output");
    *out = nullptr;
    auto p = std::make_unique<SpjParquet>();
    p->path = path;
    p->fd = ::open(path, O_RDONLY);
    if (p->fd < 0) throw Error(std::string("parquet: cannot open ") + path);
    struct stat st;
    if (fstat(p->fd, &st) != 0) throw Error("parquet: cannot stat the file");
    p->file_len = (uint64_t)st.st_size;
    SPJ_CHECK(p->file_len >= 12, "parquet: file too short");
    uint64_t want = std::min<uint64_t>(p->file_len, 1 << 16);
    std::vector<uint8_t> tail;
    for (int tries = 0;; tries++) {
      tail.resize(want);
      p->read_at(p->file_len - want, want, tail.data());
      const uint64_t need = pq::parse_footer(tail.data(), want, p->file_len, p->meta);
      if (need == 0) break;
      SPJ_CHECK(tries == 0 && need <= p->file_len, "parquet: footer larger than announced");
      want = need;
    }
    *out = p.release();
    g_pq_error.clear();
    return 0;
  } catch (const std::exception& e) {
    return pq_fail(nullptr, e);
  }
}

extern "C" void SpjParquetRelease(SpjParquet* p) { delete p; }

extern "C" const char* SpjParquetLastError(SpjParquet* p) {
  return p ? p->last_error.c_str() : g_pq_error.c_str();
}

extern "C" int SpjParquetInfo(SpjParquet* p, int64_t* num_rows, int32_t* num_row_groups,
                              int32_t* num_columns) {
  try {
    SPJ_CHECK(p && num_rows && num_row_groups && num_columns, "null argument");
    *num_rows = p->meta.num_rows;
    *num_row_groups = (int32_t)p->meta.row_groups.size();
    *num_columns = (int32_t)p->meta.leaves.size();
    return 0;
  } catch (const std::exception& e) {
    return pq_fail(p, e);
  }
}

extern "C" int SpjParquetColumnName(SpjParquet* p, int32_t i, char* buf, uint64_t cap) {
  try {
    SPJ_CHECK(p && buf && cap > 0, "null argument");
    std::string name;
    if (i < 0) {
      SPJ_CHECK(!p->meta.primary_column.empty(), "the file has no GeoParquet primary column");
      name = p->meta.primary_column;
    } else {
      SPJ_CHECK((size_t)i < p->meta.leaves.size(), "column index out of range");
      name = p->meta.leaves[i].name;
    }
    SPJ_CHECK(name.size() < cap, "name buffer too small");
    memcpy(buf, name.c_str(), name.size() + 1);
    return 0;
  } catch (const std::exception& e) {
    return pq_fail(p, e);
  }
}

extern "C" int SpjParquetRowGroupRows(SpjParquet* p, int32_t rg, int64_t* rows) {
  try {
    SPJ_CHECK(p && rows, "null argument");
    SPJ_CHECK(rg >= 0 && (size_t)rg < p->meta.row_groups.size(), "row group out of range");
    *rows = p->meta.row_groups[rg].num_rows;
    return 0;
  } catch (const std::exception& e) {
    return pq_fail(p, e);
  }
}

extern "C" int SpjParquetReadWkb(SpjParquet* p, const char* column, int32_t rg_begin,
                                 int32_t rg_end, int32_t device, SpjDeviceWkb* out) {
  using namespace spj::pq;
  try {
    SPJ_CHECK(p && out, "null argument");
    const FileMeta& m = p->meta;
    const std::string name = column ? column : m.primary_column;
    SPJ_CHECK(!name.empty(), "no column given and the file has no GeoParquet primary column");
    for (auto& ge : m.geo_encodings)
      if (ge.first == name && ge.second != "WKB")
        throw Error("column " + name + " has GeoParquet encoding " + ge.second +
                    " (only WKB columns are read)");
    const int ci = find_leaf(m, name);
    SPJ_CHECK(ci >= 0, "no column named " + name);
    const Leaf& leaf = m.leaves[ci];
    SPJ_CHECK(leaf.top_level && leaf.max_rep == 0, "column " + name + " is nested");
    SPJ_CHECK(leaf.type == kByteArray, "column " + name + " is not BYTE_ARRAY");
    const int nrg = (int)m.row_groups.size();
    if (rg_end < 0 || rg_end > nrg) rg_end = nrg;
    SPJ_CHECK(rg_begin >= 0 && rg_begin <= rg_end, "bad row group range");

    // device and stream
    if (p->device != device && p->device >= 0) {
      SPJ_CUDA(cudaSetDevice(p->device));
      p->release_device();
    }
    p->device = device;
    SPJ_CUDA(cudaSetDevice(device));
    if (!p->stream) {
      SPJ_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
      for (auto& e : p->ev) SPJ_CUDA(cudaEventCreate(&e));
    }
    cudaStream_t s = p->stream;

    // the column chunks' byte ranges, read into the page-locked buffer
    struct Range {
      uint64_t off, len, at;
      int codec;
    };
    std::vector<Range> ranges;
    uint64_t total = 0, rows_expected = 0;
    for (int g = rg_begin; g < rg_end; g++) {
      const ColumnChunk& c = m.row_groups[g].columns[ci];
      SPJ_CHECK(c.type == kByteArray, "column chunk type is not BYTE_ARRAY");
      int64_t start = c.data_page_offset;
      if (c.dictionary_page_offset > 0 && c.dictionary_page_offset < start)
        start = c.dictionary_page_offset;
      SPJ_CHECK(start >= 4 && c.total_compressed >= 0 &&
                    (uint64_t)start + (uint64_t)c.total_compressed <= p->file_len,
                "column chunk outside the file");
      ranges.push_back({(uint64_t)start, (uint64_t)c.total_compressed, total, c.codec});
      total += (uint64_t)c.total_compressed;
      rows_expected += (uint64_t)m.row_groups[g].num_rows;
    }
    SPJ_CHECK(rows_expected < (1ull << 32), "more than 2^32 - 1 rows in one read");
    if (total + 16 > p->stage_h_cap) {
      p->stage_h.reserve(total + 16);
      p->stage_h_cap = total + 16;
    }
    uint8_t* hb = p->stage_h.as<uint8_t>();
    p->file_bytes = total;

    // The page table, from the page headers read straight from the file
    // (small reads), so that the reader threads can index the Snappy pages
    // they have just read while the bytes are in cache.  A header longer than
    // the read window (large statistics) falls back to reading the chunks
    // first and walking the pages in memory.
    std::vector<PageInfo> pages;
    std::vector<uint64_t> hpos;  // staging position of each page's header
    uint64_t row = 0;
    int ndict = 0;
    bool prewalked = true;
    try {
      std::vector<uint8_t> win;
      for (auto& r : ranges) {
        auto bytes_at = [&](uint64_t pos) {
          const uint64_t want = std::min<uint64_t>(kHeaderWindow, r.at + r.len - pos);
          win.resize(want);
          p->read_at(r.off + (pos - r.at), want, win.data());
          return std::make_pair((const uint8_t*)win.data(), (const uint8_t*)win.data() + want);
        };
        if (walk_pages(bytes_at, r.at, r.at + r.len, r.codec, leaf.max_def, ndict, &row, pages,
                       &hpos))
          ndict++;
      }
    } catch (const Error&) {
      prewalked = false;
    }
    if (!prewalked) {
      pages.clear();
      hpos.clear();
      row = 0;
      ndict = 0;
      std::vector<SpjParquet::ReadPiece> rd;
      for (auto& r : ranges) rd.push_back({r.off, r.len, hb + r.at});
      p->read_parallel(rd);
      for (auto& r : ranges)
        if (walk_pages(hb, r.at, r.at + r.len, r.codec, leaf.max_def, ndict, &row, pages)) ndict++;
    }
    SPJ_CHECK(row == rows_expected, "the pages hold " + std::to_string(row) +
                                        " values, the row groups " +
                                        std::to_string(rows_expected) + " rows");
    const uint64_t n = row;
    uint64_t dst = 0, dict_total = 0, pbytes = 0;
    std::vector<uint64_t> dict_base(ndict + 1, 0);
    std::vector<uint32_t> dict_n(ndict + 1, 0);
    for (auto& pg : pages) {
      pbytes += pg.raw_size;
      if (!pg.in_src) {
        pg.dst = dst;
        dst += (pg.raw_size + 15) & ~15ull;
      }
      if (pg.kind == 0) {
        dict_base[pg.dict] = dict_total;
        dict_n[pg.dict] = pg.num_values;
        dict_total += pg.num_values;
      }
    }
    p->page_bytes = pbytes;
    const uint32_t np = (uint32_t)pages.size();
    // Snappy work: per compressed page one item per 64 KiB output block (at
    // least one, which also copies a v2 page's level bytes)
    std::vector<uint64_t> frag_base(np + 1, 0);
    std::vector<uint2> work;
    uint64_t nfrag = 0;
    for (uint32_t i = 0; i < np; i++) {
      frag_base[i] = nfrag;
      if (pages[i].in_src) continue;
      const uint64_t out_n = pages[i].raw_size >= pages[i].lvl_bytes
                                 ? pages[i].raw_size - pages[i].lvl_bytes : 0;
      const uint64_t nf = std::max<uint64_t>(1, (out_n + kFragBytes - 1) / kFragBytes);
      for (uint64_t k = 0; k < nf; k++) work.push_back(make_uint2(i, (uint32_t)k));
      nfrag += nf;
    }
    frag_base[np] = nfrag;
    const uint32_t nwork = (uint32_t)work.size();

    // the Snappy block index of every compressed page (host threads)
    std::vector<uint8_t> mode(np + 1, kModeStored);
    std::vector<uint32_t> frag_ip(nfrag + 1, 0);
    auto index_page = [&](uint32_t i) {
      const PageInfo& pg = pages[i];
      if (pg.in_src) return;
      mode[i] = pg.lvl_bytes < pg.src_size && pg.lvl_bytes <= pg.raw_size
                    ? snappy_block_index(hb + pg.src + pg.lvl_bytes, pg.src_size - pg.lvl_bytes,
                                         pg.raw_size - pg.lvl_bytes,
                                         frag_ip.data() + frag_base[i])
                    : (uint8_t)kModeBad;
    };
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    if (prewalked) {
      // the chunk bytes in groups of whole pages (kReadGroup bytes or so): a
      // thread reads a group, then indexes its pages while they are in cache
      struct Group {
        uint64_t beg, end, file;
        uint32_t p0, p1;
      };
      std::vector<Group> groups;
      uint32_t i = 0;
      for (auto& r : ranges) {
        const uint64_t rend = r.at + r.len;
        uint64_t beg = r.at;
        uint32_t p0 = i;
        while (i < np && hpos[i] < rend) {
          const uint64_t pend = i + 1 < np && hpos[i + 1] < rend ? hpos[i + 1] : rend;
          i++;
          if (pend - beg >= kReadGroup || pend == rend) {
            groups.push_back({beg, pend, r.off + (beg - r.at), p0, i});
            beg = pend;
            p0 = i;
          }
        }
        if (beg < rend) groups.push_back({beg, rend, r.off + (beg - r.at), p0, i});
      }
      std::atomic<size_t> next{0};
      const size_t nt = std::min<size_t>({16, hw, groups.size()});
      std::vector<std::exception_ptr> err(std::max<size_t>(nt, 1));
      auto run = [&](size_t t) {
        try {
          for (size_t g = next++; g < groups.size(); g = next++) {
            const Group& gr = groups[g];
            p->read_at(gr.file, gr.end - gr.beg, hb + gr.beg);
            for (uint32_t k = gr.p0; k < gr.p1; k++) index_page(k);
          }
        } catch (...) {
          err[t] = std::current_exception();
        }
      };
      std::vector<std::thread> th;
      for (size_t t = 1; t < nt; t++) th.emplace_back(run, t);
      run(0);
      for (auto& t : th) t.join();
      for (auto& e : err)
        if (e) std::rethrow_exception(e);
    }
    SPJ_CUDA(cudaEventRecord(p->ev[0], s));
    p->stage.reserve(total + 16, s);
    SPJ_CUDA(cudaMemcpyAsync(p->stage.get(), hb, total, cudaMemcpyHostToDevice, s));
    SPJ_CUDA(cudaEventRecord(p->ev[1], s));
    if (!prewalked) {
      // while the chunk bytes travel (before any copy from pageable memory,
      // which would wait for the copy above)
      std::vector<uint32_t> todo;
      for (uint32_t k = 0; k < np; k++)
        if (!pages[k].in_src) todo.push_back(k);
      auto run = [&](size_t t, size_t nt) {
        for (size_t j = t; j < todo.size(); j += nt) index_page(todo[j]);
      };
      const size_t nt = std::min<size_t>({16, hw, (todo.size() + 3) / 4});
      std::vector<std::thread> th;
      for (size_t t = 1; t < nt; t++) th.emplace_back(run, t, nt);
      run(0, std::max<size_t>(nt, 1));
      for (auto& t : th) t.join();
    }
    for (uint32_t k = 0; k < np; k++)
      if (mode[k] == kModeBad)
        throw Error("parquet: malformed Snappy data in page " + std::to_string(k) +
                    " of the read (" + std::to_string(np) + " pages)");
    // the small tables come from pageable vectors: the copies complete
    // before the stream synchronisation below, while the vectors live
    p->pages.reserve(sizeof(PageInfo) * (np + 1), s);
    SPJ_CUDA(cudaMemcpyAsync(p->pages.get(), pages.data(), sizeof(PageInfo) * np,
                             cudaMemcpyHostToDevice, s));
    p->dict_base.reserve(8 * (ndict + 1), s);
    p->dict_n.reserve(4 * (ndict + 1), s);
    SPJ_CUDA(cudaMemcpyAsync(p->dict_base.get(), dict_base.data(), 8 * (ndict + 1),
                             cudaMemcpyHostToDevice, s));
    SPJ_CUDA(cudaMemcpyAsync(p->dict_n.get(), dict_n.data(), 4 * (ndict + 1),
                             cudaMemcpyHostToDevice, s));
    p->frag_base.reserve(8 * (np + 1), s);
    p->frag_ip.reserve(4 * (nfrag + 1), s);
    p->mode.reserve(np + 16, s);
    p->work.reserve(8 * (nwork + 1), s);
    SPJ_CUDA(cudaMemcpyAsync(p->frag_base.get(), frag_base.data(), 8 * (np + 1),
                             cudaMemcpyHostToDevice, s));
    SPJ_CUDA(cudaMemcpyAsync(p->frag_ip.get(), frag_ip.data(), 4 * (nfrag + 1),
                             cudaMemcpyHostToDevice, s));
    SPJ_CUDA(cudaMemcpyAsync(p->mode.get(), mode.data(), np + 1, cudaMemcpyHostToDevice, s));
    if (nwork)
      SPJ_CUDA(cudaMemcpyAsync(p->work.get(), work.data(), 8 * (size_t)nwork,
                               cudaMemcpyHostToDevice, s));
    p->pagebuf.reserve(dst + 16, s);
    p->dict_ptr.reserve(8 * (dict_total + 1), s);
    p->dict_len.reserve(4 * (dict_total + 1), s);
    p->valid.reserve(n + 16, s);
    p->tmp_ptr.reserve(8 * (n + 1), s);
    p->tmp_len.reserve(4 * (n + 1), s);
    p->vptr.reserve(8 * (n + 1), s);
    p->vlen.reserve(4 * (n + 1), s);
    p->pos.reserve(8 * (n + 1), s);
    p->out_off.reserve(8 * (n + 1), s);
    p->status.reserve(8, s);
    p->nulls.reserve(8, s);
    SPJ_CUDA(cudaMemsetAsync(p->status.get(), 0, 8, s));
    SPJ_CUDA(cudaMemsetAsync(p->nulls.get(), 0, 8, s));
    const PageInfo* dpages = p->pages.as<PageInfo>();
    const uint8_t* dsrc = p->stage.as<uint8_t>();
    uint8_t* dpb = p->pagebuf.as<uint8_t>();
    uint32_t* st = p->status.as<uint32_t>();
    if (nwork) {
      // Snappy: block-parallel decode, then the pages that are not
      // block-independent
      k_snappy_frags<<<grid_for((int64_t)nwork * 32, 128, kNumSMs * 16), 128,
                       4 * (kFragWin + 16), s>>>(
          dpages, p->work.as<uint2>(), nwork, dsrc, dpb, p->frag_base.as<uint64_t>(),
          p->frag_ip.as<uint32_t>(), p->mode.as<uint8_t>(), st);
      k_snappy_pages<<<grid_for((int64_t)np * 32, 128, kNumSMs * 16), 128, 0, s>>>(
          dpages, np, dsrc, dpb, p->mode.as<uint8_t>(), st);
    }
    SPJ_CUDA(cudaEventRecord(p->ev[2], s));
    // a walk restages its window when it runs past it: 16 KiB windows halve
    // the restages, and 4 warps per block keep a block's windows at 64 KiB
    const int g = grid_for((int64_t)np * 32, kWalkThreads, kNumSMs * 16);
    const int walk_smem = (kWalkThreads / 32) * (kWalkWin + 16);
    if (np) {
      SPJ_CUDA(cudaFuncSetAttribute(k_dict_pages, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    walk_smem));
      SPJ_CUDA(cudaFuncSetAttribute(k_data_pages, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    walk_smem));
      if (ndict)
        k_dict_pages<<<g, kWalkThreads, walk_smem, s>>>(dpages, np, dsrc, dpb,
                                               p->dict_base.as<uint64_t>(),
                                               p->dict_ptr.as<uint64_t>(),
                                               p->dict_len.as<uint32_t>(), st);
      RowArrays ra{p->valid.as<uint8_t>(),    p->tmp_ptr.as<uint64_t>(),
                   p->tmp_len.as<uint32_t>(), p->vptr.as<uint64_t>(),
                   p->vlen.as<uint32_t>(),    p->nulls.as<unsigned long long>()};
      k_data_pages<<<g, kWalkThreads, walk_smem, s>>>(dpages, np, dsrc, dpb, p->dict_base.as<uint64_t>(),
                                     p->dict_n.as<uint32_t>(), p->dict_ptr.as<uint64_t>(),
                                     p->dict_len.as<uint32_t>(), ra, st);
      SPJ_CUDA(cudaGetLastError());
    }
    SPJ_CUDA(cudaEventRecord(p->ev[3], s));
    uint32_t hst[2] = {0, 0};
    SPJ_CUDA(cudaMemcpyAsync(hst, st, 8, cudaMemcpyDeviceToHost, s));
    unsigned long long hnulls = 0;
    SPJ_CUDA(cudaMemcpyAsync(&hnulls, p->nulls.get(), 8, cudaMemcpyDeviceToHost, s));
    scan_u32_u64(p->vlen.as<uint32_t>(), p->pos.as<uint64_t>(), (int64_t)n, p->scan_tmp, s);
    uint64_t vbytes = 0;
    SPJ_CUDA(cudaMemcpyAsync(&vbytes, p->pos.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    if (hst[0]) {
      const uint32_t bad = hst[1] < np ? hst[1] : 0;
      throw Error(std::string("parquet: ") + pq::error_name(hst[0]) + " in page " +
                  std::to_string(bad) + " of the read (" + std::to_string(np) + " pages)");
    }
    p->value_bytes = vbytes;
    p->out_data.reserve(vbytes + 16, s);
    SPJ_CUDA(cudaEventRecord(p->ev[4], s));
    k_offsets64<<<grid_for((int64_t)n + 1, 256), 256, 0, s>>>(p->pos.as<uint64_t>(), n,
                                                              p->out_off.as<int64_t>());
    if (n)
      k_copy_values<<<grid_for((int64_t)n * 32, 256, kNumSMs * 32), 256, 0, s>>>(
          p->vptr.as<uint64_t>(), p->vlen.as<uint32_t>(), p->pos.as<uint64_t>(), n,
          p->out_data.as<uint8_t>());
    const uint8_t* validity = nullptr;
    if (hnulls) {
      p->out_valid.reserve(((n + 31) / 32) * 4 + 16, s);
      k_pack_valid<<<grid_for((int64_t)(n + 31) / 32, 256), 256, 0, s>>>(
          p->valid.as<uint8_t>(), n, p->out_valid.as<uint32_t>());
      validity = p->out_valid.as<uint8_t>();
    }
    SPJ_CUDA(cudaGetLastError());
    SPJ_CUDA(cudaEventRecord(p->ev[5], s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    float ms = 0;
    SPJ_CUDA(cudaEventElapsedTime(&ms, p->ev[0], p->ev[5]));
    p->ms = ms;
    const int from[4] = {0, 1, 2, 4}, to[4] = {1, 2, 3, 5};
    for (int i = 0; i < 4; i++) {
      SPJ_CUDA(cudaEventElapsedTime(&ms, p->ev[from[i]], p->ev[to[i]]));
      p->ms_phase[i] = ms;
    }
    out->length = (int64_t)n;
    out->offsets = p->out_off.get();
    out->offsets_are_64bit = 1;
    out->data = p->out_data.as<uint8_t>();
    out->data_length = vbytes;
    out->validity = validity;
    out->validity_offset = 0;
    p->last_error.clear();
    return 0;
  } catch (const std::exception& e) {
    return pq_fail(p, e);
  }
}

extern "C" int SpjParquetGetStats(SpjParquet* p, double* ms_device, uint64_t* file_bytes,
                                  uint64_t* page_bytes, uint64_t* value_bytes) {
  try {
    SPJ_CHECK(p && ms_device && file_bytes && page_bytes && value_bytes, "null argument");
    *ms_device = p->ms;
    *file_bytes = p->file_bytes;
    *page_bytes = p->page_bytes;
    *value_bytes = p->value_bytes;
    return 0;
  } catch (const std::exception& e) {
    return pq_fail(p, e);
  }
}

extern "C" int SpjParquetGetPhases(SpjParquet* p, double* ms_h2d, double* ms_decompress,
                                   double* ms_decode, double* ms_values) {
  try {
    SPJ_CHECK(p && ms_h2d && ms_decompress && ms_decode && ms_values, "null argument");
    *ms_h2d = p->ms_phase[0];
    *ms_decompress = p->ms_phase[1];
    *ms_decode = p->ms_phase[2];
    *ms_values = p->ms_phase[3];
    return 0;
  } catch (const std::exception& e) {
    return pq_fail(p, e);
  }
}

extern "C" int SpjParquetWriteWkb(const char* path, const char* column, int64_t length,
                                  const void* offsets, int32_t offsets_are_64bit,
                                  const uint8_t* data, const uint8_t* validity,
                                  int64_t validity_offset,
                                  const SpjParquetWriteOptions* options) {
  try {
    pq::WriteOptions o;
    if (options) {
      o.compression = options->compression;
      o.page_version = options->page_version;
      if (options->row_group_rows > 0) o.row_group_rows = options->row_group_rows;
      if (options->page_bytes > 0) o.page_bytes = options->page_bytes;
    }
    pq::write_wkb(path, column, length, offsets, offsets_are_64bit != 0, data, validity,
                  validity_offset, o);
    g_pq_error.clear();
    return 0;
  } catch (const std::exception& e) {
    return pq_fail(nullptr, e);
  }
}
