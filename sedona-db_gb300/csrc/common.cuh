// common.cuh — shared host/device plumbing for the GB300 spatial-join library.
//
// Error model: host code throws spj::Error (caught at the C ABI and turned
// into EINVAL + last_error, like the reference's SafeExecute wrapper in
// c/sedona-libgpuspatial/libgpuspatial/src/gpuspatial_c.cc:45-58).  Device
// code never traps: kernels record failures in a DeviceStatus word that the
// host reads after the launch (the reference's QueueView::Append __trap()s on
// overflow, include/gpuspatial/utils/queue_view.hpp:35-47; this build does not).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace spj {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define SPJ_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      throw ::spj::Error(std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " + \
                         __FILE__ + ":" + std::to_string(__LINE__));                     \
    }                                                                                    \
  } while (0)

#define SPJ_CHECK(cond, msg)                          \
  do {                                                \
    if (!(cond)) throw ::spj::Error(std::string(msg)); \
  } while (0)

constexpr int kWarp = 32;
constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs

inline int grid_for(int64_t n, int block, int max_blocks = kNumSMs * 16) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (int)g;
}

// Device-side status word: first failing row and an error code.  Kernels
// set it with atomics; the host decodes it after the stream syncs.
struct DeviceStatus {
  unsigned long long first_bad;  // (code << 40) | row, minimum wins
  unsigned long long counters[8];
};

enum StatusCode : uint32_t {
  kOk = 0,
  kWkbTruncated = 1,
  kWkbByteOrder = 2,
  kWkbType = 3,
  kWkbDims = 4,
  kWkbCount = 5,
  kOverflow = 6,
  kUnsupported = 7,
};

const char* status_message(uint32_t code);

__device__ __forceinline__ void status_fail(DeviceStatus* st, uint32_t code, uint64_t row) {
  unsigned long long v = ((unsigned long long)code << 40) | (row & 0xFFFFFFFFFFull);
  atomicMin(&st->first_bad, v);
}

// IEEE nextafter toward +inf / -inf (bit stepping), device and host.
__host__ __device__ __forceinline__ double next_up(double x) {
  if (x != x || x == __builtin_huge_val()) return x;
  if (x == 0.0) return 4.9406564584124654e-324;
  long long b;
  memcpy(&b, &x, 8);
  b += (x > 0) ? 1 : -1;
  double r;
  memcpy(&r, &b, 8);
  return r;
}
__host__ __device__ __forceinline__ double next_down(double x) { return -next_up(-x); }
__host__ __device__ __forceinline__ float next_upf(float x) {
  if (x != x || x == __builtin_huge_valf()) return x;
  if (x == 0.0f) return 1.40129846e-45f;
  int b;
  memcpy(&b, &x, 4);
  b += (x > 0) ? 1 : -1;
  float r;
  memcpy(&r, &b, 4);
  return r;
}
__host__ __device__ __forceinline__ float next_downf(float x) { return -next_upf(-x); }

// 32-byte aligned FP64 rectangle (min x, min y, max x, max y): one 256-bit load
struct __align__(32) Rect64 {
  double x, y, z, w;
};
__host__ __device__ __forceinline__ Rect64 make_rect64(double a, double b, double c, double d) {
  Rect64 r;
  r.x = a;
  r.y = b;
  r.z = c;
  r.w = d;
  return r;
}

// Count of buffers the library has allocated (device and page-locked host),
// exported as SpjAllocationCount; defined in capi.cu.
extern std::atomic<uint64_t> g_allocations;

// ---------------------------------------------------------------------------
// Stream-ordered device buffers (cudaMallocAsync from the device's default
// pool; the pool's release threshold is raised at runtime init so freed
// blocks stay cached across calls).

class DevBuf {
 public:
  DevBuf() = default;
  DevBuf(size_t bytes, cudaStream_t s) { alloc(bytes, s); }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p_(o.p_), n_(o.n_), s_(o.s_) {
    o.p_ = nullptr;
    o.n_ = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p_ = o.p_;
      n_ = o.n_;
      s_ = o.s_;
      o.p_ = nullptr;
      o.n_ = 0;
    }
    return *this;
  }
  void alloc(size_t bytes, cudaStream_t s) {
    release();
    s_ = s;
    n_ = bytes;
    if (bytes) {
      SPJ_CUDA(cudaMallocAsync(&p_, bytes, s));
      g_allocations.fetch_add(1, std::memory_order_relaxed);
    }
  }
  // grow-only reallocation (contents not preserved)
  void reserve(size_t bytes, cudaStream_t s) {
    if (bytes > n_ || p_ == nullptr) alloc(bytes > 0 ? bytes : 16, s);
    s_ = s;
  }
  void release() {
    if (p_) cudaFreeAsync(p_, s_);
    p_ = nullptr;
    n_ = 0;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p_);
  }
  void* get() const { return p_; }
  size_t size() const { return n_; }

 private:
  void* p_ = nullptr;
  size_t n_ = 0;
  cudaStream_t s_ = 0;
};

// Pinned host staging buffer (grow-only).
class PinnedBuf {
 public:
  ~PinnedBuf() {
    if (p_) cudaFreeHost(p_);
  }
  void reserve(size_t bytes) {
    if (bytes <= n_) return;
    if (p_) cudaFreeHost(p_);
    p_ = nullptr;
    SPJ_CUDA(cudaMallocHost(&p_, bytes));
    g_allocations.fetch_add(1, std::memory_order_relaxed);
    n_ = bytes;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p_);
  }

 private:
  void* p_ = nullptr;
  size_t n_ = 0;
};

}  // namespace spj
