// noalloc.cu — SpjIndexProbeNoAlloc: the candidate filter of a built
// SedonaFloatIndex2D for callers that cannot allocate device memory while
// they probe.
//
// Who needs it: an executor that hands the device's memory budget to its own
// arena at start-up (so a cudaMalloc at probe time fails or breaks the
// budget), or a latency-critical probe loop that must not touch the CUDA
// allocator at all.  The regular probe path allocates its per-probe count and
// offset arrays and its result buffers; this entry point allocates nothing.
//
// How: the count / offset / scan scratch lives in one file-scope
// `static __device__` array of kNoAllocScratchBytes (4 MiB) that every GPU
// loading the library holds until the process exits.  That bounds one call
// to kNoAllocMaxProbes (2^18) probe rects.  The caller passes the probe rects
// and the output buffers in device memory and gets the pair count back.
//
// Host code cannot use the array's name as a device address (in host code it
// is a host-side stand-in).  The first call on each device therefore looks up
// the array's device address with cudaGetSymbolAddress, with that device
// current, and caches it; that set-up allocates nothing, but it is a CUDA API
// call, so make the first call on a device before any stream capture.
//
// Every call shares the one array: calls that overlap on the GPU (different
// streams, or different host threads on one device) race on it and must be
// serialized by the caller.  Nothing in it needs clearing between calls: each
// call writes every count, offset and tile sum it reads.
//
// Pointer checks happen before any launch: d_rects must be 16-byte aligned
// (one float4 load per rect), the outputs 4-byte aligned, and all three
// device memory of the index's device.  A traversal fault recorded by either
// pass fails the call; the fault stays recorded in the index (see
// SpjIndexProbeNoAlloc in spj_gb300.h), so later probes of that index fail
// too until it is rebuilt.
#include <errno.h>

#include <mutex>
#include <string>

#include "../../include/gpuspatial_c.h"
#include "../../include/spj_gb300.h"
#include "lbvh.cuh"
#include "prims.cuh"

namespace spj {
// defined in capi.cu: the LBVH and device of a built SedonaFloatIndex2D
const Lbvh* index_lbvh(SedonaFloatIndex2D* index, int* device, std::string** last_error);
}  // namespace spj

namespace {

constexpr uint32_t kNoAllocMaxProbes = SPJ_NOALLOC_MAX_PROBES;
// counts (u32) + offsets (u64, one extra for the total) + scan tile sums
constexpr size_t kCountsBytes = (size_t)kNoAllocMaxProbes * 4;
constexpr size_t kOffsetsBytes = ((size_t)kNoAllocMaxProbes + 1) * 8;
constexpr size_t kNoAllocScratchBytes = 4u << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `device` (current), looked up once.
void* scratch_on(int device) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      throw spj::Error(std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    g_scratch_addr[device] = p;
  }
  return g_scratch_addr[device];
}

}  // namespace

extern "C" int SpjIndexProbeNoAlloc(struct SedonaFloatIndex2D* index, const float* d_rects,
                                    uint32_t n_rects, uint32_t* d_out_build,
                                    uint32_t* d_out_probe, uint64_t capacity, uint64_t* n_pairs,
                                    void* stream) {
  if (!index || !index->private_data) return EINVAL;
  int device = 0;
  std::string* err = nullptr;
  const spj::Lbvh* bvh = nullptr;
  try {
    bvh = spj::index_lbvh(index, &device, &err);
  } catch (const std::exception&) {
    return EINVAL;
  }
  try {
    SPJ_CHECK(bvh != nullptr, "index is not built (call finish_building first)");
    SPJ_CHECK(n_pairs != nullptr, "null n_pairs");
    SPJ_CHECK(n_rects <= kNoAllocMaxProbes,
              "n_rects " + std::to_string(n_rects) + " exceeds the no-allocation maximum of " +
                  std::to_string(kNoAllocMaxProbes) + " probe rects per call");
    SPJ_CHECK(n_rects == 0 || d_rects != nullptr, "null probe rects");
    // the traversal reads each rect with one 16-byte load and the scatter
    // writes 4-byte ids: a pointer off those boundaries would fault the
    // context, so it is rejected here, before anything is launched
    SPJ_CHECK(reinterpret_cast<uintptr_t>(d_rects) % 16 == 0,
              "d_rects is not 16-byte aligned (each rect is read as one float4)");
    SPJ_CHECK(reinterpret_cast<uintptr_t>(d_out_build) % 4 == 0 &&
                  reinterpret_cast<uintptr_t>(d_out_probe) % 4 == 0,
              "output buffers are not 4-byte aligned");
    SPJ_CHECK(device >= 0 && device < kMaxDevices, "device id out of range");
    // the caller's pointers must be device memory that the index's device can
    // address (cudaPointerGetAttributes allocates nothing)
    for (const void* ptr : {static_cast<const void*>(d_rects), static_cast<const void*>(d_out_build),
                            static_cast<const void*>(d_out_probe)}) {
      if (ptr == nullptr) continue;
      cudaPointerAttributes a{};
      if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();  // clear the error the failed query left behind
        throw spj::Error("a buffer pointer is not known to CUDA");
      }
      SPJ_CHECK(a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged,
                "d_rects and the output buffers must be device (or managed) memory");
      SPJ_CHECK(a.type == cudaMemoryTypeManaged || a.device == device,
                "a buffer lives on device " + std::to_string(a.device) +
                    ", the index on device " + std::to_string(device));
    }
    static_assert(kCountsBytes + kOffsetsBytes + 4096 <= kNoAllocScratchBytes,
                  "scratch too small");
    SPJ_CUDA(cudaSetDevice(device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char* base = static_cast<unsigned char*>(scratch_on(device));
    uint32_t* counts = reinterpret_cast<uint32_t*>(base);
    uint64_t* offs = reinterpret_cast<uint64_t*>(base + kCountsBytes);
    uint64_t* sums = reinterpret_cast<uint64_t*>(base + kCountsBytes + kOffsetsBytes);
    SPJ_CHECK(spj::scan_tile_sums_bytes(n_rects) <= kNoAllocScratchBytes - kCountsBytes -
                                                       kOffsetsBytes,
              "scan scratch too small");
    const spj::LbvhView t = bvh->view();
    const float4* boxes = reinterpret_cast<const float4*>(d_rects);
    spj::probe_count_into(t, boxes, n_rects, counts, s);
    spj::scan_u32_u64_into(counts, offs, n_rects, sums, s);
    uint64_t total = 0;
    SPJ_CUDA(cudaMemcpyAsync(&total, offs + n_rects, sizeof total, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    spj::check_traversal(t, s);
    *n_pairs = total;
    if (total > capacity) {
      if (err) *err = "output capacity " + std::to_string(capacity) + " < " +
                      std::to_string(total) + " candidate pairs";
      return ENOSPC;
    }
    SPJ_CHECK(total == 0 || (d_out_build && d_out_probe), "null output buffers");
    spj::probe_scatter_from(t, boxes, n_rects, offs, 0, d_out_build, d_out_probe, s);
    SPJ_CUDA(cudaStreamSynchronize(s));
    // a fault recorded by the scatter pass fails the call as well
    spj::check_traversal(t, s);
    if (err) err->clear();
    return 0;
  } catch (const std::exception& e) {
    if (err) *err = e.what();
    return EINVAL;
  }
}
