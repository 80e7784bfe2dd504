// capi.cu — the C ABI: the reference's GpuSpatialRuntime / SedonaFloatIndex2D /
// SedonaSpatialRefiner objects (include/gpuspatial_c.h) and the SpjJoin /
// SpjKnn extensions (include/spj_gb300.h), over the device engine.
//
// Error convention as the reference's SafeExecute
// (c/sedona-libgpuspatial/libgpuspatial/src/gpuspatial_c.cc:45-58): any
// exception becomes EINVAL plus a message kept on the object (or on the probe
// context, so concurrent probes do not overwrite each other's message).
#include <errno.h>

#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gpuspatial_c.h"
#include "../../include/spj_gb300.h"
#include "engine.cuh"
#include "knn.cuh"
#include "learned.cuh"
#include "partition.cuh"
#include "stream.cuh"
#include "prims.cuh"

// Arrow C data interface (https://arrow.apache.org/docs/format/CDataInterface.html)
#ifndef ARROW_C_DATA_INTERFACE
#define ARROW_C_DATA_INTERFACE
struct ArrowSchema {
  const char* format;
  const char* name;
  const char* metadata;
  int64_t flags;
  int64_t n_children;
  struct ArrowSchema** children;
  struct ArrowSchema* dictionary;
  void (*release)(struct ArrowSchema*);
  void* private_data;
};
struct ArrowArray {
  int64_t length;
  int64_t null_count;
  int64_t offset;
  int64_t n_buffers;
  int64_t n_children;
  const void** buffers;
  struct ArrowArray** children;
  struct ArrowArray* dictionary;
  void (*release)(struct ArrowArray*);
  void* private_data;
};
#endif

namespace {

using namespace spj;

template <class F>
int guarded(std::string& last_error, F&& f) {
  try {
    f();
    last_error.clear();
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return EINVAL;
  } catch (...) {
    last_error = "unknown internal error";
    return EINVAL;
  }
}

// --- runtime ----------------------------------------------------------------

struct RuntimeData {
  int device_id = 0;
  bool initialized = false;
  std::string last_error;
};

int rt_init(GpuSpatialRuntime* self, GpuSpatialRuntimeConfig* config) {
  auto* d = static_cast<RuntimeData*>(self->private_data);
  return guarded(d->last_error, [&] {
    SPJ_CHECK(config != nullptr, "null runtime config");
    int ndev = 0;
    SPJ_CUDA(cudaGetDeviceCount(&ndev));
    SPJ_CHECK(config->device_id >= 0 && config->device_id < ndev,
              "device_id " + std::to_string(config->device_id) + " out of range");
    SPJ_CUDA(cudaSetDevice(config->device_id));
    cudaMemPool_t pool;
    SPJ_CUDA(cudaDeviceGetDefaultMemPool(&pool, config->device_id));
    uint64_t thresh = UINT64_MAX;  // keep freed blocks cached across calls
    SPJ_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thresh));
    if (config->use_cuda_memory_pool && config->cuda_memory_pool_init_precent > 0) {
      SPJ_CHECK(config->cuda_memory_pool_init_precent <= 100,
                "cuda_memory_pool_init_precent must be in [0, 100]");
      size_t free_b = 0, total_b = 0;
      SPJ_CUDA(cudaMemGetInfo(&free_b, &total_b));
      size_t want = total_b / 100 * (size_t)config->cuda_memory_pool_init_precent;
      if (want > free_b / 10 * 9) want = free_b / 10 * 9;
      void* p = nullptr;
      SPJ_CUDA(cudaMallocAsync(&p, want, 0));
      g_allocations.fetch_add(1, std::memory_order_relaxed);
      SPJ_CUDA(cudaFreeAsync(p, 0));
      SPJ_CUDA(cudaStreamSynchronize(0));
    }
    d->device_id = config->device_id;
    d->initialized = true;
  });
}

void rt_release(GpuSpatialRuntime* self) {
  delete static_cast<RuntimeData*>(self->private_data);
  self->private_data = nullptr;
}

const char* rt_error(GpuSpatialRuntime* self) {
  return static_cast<RuntimeData*>(self->private_data)->last_error.c_str();
}

RuntimeData* runtime_of(const GpuSpatialRuntime* rt) {
  SPJ_CHECK(rt != nullptr && rt->private_data != nullptr, "null runtime");
  auto* d = static_cast<RuntimeData*>(rt->private_data);
  SPJ_CHECK(d->initialized, "runtime is not initialized");
  return d;
}

// --- workspace pool: one per concurrent caller -------------------------------

class WorkspacePool {
 public:
  explicit WorkspacePool(int device) : device_(device) {}
  std::unique_ptr<Workspace> acquire() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (!free_.empty()) {
        auto w = std::move(free_.back());
        free_.pop_back();
        return w;
      }
    }
    SPJ_CUDA(cudaSetDevice(device_));
    return std::make_unique<Workspace>();
  }
  void release(std::unique_ptr<Workspace> w) {
    std::lock_guard<std::mutex> lk(mu_);
    free_.push_back(std::move(w));
  }
  void clear() {
    std::lock_guard<std::mutex> lk(mu_);
    free_.clear();
  }

 private:
  int device_;
  std::mutex mu_;
  std::vector<std::unique_ptr<Workspace>> free_;
};

struct WsLease {
  WorkspacePool& pool;
  std::unique_ptr<Workspace> ws;
  explicit WsLease(WorkspacePool& p) : pool(p), ws(p.acquire()) {}
  ~WsLease() {
    if (ws) pool.release(std::move(ws));
  }
  Workspace& operator*() { return *ws; }
  Workspace* operator->() { return ws.get(); }
};

// --- Arrow binary parsing -----------------------------------------------------

HostWkbColumn parse_arrow(const ArrowSchema* schema, const ArrowArray* array) {
  SPJ_CHECK(schema != nullptr && array != nullptr, "null Arrow schema or array");
  SPJ_CHECK(schema->format != nullptr, "Arrow schema without format");
  const std::string fmt(schema->format);
  HostWkbColumn c;
  if (fmt == "z") c.offsets64 = false;
  else if (fmt == "Z") c.offsets64 = true;
  else throw Error("unsupported Arrow type '" + fmt + "': expected binary WKB (z or Z)");
  SPJ_CHECK(array->n_buffers == 3, "binary Arrow array must have 3 buffers");
  c.n = array->length;
  const size_t osz = c.offsets64 ? 8 : 4;
  c.offsets = static_cast<const uint8_t*>(array->buffers[1]) + (size_t)array->offset * osz;
  c.data = static_cast<const uint8_t*>(array->buffers[2]);
  if (array->null_count != 0 && array->buffers[0] != nullptr) {
    c.validity = static_cast<const uint8_t*>(array->buffers[0]);
    c.validity_offset = array->offset;
  }
  if (c.n > 0) SPJ_CHECK(array->buffers[1] != nullptr, "binary Arrow array without offsets");
  return c;
}

// Concatenation of pushed host batches (offsets rebased to one data buffer).
struct HostColumnBuilder {
  std::vector<int64_t> offsets{0};
  std::vector<uint8_t> data;
  std::vector<uint8_t> valid;  // one byte per row
  bool any_null = false;
  void append(const HostWkbColumn& c) {
    for (int64_t i = 0; i < c.n; i++) {
      int64_t s, e;
      if (c.offsets64) {
        s = reinterpret_cast<const int64_t*>(c.offsets)[i];
        e = reinterpret_cast<const int64_t*>(c.offsets)[i + 1];
      } else {
        s = reinterpret_cast<const int32_t*>(c.offsets)[i];
        e = reinterpret_cast<const int32_t*>(c.offsets)[i + 1];
      }
      bool v = true;
      if (c.validity) {
        int64_t b = c.validity_offset + i;
        v = (c.validity[b >> 3] >> (b & 7)) & 1;
      }
      valid.push_back(v ? 1 : 0);
      if (!v) any_null = true;
      if (v && e > s) data.insert(data.end(), c.data + s, c.data + e);
      offsets.push_back((int64_t)data.size());
    }
  }
  int64_t rows() const { return (int64_t)offsets.size() - 1; }
  void clear() {
    offsets.assign(1, 0);
    data.clear();
    valid.clear();
    any_null = false;
  }
  std::vector<uint8_t> bitmap() const {
    std::vector<uint8_t> bm((valid.size() + 7) / 8, 0);
    for (size_t i = 0; i < valid.size(); i++)
      if (valid[i]) bm[i >> 3] |= (uint8_t)(1u << (i & 7));
    return bm;
  }
};

// Build a join engine from a host column (H2D staged through a workspace).
void build_engine_from_host(JoinEngine& eng, WorkspacePool& pool, const HostColumnBuilder& hb) {
  WsLease ws(pool);
  std::vector<uint8_t> bm;
  HostWkbColumn c;
  c.n = hb.rows();
  c.offsets = hb.offsets.data();
  c.offsets64 = true;
  c.data = hb.data.data();
  if (hb.any_null) {
    bm = hb.bitmap();
    c.validity = bm.data();
  }
  uint64_t bytes = 0;
  WkbDeviceColumn d = stage_column(*ws, c, &bytes);
  SPJ_CUDA(cudaStreamSynchronize(ws->stream));  // staged column complete
  eng.build(d);
}

// --- SedonaFloatIndex2D ----------------------------------------------------

struct IndexData {
  RuntimeData* rt;
  // declared before bvh: members are destroyed in reverse order, and bvh's
  // buffers free on a pool workspace's stream
  std::unique_ptr<WorkspacePool> pool;
  std::vector<float> rects;
  Lbvh bvh;
  bool built = false;
  std::string last_error;
};

struct IndexContext {
  std::vector<uint32_t> build, probe;
  std::string last_error;
};

IndexData* idx_of(SedonaFloatIndex2D* self) {
  auto* d = static_cast<IndexData*>(self->private_data);
  SPJ_CUDA(cudaSetDevice(d->rt->device_id));
  return d;
}

int idx_clear(SedonaFloatIndex2D* self) {
  auto* d = static_cast<IndexData*>(self->private_data);
  return guarded(d->last_error, [&] {
    idx_of(self);
    d->rects.clear();
    d->bvh = Lbvh();
    d->built = false;
  });
}

void idx_create_ctx(SedonaSpatialIndexContext* ctx) { ctx->private_data = new IndexContext(); }
void idx_destroy_ctx(SedonaSpatialIndexContext* ctx) {
  delete static_cast<IndexContext*>(ctx->private_data);
  ctx->private_data = nullptr;
}

int idx_push(SedonaFloatIndex2D* self, const float* buf, uint32_t n) {
  auto* d = static_cast<IndexData*>(self->private_data);
  return guarded(d->last_error, [&] {
    idx_of(self);
    SPJ_CHECK(!d->built, "push_build after finish_building (call clear first)");
    SPJ_CHECK(n == 0 || buf != nullptr, "null rect buffer");
    d->rects.insert(d->rects.end(), buf, buf + (size_t)n * 4);
  });
}

int idx_finish(SedonaFloatIndex2D* self) {
  auto* d = static_cast<IndexData*>(self->private_data);
  return guarded(d->last_error, [&] {
    idx_of(self);
    WsLease ws(*d->pool);
    const uint32_t n = (uint32_t)(d->rects.size() / 4);
    DevBuf boxes(((size_t)n + 1) * 16, ws->stream);
    if (n)
      SPJ_CUDA(cudaMemcpyAsync(boxes.get(), d->rects.data(), (size_t)n * 16,
                               cudaMemcpyHostToDevice, ws->stream));
    build_lbvh(boxes.as<float4>(), n, 4, d->bvh, ws->stream);
    SPJ_CUDA(cudaStreamSynchronize(ws->stream));
    d->built = true;
  });
}

int idx_probe(SedonaFloatIndex2D* self, SedonaSpatialIndexContext* context, const float* buf,
              uint32_t n,
              int (*callback)(const uint32_t*, const uint32_t*, uint32_t, void*),
              void* user_data) {
  auto* d = static_cast<IndexData*>(self->private_data);
  auto* ctx = static_cast<IndexContext*>(context->private_data);
  int cb_status = 0;
  int rc = guarded(ctx->last_error, [&] {
    idx_of(self);
    SPJ_CHECK(d->built, "probe before finish_building");
    SPJ_CHECK(n == 0 || buf != nullptr, "null rect buffer");
    SPJ_CHECK(callback != nullptr, "null callback");
    WsLease ws(*d->pool);
    cudaStream_t s = ws->stream;
    ws->boxes_tmp.reserve(((size_t)n + 1) * 16, s);
    if (n)
      SPJ_CUDA(cudaMemcpyAsync(ws->boxes_tmp.get(), buf, (size_t)n * 16, cudaMemcpyHostToDevice,
                               s));
    const LbvhView tv = d->bvh.view();
    uint64_t m = probe_count(tv, ws->boxes_tmp.as<float4>(), n, ws->psc, s);
    SPJ_CHECK(m <= 0xFFFFFFFFull, "candidate count exceeds the 32-bit callback length");
    ws->cand_build.reserve((m + 1) * 4, s);
    ws->cand_probe.reserve((m + 1) * 4, s);
    probe_scatter(tv, ws->boxes_tmp.as<float4>(), n, ws->psc, 0, ws->cand_build.as<uint32_t>(),
                  ws->cand_probe.as<uint32_t>(), s);
    ctx->build.resize(m);
    ctx->probe.resize(m);
    if (m) {
      SPJ_CUDA(cudaMemcpyAsync(ctx->build.data(), ws->cand_build.get(), m * 4,
                               cudaMemcpyDeviceToHost, s));
      SPJ_CUDA(cudaMemcpyAsync(ctx->probe.data(), ws->cand_probe.get(), m * 4,
                               cudaMemcpyDeviceToHost, s));
    }
    SPJ_CUDA(cudaStreamSynchronize(s));
    cb_status = callback(ctx->build.data(), ctx->probe.data(), (uint32_t)m, user_data);
  });
  if (rc) return rc;
  return cb_status;
}

const char* idx_error(SedonaFloatIndex2D* self) {
  return static_cast<IndexData*>(self->private_data)->last_error.c_str();
}
const char* idx_ctx_error(SedonaSpatialIndexContext* ctx) {
  return static_cast<IndexContext*>(ctx->private_data)->last_error.c_str();
}
void idx_release(SedonaFloatIndex2D* self) {
  auto* d = static_cast<IndexData*>(self->private_data);
  if (d) {
    cudaSetDevice(d->rt->device_id);
    delete d;
  }
  self->private_data = nullptr;
}

// --- SedonaSpatialRefiner ----------------------------------------------------

struct RefinerData {
  RuntimeData* rt;
  std::string build_format;
  HostColumnBuilder host;
  std::unique_ptr<JoinEngine> engine;
  std::unique_ptr<WorkspacePool> pool;
  std::string last_error;
};

RefinerData* ref_of(SedonaSpatialRefiner* self) {
  auto* d = static_cast<RefinerData*>(self->private_data);
  SPJ_CUDA(cudaSetDevice(d->rt->device_id));
  return d;
}

int ref_clear(SedonaSpatialRefiner* self) {
  auto* d = static_cast<RefinerData*>(self->private_data);
  return guarded(d->last_error, [&] {
    ref_of(self);
    d->host.clear();
    EngineConfig cfg = d->engine->config();
    d->engine = std::make_unique<JoinEngine>(d->rt->device_id, cfg);
  });
}

int ref_init_schema(SedonaSpatialRefiner* self, const ArrowSchema* schema) {
  auto* d = static_cast<RefinerData*>(self->private_data);
  return guarded(d->last_error, [&] {
    SPJ_CHECK(schema != nullptr && schema->format != nullptr, "null build schema");
    std::string f(schema->format);
    SPJ_CHECK(f == "z" || f == "Z", "unsupported build Arrow type '" + f + "'");
    d->build_format = f;
  });
}

int ref_push(SedonaSpatialRefiner* self, const ArrowArray* array) {
  auto* d = static_cast<RefinerData*>(self->private_data);
  return guarded(d->last_error, [&] {
    SPJ_CHECK(!d->build_format.empty(), "push_build before init_build_schema");
    ArrowSchema sch{};
    sch.format = d->build_format.c_str();
    d->host.append(parse_arrow(&sch, array));
  });
}

int ref_finish(SedonaSpatialRefiner* self) {
  auto* d = static_cast<RefinerData*>(self->private_data);
  return guarded(d->last_error, [&] {
    ref_of(self);
    build_engine_from_host(*d->engine, *d->pool, d->host);
  });
}

int ref_refine(SedonaSpatialRefiner* self, const ArrowSchema* probe_schema,
               const ArrowArray* probe_array, SedonaSpatialRelationPredicate predicate,
               uint32_t* build_indices, uint32_t* probe_indices, uint32_t n,
               uint32_t* new_n) {
  auto* d = static_cast<RefinerData*>(self->private_data);
  return guarded(d->last_error, [&] {
    ref_of(self);
    SPJ_CHECK(d->engine->built(), "refine before finish_building");
    SPJ_CHECK(new_n != nullptr, "null new_indices_size");
    SPJ_CHECK(n == 0 || (build_indices && probe_indices), "null index arrays");
    const int p = (int)predicate;
    SPJ_CHECK(p >= 0 && p <= 7, "unknown predicate");
    HostWkbColumn pc = parse_arrow(probe_schema, probe_array);
    WsLease ws(*d->pool);
    cudaStream_t s = ws->stream;
    // bounds of the caller's indices are checked on the host: cheap and exact
    const uint32_t nb = d->engine->build_geoms().n;
    for (uint32_t i = 0; i < n; i++) {
      SPJ_CHECK(build_indices[i] < nb, "build index out of range");
      SPJ_CHECK(probe_indices[i] < (uint64_t)pc.n, "probe index out of range");
    }
    uint64_t bytes = 0;
    WkbDeviceColumn dc = stage_column(*ws, pc, &bytes);
    decode_wkb(dc, ws->probe, ws->dsc, false, s);
    ws->cand_build.reserve(((size_t)n + 1) * 4, s);
    ws->cand_probe.reserve(((size_t)n + 1) * 4, s);
    if (n) {
      SPJ_CUDA(cudaMemcpyAsync(ws->cand_build.get(), build_indices, (size_t)n * 4,
                               cudaMemcpyHostToDevice, s));
      SPJ_CUDA(cudaMemcpyAsync(ws->cand_probe.get(), probe_indices, (size_t)n * 4,
                               cudaMemcpyHostToDevice, s));
    }
    uint64_t kept = d->engine->refine_pairs(*ws, ws->probe.view(), ws->cand_build.as<uint32_t>(),
                                            ws->cand_probe.as<uint32_t>(), n, p, 0.0);
    // output ordered by probe index (reference: sort_probe_indices,
    // include/gpuspatial/refine/rt_spatial_refiner.hpp:48); the sort is
    // stable, so pairs of one probe keep their input order
    if (kept > 1) {
      DevBuf ak(kept * 4, s), av(kept * 4, s), tmp;
      int bits = 1;
      while (bits < 32 && ((uint64_t)pc.n >> bits) != 0) bits++;
      radix_sort_pairs(ws->out_probe.as<uint32_t>(), ws->out_build.as<uint32_t>(),
                       ak.as<uint32_t>(), av.as<uint32_t>(), (int64_t)kept, (bits + 7) / 8 * 8,
                       tmp, s);
    }
    if (kept) {
      SPJ_CUDA(cudaMemcpyAsync(build_indices, ws->out_build.get(), kept * 4,
                               cudaMemcpyDeviceToHost, s));
      SPJ_CUDA(cudaMemcpyAsync(probe_indices, ws->out_probe.get(), kept * 4,
                               cudaMemcpyDeviceToHost, s));
    }
    SPJ_CUDA(cudaStreamSynchronize(s));
    *new_n = (uint32_t)kept;
  });
}

const char* ref_error(SedonaSpatialRefiner* self) {
  return static_cast<RefinerData*>(self->private_data)->last_error.c_str();
}
void ref_release(SedonaSpatialRefiner* self) {
  auto* d = static_cast<RefinerData*>(self->private_data);
  if (d) {
    cudaSetDevice(d->rt->device_id);
    delete d;
  }
  self->private_data = nullptr;
}

}  // namespace

namespace spj {
// The LBVH of a built SedonaFloatIndex2D (nullptr before finish_building), its
// runtime's device and its last-error slot; used by SpjIndexProbeNoAlloc.
const Lbvh* index_lbvh(SedonaFloatIndex2D* index, int* device, std::string** last_error) {
  auto* d = static_cast<IndexData*>(index->private_data);
  *device = d->rt->device_id;
  *last_error = &d->last_error;
  return d->built ? &d->bvh : nullptr;
}
}  // namespace spj

// =============================================================================
// exported: reference interface

extern "C" void GpuSpatialRuntimeCreate(GpuSpatialRuntime* runtime) {
  runtime->init = rt_init;
  runtime->release = rt_release;
  runtime->get_last_error = rt_error;
  runtime->private_data = new RuntimeData();
}

extern "C" int GpuSpatialIndexFloat2DCreate(SedonaFloatIndex2D* index,
                                            const GpuSpatialIndexConfig* config) {
  try {
    SPJ_CHECK(index && config, "null index or config");
    RuntimeData* rt = runtime_of(config->runtime);
    SPJ_CUDA(cudaSetDevice(rt->device_id));
    auto* d = new IndexData();
    d->rt = rt;
    d->pool = std::make_unique<WorkspacePool>(rt->device_id);
    index->clear = idx_clear;
    index->create_context = idx_create_ctx;
    index->destroy_context = idx_destroy_ctx;
    index->push_build = idx_push;
    index->finish_building = idx_finish;
    index->probe = idx_probe;
    index->get_last_error = idx_error;
    index->context_get_last_error = idx_ctx_error;
    index->release = idx_release;
    index->private_data = d;
    return 0;
  } catch (const std::exception& e) {
    fprintf(stderr, "GpuSpatialIndexFloat2DCreate: %s\n", e.what());
    return EINVAL;
  }
}

extern "C" int GpuSpatialRefinerCreate(SedonaSpatialRefiner* refiner,
                                       const GpuSpatialRefinerConfig* config) {
  try {
    SPJ_CHECK(refiner && config, "null refiner or config");
    RuntimeData* rt = runtime_of(config->runtime);
    SPJ_CUDA(cudaSetDevice(rt->device_id));
    auto* d = new RefinerData();
    d->rt = rt;
    d->engine = std::make_unique<JoinEngine>(rt->device_id, EngineConfig());
    d->pool = std::make_unique<WorkspacePool>(rt->device_id);
    refiner->clear = ref_clear;
    refiner->init_build_schema = ref_init_schema;
    refiner->push_build = ref_push;
    refiner->finish_building = ref_finish;
    refiner->refine = ref_refine;
    refiner->get_last_error = ref_error;
    refiner->release = ref_release;
    refiner->private_data = d;
    return 0;
  } catch (const std::exception& e) {
    fprintf(stderr, "GpuSpatialRefinerCreate: %s\n", e.what());
    return EINVAL;
  }
}

// =============================================================================
// exported: SpjJoin

struct SpjJoin {
  RuntimeData* rt = nullptr;
  std::unique_ptr<JoinEngine> engine;
  // ST_DWithin distance column (one per probe row), set by
  // SpjJoinSetProbeDistances; freed on the join's own stream
  DevBuf dist;
  uint64_t dist_n = 0;
  bool has_dist = false;
  std::unique_ptr<WorkspacePool> pool;
  std::unique_ptr<Workspace> ws;   // the join's own stream and scratch
  std::unique_ptr<Workspace> ws2;  // second slot of the sliced host probe
  HostColumnBuilder host;
  std::vector<uint32_t> hb, hp;
  std::string last_error;
  PartitionLayout layout;  // the last partitioned join's partitioning
  // per workspace slot: a second stream for device -> host pair copies (two
  // copy engines at once) and its fork / join events
  struct CopyLane {
    cudaStream_t stream = nullptr;
    cudaEvent_t ready = nullptr, copied = nullptr;
    // sliced host probe: a slice's pair buffers, handed over by its
    // workspace while their device -> host copy runs
    DevBuf hold_build, hold_probe;
    bool pending = false;  // `copied` marks a copy of the hold buffers
  } lanes[2];
  ~SpjJoin() {
    // the distance column frees on the workspace's stream: before it goes
    if (ws) {
      dist.release();
      cudaStreamSynchronize(ws->stream);
    }
    for (auto& l : lanes) {
      if (l.stream) {
        cudaStreamSynchronize(l.stream);
        cudaStreamDestroy(l.stream);
      }
      if (l.ready) cudaEventDestroy(l.ready);
      if (l.copied) cudaEventDestroy(l.copied);
    }
  }
};

// Both pair arrays to host memory: build ids on the workspace's stream, probe
// ids on the lane's second stream, so that two copy engines move them at
// once.  Stream-ordered: the workspace's stream waits for both copies.
static void copy_pairs_to_host(SpjJoin* j, Workspace& w, int lane, const uint32_t* db,
                               const uint32_t* dp, uint64_t m, uint32_t* hb, uint32_t* hp) {
  cudaStream_t s = w.stream;
  SpjJoin::CopyLane& l = j->lanes[lane];
  if (!l.stream) {
    SPJ_CUDA(cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking));
    SPJ_CUDA(cudaEventCreateWithFlags(&l.ready, cudaEventDisableTiming));
    SPJ_CUDA(cudaEventCreateWithFlags(&l.copied, cudaEventDisableTiming));
  }
  SPJ_CUDA(cudaEventRecord(l.ready, s));
  SPJ_CUDA(cudaStreamWaitEvent(l.stream, l.ready, 0));
  SPJ_CUDA(cudaMemcpyAsync(hp, dp, m * 4, cudaMemcpyDeviceToHost, l.stream));
  SPJ_CUDA(cudaMemcpyAsync(hb, db, m * 4, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaEventRecord(l.copied, l.stream));
  SPJ_CUDA(cudaStreamWaitEvent(s, l.copied, 0));
}
static void copy_pairs_to_host(SpjJoin* j, const uint32_t* db, const uint32_t* dp, uint64_t m,
                               uint32_t* hb, uint32_t* hp) {
  copy_pairs_to_host(j, *j->ws, 0, db, dp, m, hb, hp);
}

// One slice's pairs (in w.out_*) to host memory without holding up w's next
// slice: w's output buffers are swapped with the lane's hold buffers (whose
// previous copy w's stream first waits for, long finished in steady state),
// and the copies read the handed-over buffers on the lane's stream.
static void copy_slice_to_host(SpjJoin* j, Workspace& w, int lane, const uint32_t* db,
                               const uint32_t* dp, uint64_t m, uint32_t* hb, uint32_t* hp) {
  SpjJoin::CopyLane& l = j->lanes[lane];
  if (!l.stream) {
    SPJ_CUDA(cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking));
    SPJ_CUDA(cudaEventCreateWithFlags(&l.ready, cudaEventDisableTiming));
    SPJ_CUDA(cudaEventCreateWithFlags(&l.copied, cudaEventDisableTiming));
  }
  if (l.pending) SPJ_CUDA(cudaStreamWaitEvent(w.stream, l.copied, 0));
  std::swap(w.out_build, l.hold_build);
  std::swap(w.out_probe, l.hold_probe);
  SPJ_CUDA(cudaEventRecord(l.ready, w.stream));
  SPJ_CUDA(cudaStreamWaitEvent(l.stream, l.ready, 0));
  SPJ_CUDA(cudaMemcpyAsync(hb, db, m * 4, cudaMemcpyDeviceToHost, l.stream));
  SPJ_CUDA(cudaMemcpyAsync(hp, dp, m * 4, cudaMemcpyDeviceToHost, l.stream));
  SPJ_CUDA(cudaEventRecord(l.copied, l.stream));
  l.pending = true;
}

// Sliced host probe: the rows are cut into slices, probed by two host
// threads on two workspaces (even and odd slices).  Pairs come out in the
// same order as one call over all rows (slices are row ranges in order, each
// call groups its pairs by probe row, and slice i lands after slice i-1).
constexpr int64_t kSliceMinRows = 1 << 18;

// Auto: two slices from 2 x kSliceMinRows rows.  Each of the two threads then
// probes one half, both halves' kernels share the GPU, and each half's copies
// overlap the other's kernels.  2M x 50k polygons, host-to-host per call:
// 2 slices 56.1 ms, 3 60.7, 4 65.7, 8 68.7 (the device-resident step is
// 55.4 ms): every slice adds its own host syncs and launch tails.
static int host_slices(const HostWkbColumn& c, int configured) {
  if (c.offsets == nullptr || c.n == 0) return 1;
  if (configured > 0) return (int)std::max<int64_t>(1, std::min<int64_t>(configured, c.n));
  return c.n < 2 * kSliceMinRows ? 1 : 2;
}

static HostWkbColumn host_slice(const HostWkbColumn& c, int64_t r0, int64_t r1) {
  HostWkbColumn s = c;
  s.n = r1 - r0;
  s.offsets = static_cast<const uint8_t*>(c.offsets) + r0 * (c.offsets64 ? 8 : 4);
  s.validity_offset = c.validity_offset + r0;
  return s;
}

// Returns the total pair count; copies them only while they fit.
static uint64_t probe_host_sliced(SpjJoin* j, const HostWkbColumn& hc, int nslices,
                                  int32_t predicate, double distance, uint32_t probe_base,
                                  uint32_t* out_build, uint32_t* out_probe, uint64_t capacity) {
  if (!j->ws2) j->ws2 = std::make_unique<Workspace>();
  Workspace* W[2] = {j->ws.get(), j->ws2.get()};
  const int dev = j->rt->device_id;
  auto rows = [&](int i) { return hc.n * i / nslices; };
  // Two host threads, one per workspace, take the even and the odd slices:
  // both slices' kernels are in flight on the GPU at once (the slow tail of
  // one launch overlaps the other slice's work), and the copies of a slice
  // overlap the other's kernels.  Slice i's pairs go to the host offset
  // start[i], known once slice i-1 has counted its pairs.
  std::vector<uint64_t> start((size_t)nslices + 1, 0);
  std::vector<char> known((size_t)nslices + 1, 0);
  known[0] = 1;
  std::mutex mu;
  std::condition_variable cv;
  bool abort = false;
  std::exception_ptr err[2];
  auto worker = [&](int t) {
    try {
      SPJ_CUDA(cudaSetDevice(dev));
      Workspace& w = *W[t];
      for (int i = t; i < nslices; i += 2) {
        uint64_t bytes = 0;
        const WkbDeviceColumn dc = stage_column(w, host_slice(hc, rows(i), rows(i + 1)), &bytes);
        const uint32_t *db, *dp;
        const uint64_t m = j->engine->probe(w, dc, predicate, distance,
                                            probe_base + (uint32_t)rows(i), &db, &dp);
        uint64_t off = 0;
        {
          std::unique_lock<std::mutex> lk(mu);
          cv.wait(lk, [&] { return known[i] != 0 || abort; });
          if (abort) return;
          off = start[i];
          start[i + 1] = off + m;
          known[i + 1] = 1;
        }
        cv.notify_all();
        if (m && off + m <= capacity) {
          SPJ_CHECK(out_build && out_probe, "null output buffers");
          copy_slice_to_host(j, w, t, db, dp, m, out_build + off, out_probe + off);
        }
      }
      SPJ_CUDA(cudaStreamSynchronize(w.stream));
      if (j->lanes[t].stream) SPJ_CUDA(cudaStreamSynchronize(j->lanes[t].stream));
    } catch (...) {
      err[t] = std::current_exception();
      {
        std::lock_guard<std::mutex> lk(mu);
        abort = true;
      }
      cv.notify_all();
    }
  };
  std::thread second(worker, 1);
  worker(0);
  second.join();
  for (auto& e : err)
    if (e) std::rethrow_exception(e);
  return start[(size_t)nslices];
}

extern "C" int SpjJoinCreate(const SpjJoinConfig* config, SpjJoin** out) {
  try {
    SPJ_CHECK(config && out, "null config or output");
    RuntimeData* rt = runtime_of(config->runtime);
    SPJ_CUDA(cudaSetDevice(rt->device_id));
    EngineConfig ec;
    if (config->leaf_size) ec.leaf_size = config->leaf_size;
    ec.refine_form = config->refine_form;
    SPJ_CHECK(ec.refine_form == kPlainF64 || ec.refine_form == kFastF32, "unknown refine_form");
    ec.profile = config->profile != 0;
    SPJ_CHECK(config->probe_order >= -1 && config->probe_order <= 1, "unknown probe_order");
    ec.probe_order = config->probe_order;
    auto j = std::make_unique<SpjJoin>();
    j->rt = rt;
    j->engine = std::make_unique<JoinEngine>(rt->device_id, ec);
    j->pool = std::make_unique<WorkspacePool>(rt->device_id);
    j->ws = std::make_unique<Workspace>();
    *out = j.release();
    return 0;
  } catch (const std::exception& e) {
    fprintf(stderr, "SpjJoinCreate: %s\n", e.what());
    return EINVAL;
  }
}

extern "C" void SpjJoinRelease(SpjJoin* j) {
  if (!j) return;
  cudaSetDevice(j->rt->device_id);
  delete j;
}

extern "C" const char* SpjJoinLastError(SpjJoin* j) { return j->last_error.c_str(); }

extern "C" int SpjJoinSetOption(SpjJoin* j, const char* key, int64_t value) {
  return guarded(j->last_error, [&] {
    SPJ_CHECK(key != nullptr, "null option key");
    EngineConfig& c = j->engine->config();
    const std::string k(key);
    if (k == "probe_order") {
      SPJ_CHECK(value >= -1 && value <= 1, "probe_order must be -1, 0 or 1");
      c.probe_order = (int)value;
    } else if (k == "candidate_order") {
      SPJ_CHECK(value == 0 || value == 2 || value == 3, "candidate_order must be 0, 2 or 3");
      c.candidate_order = (int)value;
    } else if (k == "order_tiles") {
      SPJ_CHECK(value >= -1 && value <= 16, "order_tiles must be -1 (auto) or in [0, 16]");
      c.order_tiles = (int)value;
    } else if (k == "refine_split") {
      SPJ_CHECK(value >= 0 && value <= 3, "refine_split must be 0, 1, 2 or 3");
      c.refine_split = (int)value;
    } else if (k == "host_slices") {
      SPJ_CHECK(value >= 0 && value <= 64, "host_slices must be in [0, 64]");
      c.host_slices = (int)value;
    } else if (k == "cell_grid") {
      SPJ_CHECK(value == 0 || value == 1, "cell_grid must be 0 or 1");
      c.cell_grid = value != 0;  // takes effect at the next build
    } else if (k == "grid_rings") {
      SPJ_CHECK(value == 0 || value == 1, "grid_rings must be 0 or 1");
      c.grid_rings = value != 0;
      j->engine->set_grid_rings(c.grid_rings);
    } else if (k == "dwithin_arena") {
      SPJ_CHECK(value >= 0 && value <= 2, "dwithin_arena must be 0, 1 or 2");
      c.dwithin_arena = (int)value;
    } else if (k == "dwithin_slots") {
      SPJ_CHECK(value >= 0 && value <= 1024, "dwithin_slots must be in [0, 1024]");
      c.dwithin_slots = (uint32_t)value;
    } else if (k == "fuse_dwithin") {
      SPJ_CHECK(value == 0 || value == 1, "fuse_dwithin must be 0 or 1");
      c.fuse_dwithin = value != 0;  // takes effect at the next build
    } else if (k == "refine_min_blocks") {
      SPJ_CHECK(value == 0 || value == 4 || value == 6,
                "refine_min_blocks must be 0 (auto), 4 or 6");
      c.refine_min_blocks = (int)value;
    } else {
      throw Error("unknown option '" + k + "'");
    }
  });
}

extern "C" int SpjJoinPushBuildArrow(SpjJoin* j, const ArrowSchema* schema,
                                     const ArrowArray* array) {
  return guarded(j->last_error, [&] { j->host.append(parse_arrow(schema, array)); });
}

extern "C" int SpjJoinFinishBuild(SpjJoin* j) {
  return guarded(j->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(j->rt->device_id));
    build_engine_from_host(*j->engine, *j->pool, j->host);
    j->host.clear();
  });
}

static WkbDeviceColumn device_column(const SpjDeviceWkb* c) {
  SPJ_CHECK(c != nullptr, "null column");
  SPJ_CHECK(c->length >= 0, "negative column length");
  SPJ_CHECK(c->length == 0 || (c->offsets && c->data), "null device buffers");
  WkbDeviceColumn d;
  d.n = c->length;
  d.offsets = c->offsets;
  d.offsets64 = c->offsets_are_64bit != 0;
  d.data = c->data;
  d.data_len = c->data_length;
  d.validity = c->validity;
  d.validity_offset = c->validity_offset;
  return d;
}

extern "C" int SpjJoinBuildDevice(SpjJoin* j, const SpjDeviceWkb* column) {
  return guarded(j->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(j->rt->device_id));
    j->host.clear();
    SPJ_CUDA(cudaDeviceSynchronize());  // the caller's column is complete
    j->engine->build(device_column(column));
  });
}

// The distance column for this probe (nullptr: the call's one distance).
static const double* probe_distances(SpjJoin* j, int32_t predicate, int64_t rows) {
  if (predicate != SPJ_PREDICATE_DWITHIN || !j->has_dist) return nullptr;
  SPJ_CHECK((uint64_t)rows == j->dist_n,
            "distance column has " + std::to_string(j->dist_n) + " rows, the probe column " +
                std::to_string(rows));
  return j->dist.as<double>();
}

extern "C" int SpjJoinSetProbeDistances(SpjJoin* j, const double* distances, uint64_t n,
                                        int32_t device) {
  return guarded(j->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(j->rt->device_id));
    j->has_dist = false;
    j->dist_n = 0;
    if (distances == nullptr) return;
    cudaStream_t s = j->ws->stream;
    j->dist.reserve((n + 1) * sizeof(double), s);
    if (n)
      SPJ_CUDA(cudaMemcpyAsync(j->dist.get(), distances, n * sizeof(double),
                               device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    j->dist_n = n;
    j->has_dist = true;
  });
}

static HostWkbColumn host_column(const SpjHostWkb* c) {
  SPJ_CHECK(c != nullptr, "null column");
  SPJ_CHECK(c->length >= 0 && (c->length == 0 || (c->offsets && c->data)), "null buffers");
  HostWkbColumn h;
  h.n = c->length;
  h.offsets = c->offsets;
  h.offsets64 = c->offsets_are_64bit != 0;
  h.data = c->data;
  h.validity = c->validity;
  h.validity_offset = c->validity_offset;
  return h;
}

extern "C" int SpjJoinPartitioned(SpjJoin* j, const SpjHostWkb* build, const SpjHostWkb* probe,
                                  int32_t predicate, double distance,
                                  const SpjPartitionOptions* options,
                                  int (*callback)(const uint32_t*, const uint32_t*, uint64_t,
                                                  void*),
                                  void* user_data, SpjPartitionStats* stats) {
  int cb_status = 0;
  int rc = guarded(j->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(j->rt->device_id));
    SPJ_CHECK(callback != nullptr, "null callback");
    const HostWkbColumn hb = host_column(build), hp = host_column(probe);
    PartitionOptions o;
    if (options) {
      o.num_partitions = options->num_partitions;
      o.sample_rows = options->sample_rows;
      o.build_budget_bytes = options->build_budget_bytes;
      o.seed = options->seed;
      o.host_gather = options->host_gather != 0;
      o.record_layout = options->record_layout != 0;
    }
    const double* dr = probe_distances(j, predicate, hp.n);
    j->host.clear();
    PartitionStats st;
    cb_status = run_partitioned(
        *j->engine, *j->ws, hb, hp, predicate, distance, dr, o, &st, &j->layout,
        [&](const uint32_t* b, const uint32_t* p, uint64_t n) {
          return callback(b, p, n, user_data);
        });
    if (stats) {
      stats->partitions = st.partitions;
      stats->passes = st.passes;
      stats->build_rows_max = st.build_rows_max;
      stats->probe_rows_multi = st.probe_rows_multi;
      stats->probe_rows_none = st.probe_rows_none;
      stats->probe_rows_probed = st.probe_rows_probed;
      stats->pairs = st.pairs;
      stats->ms_boxes = st.ms_boxes;
      stats->ms_partition = st.ms_partition;
      stats->ms_passes = st.ms_passes;
      stats->direct_host_reads = st.direct_host_reads ? 1 : 0;
    }
  });
  return rc ? rc : cb_status;
}

extern "C" int SpjJoinPartitionLayout(SpjJoin* j, uint32_t* counts, float* extent, float* leaves,
                                      float* bounds, float* samples, uint32_t* build_part,
                                      uint32_t* probe_part) {
  return guarded(j->last_error, [&] {
    SPJ_CHECK(counts != nullptr, "null counts");
    const PartitionLayout& L = j->layout;
    counts[0] = (uint32_t)L.leaves.size();
    counts[1] = (uint32_t)L.samples.size();
    counts[2] = L.max_items;
    counts[3] = L.max_levels;
    if (extent) memcpy(extent, &L.extent, 16);
    if (leaves && !L.leaves.empty()) memcpy(leaves, L.leaves.data(), 16 * L.leaves.size());
    if (bounds && !L.bounds.empty()) memcpy(bounds, L.bounds.data(), 16 * L.bounds.size());
    if (samples && !L.samples.empty()) memcpy(samples, L.samples.data(), 16 * L.samples.size());
    if (build_part && !L.build_part.empty())
      memcpy(build_part, L.build_part.data(), 4 * L.build_part.size());
    if (probe_part && !L.probe_part.empty())
      memcpy(probe_part, L.probe_part.data(), 4 * L.probe_part.size());
  });
}

extern "C" int SpjJoinProbeDevice(SpjJoin* j, const SpjDeviceWkb* column, int32_t predicate,
                                  double distance, uint32_t probe_base, const uint32_t** d_build,
                                  const uint32_t** d_probe, uint64_t* n_pairs) {
  return guarded(j->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(j->rt->device_id));
    SPJ_CHECK(d_build && d_probe && n_pairs, "null outputs");
    SPJ_CHECK(column != nullptr, "null column");
    const double* dr = probe_distances(j, predicate, column->length);
    *n_pairs = j->engine->probe(*j->ws, device_column(column), predicate, distance, probe_base,
                                d_build, d_probe, dr);
  });
}

extern "C" int SpjJoinProbeArrow(SpjJoin* j, const ArrowSchema* schema, const ArrowArray* array,
                                 int32_t predicate, double distance, uint32_t probe_base,
                                 int (*callback)(const uint32_t*, const uint32_t*, uint64_t,
                                                 void*),
                                 void* user_data) {
  int cb_status = 0;
  int rc = guarded(j->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(j->rt->device_id));
    SPJ_CHECK(callback != nullptr, "null callback");
    HostWkbColumn hc = parse_arrow(schema, array);
    const double* dr = probe_distances(j, predicate, hc.n);
    uint64_t bytes = 0;
    WkbDeviceColumn dc = stage_column(*j->ws, hc, &bytes);
    const uint32_t *db, *dp;
    uint64_t m = j->engine->probe(*j->ws, dc, predicate, distance, probe_base, &db, &dp, dr);
    j->hb.resize(m);
    j->hp.resize(m);
    if (m) copy_pairs_to_host(j, db, dp, m, j->hb.data(), j->hp.data());
    SPJ_CUDA(cudaStreamSynchronize(j->ws->stream));
    cb_status = callback(j->hb.data(), j->hp.data(), m, user_data);
  });
  return rc ? rc : cb_status;
}

extern "C" int SpjJoinProbeHost(SpjJoin* j, int64_t length, const void* offsets,
                                int32_t offsets_are_64bit, const uint8_t* data,
                                const uint8_t* validity, int32_t predicate, double distance,
                                uint32_t probe_base, uint32_t* out_build, uint32_t* out_probe,
                                uint64_t capacity, uint64_t* n_pairs) {
  int rc = 0;
  int g = guarded(j->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(j->rt->device_id));
    SPJ_CHECK(n_pairs != nullptr, "null n_pairs");
    HostWkbColumn hc;
    hc.n = length;
    hc.offsets = offsets;
    hc.offsets64 = offsets_are_64bit != 0;
    hc.data = data;
    hc.validity = validity;
    const double* dr = probe_distances(j, predicate, length);
    // (a distance column is probed in one call: its rows stay aligned)
    const int nslices = dr ? 1 : host_slices(hc, j->engine->config().host_slices);
    if (nslices > 1) {
      const uint64_t m = probe_host_sliced(j, hc, nslices, predicate, distance, probe_base,
                                           out_build, out_probe, capacity);
      *n_pairs = m;
      if (m > capacity) rc = ENOSPC;
      return;
    }
    uint64_t bytes = 0;
    WkbDeviceColumn dc = stage_column(*j->ws, hc, &bytes);
    const uint32_t *db, *dp;
    uint64_t m = j->engine->probe(*j->ws, dc, predicate, distance, probe_base, &db, &dp, dr);
    *n_pairs = m;
    if (m > capacity) {
      rc = ENOSPC;
      return;
    }
    if (m) {
      SPJ_CHECK(out_build && out_probe, "null output buffers");
      copy_pairs_to_host(j, db, dp, m, out_build, out_probe);
    }
    SPJ_CUDA(cudaStreamSynchronize(j->ws->stream));
  });
  if (g) return g;
  if (rc) {
    // (set after guarded(), which clears the message of a call that returns)
    j->last_error = "output capacity too small: need " + std::to_string(*n_pairs) + " pairs";
    return rc;
  }
  return 0;
}

extern "C" void* SpjJoinStream(SpjJoin* j) { return (void*)j->ws->stream; }

extern "C" int SpjJoinGetStats(SpjJoin* j, SpjJoinStats* out) {
  return guarded(j->last_error, [&] {
    SPJ_CHECK(out != nullptr, "null stats");
    JoinStats s = j->engine->stats();
    out->ms_decode = s.ms_decode;
    out->ms_filter = s.ms_filter;
    out->ms_refine = s.ms_refine;
    out->ms_compact = s.ms_compact;
    out->calls = s.calls;
    out->probe_rows = s.probe_rows;
    out->candidates = s.candidates;
    out->results = s.results;
    out->escalations = s.escalations;
    out->pairs_evaluated = s.pairs_evaluated;
    out->kernel_launches = s.kernel_launches;
    out->probe_bytes = s.probe_bytes;
    const DeviceGeoms& g = j->engine->build_geoms();
    out->build_rows = g.n;
    out->build_vertices = g.nverts;
    out->build_device_bytes = g.device_bytes() + j->engine->lbvh().device_bytes();
  });
}

extern "C" int SpjJoinResetStats(SpjJoin* j) {
  return guarded(j->last_error, [&] { j->engine->reset_stats(); });
}

// =============================================================================
// exported: SpjStream

struct SpjStream {
  SpjJoin* join = nullptr;
  std::unique_ptr<StreamJoin> s;
  std::string last_error;
};

extern "C" int SpjStreamCreate(SpjJoin* j, SpjStream** out) {
  if (!j || !out) return EINVAL;
  return guarded(j->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(j->rt->device_id));
    SPJ_CHECK(j->engine->built(), "stream on a join whose build side is not finished");
    auto st = std::make_unique<SpjStream>();
    st->join = j;
    st->s = std::make_unique<StreamJoin>(*j->engine);
    *out = st.release();
  });
}

extern "C" void SpjStreamRelease(SpjStream* st) {
  if (!st) return;
  cudaSetDevice(st->join->rt->device_id);
  delete st;
}

extern "C" const char* SpjStreamLastError(SpjStream* st) { return st->last_error.c_str(); }

extern "C" int SpjStreamSetBatches(SpjStream* st, const SpjDeviceWkb* batches, int32_t n) {
  return guarded(st->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(st->join->rt->device_id));
    SPJ_CHECK(n >= 0 && (n == 0 || batches != nullptr), "bad batch list");
    std::vector<WkbDeviceColumn> cols;
    for (int32_t i = 0; i < n; i++) cols.push_back(device_column(&batches[i]));
    st->s->set_batches(cols);
  });
}

extern "C" int SpjStreamRun(SpjStream* st, int32_t predicate, const uint32_t** d_build,
                            const uint32_t** d_probe, uint64_t* n_pairs) {
  return guarded(st->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(st->join->rt->device_id));
    SPJ_CHECK(d_build && d_probe && n_pairs, "null outputs");
    *n_pairs = st->s->run(predicate, d_build, d_probe);
  });
}

extern "C" int SpjStreamSetParams(SpjStream* st, int32_t block, uint32_t chunk_rows,
                                  uint32_t leaf_size) {
  return guarded(st->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(st->join->rt->device_id));
    st->s->set_params(StreamParams{block, chunk_rows, leaf_size});
  });
}

extern "C" int SpjStreamAutotune(SpjStream* st, int32_t predicate, const char* cache_path,
                                 int32_t* block, uint32_t* chunk_rows, uint32_t* leaf_size) {
  return guarded(st->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(st->join->rt->device_id));
    StreamParams p = st->s->autotune(predicate, cache_path ? std::string(cache_path) : "");
    if (block) *block = p.block;
    if (chunk_rows) *chunk_rows = p.chunk_rows;
    if (leaf_size) *leaf_size = p.leaf_size;
  });
}

extern "C" int SpjStreamGetStats(SpjStream* st, double* ms_last, uint64_t* escalations,
                                 uint64_t* launches) {
  return guarded(st->last_error, [&] {
    const StreamStats& s = st->s->stats();
    if (ms_last) *ms_last = s.ms_last;
    if (escalations) *escalations = s.escalations;
    if (launches) *launches = s.launches_per_replay;
  });
}

extern "C" void* SpjStreamCudaStream(SpjStream* st) { return (void*)st->s->stream(); }

// =============================================================================
// exported: SpjLearned

struct SpjLearned {
  RuntimeData* rt = nullptr;
  uint32_t leaves = 4096, window = 4096;
  bool trained = true;
  double ms_build = 0;
  uint64_t decode_launches = 0;  // probe-column decodes of queries
  std::unique_ptr<JoinEngine> engine;  // decodes the build points, owns the LBVH
  std::unique_ptr<Workspace> ws;
  std::unique_ptr<LearnedIndex> index;
  DevBuf out_b, out_p;
  std::string last_error;
  ~SpjLearned() {
    if (ws) cudaStreamSynchronize(ws->stream);
    out_b.release();
    out_p.release();
    index.reset();
  }
};

extern "C" int SpjLearnedCreate(const SpjLearnedConfig* config, SpjLearned** out) {
  try {
    SPJ_CHECK(config && out, "null config or output");
    RuntimeData* rt = runtime_of(config->runtime);
    SPJ_CUDA(cudaSetDevice(rt->device_id));
    auto li = std::make_unique<SpjLearned>();
    li->rt = rt;
    if (config->leaves) li->leaves = config->leaves;
    if (config->window) li->window = config->window;
    SPJ_CHECK(li->leaves <= 65535, "leaves must be at most 65535");
    // the fallback LBVH serves range boxes and lookups: 4 points per leaf
    // (16, the default for point build sides, suits distance joins)
    EngineConfig lc;
    lc.leaf_size = 4;
    li->engine = std::make_unique<JoinEngine>(rt->device_id, lc);
    li->ws = std::make_unique<Workspace>();
    *out = li.release();
    return 0;
  } catch (const std::exception& e) {
    fprintf(stderr, "SpjLearnedCreate: %s\n", e.what());
    return EINVAL;
  }
}

extern "C" void SpjLearnedRelease(SpjLearned* li) {
  if (!li) return;
  cudaSetDevice(li->rt->device_id);
  delete li;
}

extern "C" const char* SpjLearnedLastError(SpjLearned* li) { return li->last_error.c_str(); }

extern "C" int SpjLearnedBuildDevice(SpjLearned* li, const SpjDeviceWkb* points) {
  return guarded(li->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(li->rt->device_id));
    SPJ_CUDA(cudaDeviceSynchronize());  // the caller's column is complete
    cudaEvent_t e0, e1;
    SPJ_CUDA(cudaEventCreate(&e0));
    SPJ_CUDA(cudaEventCreate(&e1));
    SPJ_CUDA(cudaEventRecord(e0, li->ws->stream));
    li->engine->build(device_column(points));
    li->index = std::make_unique<LearnedIndex>(li->leaves, li->window);
    li->index->build(li->engine->build_geoms(), li->engine->lbvh(), li->ws->stream);
    SPJ_CUDA(cudaEventRecord(e1, li->ws->stream));
    SPJ_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    li->ms_build = ms;
    li->trained = true;
  });
}

extern "C" int SpjLearnedSetTrained(SpjLearned* li, int32_t trained) {
  return guarded(li->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(li->rt->device_id));
    SPJ_CHECK(li->index != nullptr, "learned index is not built");
    li->index->train(trained != 0, li->ws->stream);
    li->trained = trained != 0;
  });
}

extern "C" int SpjLearnedQueryDevice(SpjLearned* li, const SpjDeviceWkb* probe, int32_t predicate,
                                     uint32_t probe_base, const uint32_t** d_build,
                                     const uint32_t** d_probe, uint64_t* n_pairs) {
  return guarded(li->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(li->rt->device_id));
    SPJ_CHECK(li->index != nullptr, "learned index is not built");
    SPJ_CHECK(d_build && d_probe && n_pairs, "null outputs");
    SPJ_CHECK(predicate >= 0 && predicate <= 7, "relation predicates only");
    Workspace& ws = *li->ws;
    const bool hint = ws.last_probe_points;
    decode_wkb(device_column(probe), ws.probe, ws.dsc, hint, ws.stream);
    // the decode's kernels: the point kernel alone, or the general path
    li->decode_launches += ws.probe.all_points && hint ? 1 : 17;
    ws.last_probe_points = ws.probe.all_points;
    *n_pairs = li->index->query(ws.probe.view(), probe_base, predicate, li->out_b, li->out_p,
                                ws.stream);
    *d_build = li->out_b.as<uint32_t>();
    *d_probe = li->out_p.as<uint32_t>();
  });
}

extern "C" int SpjLearnedSetWindow(SpjLearned* li, uint32_t window) {
  return guarded(li->last_error, [&] {
    SPJ_CHECK(li->index != nullptr, "learned index is not built");
    SPJ_CHECK(window >= 1, "window must be positive");
    li->index->set_window(window);
    li->window = window;
  });
}

extern "C" int SpjLearnedAutotuneWindow(SpjLearned* li, const SpjDeviceWkb* samples,
                                        uint32_t n_samples, int32_t predicate,
                                        uint32_t* window) {
  return guarded(li->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(li->rt->device_id));
    SPJ_CHECK(li->index != nullptr, "learned index is not built");
    SPJ_CHECK(samples && n_samples > 0 && window, "no samples or null output");
    SPJ_CHECK(predicate >= 0 && predicate <= 7, "relation predicates only");
    Workspace& ws = *li->ws;
    std::vector<uint32_t> cand;
    for (uint32_t w = 1u << 10; w <= (1u << 17); w <<= 1) cand.push_back(w);
    const uint32_t mx = li->index->stats().max_err;
    if (mx > cand.back()) cand.push_back(mx);
    cudaEvent_t e0, e1;
    SPJ_CUDA(cudaEventCreate(&e0));
    SPJ_CUDA(cudaEventCreate(&e1));
    const uint32_t before = li->index->window(), before_box = li->index->window_box();
    // the query time of all samples with windows (w lookups, wb range cells)
    auto timed = [&](uint32_t w, uint32_t wb) {
      li->index->set_windows(w, wb);
      float t_min = INFINITY;
      for (int rep = 0; rep < 2; rep++) {
        float t = 0;
        for (uint32_t k = 0; k < n_samples; k++) {
          decode_wkb(device_column(&samples[k]), ws.probe, ws.dsc, ws.last_probe_points,
                     ws.stream);
          ws.last_probe_points = ws.probe.all_points;
          SPJ_CUDA(cudaEventRecord(e0, ws.stream));
          li->index->query(ws.probe.view(), 0, predicate, li->out_b, li->out_p, ws.stream);
          SPJ_CUDA(cudaEventRecord(e1, ws.stream));
          SPJ_CUDA(cudaEventSynchronize(e1));
          float ms = 0;
          cudaEventElapsedTime(&ms, e0, e1);
          t += ms;
        }
        t_min = std::min(t_min, t);
      }
      return t_min;
    };
    // lookup rows and range rows respond to their own window: tune the range
    // window with lookups on the model throughout, then the lookup window
    uint32_t best_box = before_box, best = before;
    try {
      float best_ms = INFINITY;
      for (uint32_t wb : cand) {
        const float t = timed(cand.back(), wb);
        if (t < best_ms) {
          best_ms = t;
          best_box = wb;
        }
      }
      best_ms = INFINITY;
      for (uint32_t w : cand) {
        const float t = timed(w, best_box);
        if (t < best_ms) {
          best_ms = t;
          best = w;
        }
      }
    } catch (...) {
      li->index->set_windows(before, before_box);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    li->index->set_windows(best, best_box);
    li->window = best;
    *window = best;
  });
}

extern "C" int SpjLearnedLossAndGrad(SpjLearned* li, const double* a, const double* b,
                                     double* loss, double* grad_a, double* grad_b) {
  return guarded(li->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(li->rt->device_id));
    SPJ_CHECK(li->index != nullptr, "learned index is not built");
    std::vector<double> va(a, a + li->leaves), vb(b, b + li->leaves), l, ga, gb;
    li->index->loss_and_grad(va, vb, l, ga, gb, li->ws->stream);
    std::copy(l.begin(), l.end(), loss);
    std::copy(ga.begin(), ga.end(), grad_a);
    std::copy(gb.begin(), gb.end(), grad_b);
  });
}

extern "C" int SpjLearnedExport(SpjLearned* li, uint32_t* keys, uint32_t* leaf_start,
                                uint32_t* leaf_kc, double* a, double* b, uint32_t* err) {
  return guarded(li->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(li->rt->device_id));
    SPJ_CHECK(li->index != nullptr, "learned index is not built");
    std::vector<uint32_t> k, s, kc, e;
    std::vector<double> va, vb;
    li->index->export_model(k, s, kc, va, vb, e, li->ws->stream);
    if (keys) std::copy(k.begin(), k.end(), keys);
    if (leaf_start) std::copy(s.begin(), s.end(), leaf_start);
    if (leaf_kc) std::copy(kc.begin(), kc.end(), leaf_kc);
    if (a) std::copy(va.begin(), va.end(), a);
    if (b) std::copy(vb.begin(), vb.end(), b);
    if (err) std::copy(e.begin(), e.end(), err);
  });
}

extern "C" int SpjLearnedGetStats(SpjLearned* li, SpjLearnedStats* out) {
  return guarded(li->last_error, [&] {
    SPJ_CHECK(out != nullptr, "null stats");
    SPJ_CHECK(li->index != nullptr, "learned index is not built");
    const LearnedStats& s = li->index->stats();
    out->points = s.points;
    out->lookups = s.lookups;
    out->window_misses = s.window_misses;
    out->lbvh_fallbacks = s.lbvh_fallbacks;
    out->search_steps = s.search_steps;
    out->leaves = s.leaves;
    out->max_err = s.max_err;
    out->leaves_over_window = s.leaves_over_window;
    out->trained = li->trained ? 1 : 0;
    out->root_shift = s.root_shift;
    out->root_entries = s.root_entries;
    out->mean_err = s.mean_err;
    out->grad_norm_after = s.grad_norm_after;
    out->ms_build = li->ms_build;
    out->ranges = s.ranges;
    out->ms_order = s.ms_order;
    out->ms_ranges = s.ms_ranges;
    out->ms_eval = s.ms_eval;
    out->window = li->index->window();
    out->window_box = li->index->window_box();
    out->kernel_launches = s.kernel_launches + li->decode_launches;
  });
}

extern "C" void* SpjLearnedStream(SpjLearned* li) { return (void*)li->ws->stream; }

// =============================================================================
// exported: SpjKnn

struct SpjKnn {
  RuntimeData* rt = nullptr;
  std::unique_ptr<KnnIndex> index;
  std::unique_ptr<Workspace> ws;  // staging and decode of WKB probe columns
  std::string last_error;
};

extern "C" int SpjKnnCreate(const SpjKnnConfig* config, SpjKnn** out) {
  try {
    SPJ_CHECK(config && out, "null config or output");
    RuntimeData* rt = runtime_of(config->runtime);
    SPJ_CUDA(cudaSetDevice(rt->device_id));
    auto k = std::make_unique<SpjKnn>();
    k->rt = rt;
    k->index = std::make_unique<KnnIndex>(config->leaf_size ? config->leaf_size : 8,
                                          config->refine_form);
    *out = k.release();
    return 0;
  } catch (const std::exception& e) {
    fprintf(stderr, "SpjKnnCreate: %s\n", e.what());
    return EINVAL;
  }
}

extern "C" void SpjKnnRelease(SpjKnn* k) {
  if (!k) return;
  cudaSetDevice(k->rt->device_id);
  delete k;
}

extern "C" const char* SpjKnnLastError(SpjKnn* k) { return k->last_error.c_str(); }

extern "C" int SpjKnnBuild(SpjKnn* k, const double* xy, uint64_t n) {
  return guarded(k->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(k->rt->device_id));
    k->index->build(xy, n);
  });
}

extern "C" int SpjKnnQuery(SpjKnn* k, const double* probe_xy, uint64_t n, uint32_t kk,
                           uint32_t* out_idx, double* out_dist, int32_t device) {
  return guarded(k->last_error, [&] {
    SPJ_CUDA(cudaSetDevice(k->rt->device_id));
    k->index->query(probe_xy, n, kk, out_idx, out_dist, device != 0);
  });
}

extern "C" int SpjKnnQueryTies(SpjKnn* k, const double* probe_xy, uint64_t n, uint32_t kk,
                               int32_t include_tie_breakers, int32_t device, uint64_t* offsets,
                               uint32_t* out_idx, double* out_dist, uint64_t capacity,
                               uint64_t* total) {
  int rc = guarded(k->last_error, [&] {
    SPJ_CHECK(total != nullptr, "null total");
    SPJ_CUDA(cudaSetDevice(k->rt->device_id));
    *total = k->index->query_ties(probe_xy, n, kk, device != 0, offsets, out_idx, out_dist,
                                  capacity, include_tie_breakers != 0);
  });
  if (rc == 0 && *total > capacity) {
    k->last_error = "output capacity " + std::to_string(capacity) + " < " +
                    std::to_string(*total) + " results";
    return ENOSPC;
  }
  return rc;
}

extern "C" int SpjKnnQueryArrow(SpjKnn* k, const ArrowSchema* schema, const ArrowArray* array,
                                uint32_t kk, int32_t include_tie_breakers, uint64_t* offsets,
                                uint32_t* out_idx, double* out_dist, uint64_t capacity,
                                uint64_t* total) {
  int rc = guarded(k->last_error, [&] {
    SPJ_CHECK(total != nullptr, "null total");
    SPJ_CUDA(cudaSetDevice(k->rt->device_id));
    if (!k->ws) k->ws = std::make_unique<Workspace>();
    Workspace& ws = *k->ws;
    const HostWkbColumn col = parse_arrow(schema, array);
    uint64_t bytes = 0;
    const WkbDeviceColumn d = stage_column(ws, col, &bytes);
    decode_wkb(d, ws.probe, ws.dsc, true, ws.stream);
    SPJ_CHECK(ws.probe.all_points,
              "KNN probe rows must be points (empty and null rows give no results)");
    SPJ_CUDA(cudaStreamSynchronize(ws.stream));
    // empty and null rows decode to NaN points, which get no results
    *total = k->index->query_ties(reinterpret_cast<const double*>(ws.probe.pt.get()),
                                  (uint64_t)col.n, kk, true, offsets, out_idx, out_dist, capacity,
                                  include_tie_breakers != 0);
  });
  if (rc == 0 && *total > capacity) {
    k->last_error = "output capacity " + std::to_string(capacity) + " < " +
                    std::to_string(*total) + " results";
    return ENOSPC;
  }
  return rc;
}

extern "C" void* SpjKnnStream(SpjKnn* k) { return (void*)k->index->stream(); }

extern "C" int SpjKnnGetStats(SpjKnn* k, uint64_t* queries, uint64_t* exact_evals,
                              uint64_t* redone) {
  return guarded(k->last_error, [&] {
    SPJ_CHECK(queries && exact_evals && redone, "null output");
    *queries = k->index->queries();
    *exact_evals = k->index->exact_evals();
    *redone = k->index->redone();
  });
}

extern "C" int SpjHostRegister(void* ptr, uint64_t bytes) {
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  return e == cudaSuccess ? 0 : EINVAL;
}

extern "C" int SpjHostUnregister(void* ptr) {
  cudaError_t e = cudaHostUnregister(ptr);
  return e == cudaSuccess ? 0 : EINVAL;
}

extern "C" const char* SpjVersion(void) { return "spj-gb300 0.1.0 (sm_103a)"; }

namespace spj {
std::atomic<uint64_t> g_allocations{0};
}  // namespace spj

extern "C" uint64_t SpjAllocationCount(void) {
  return spj::g_allocations.load(std::memory_order_relaxed);
}
