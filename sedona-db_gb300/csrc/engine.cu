// engine.cu — build / probe orchestration on one stream per caller.
#include "engine.cuh"
#include "predicates.cuh"
#include "prims.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace spj {

Workspace::Workspace() {
  SPJ_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  own_stream = true;
  for (auto& e : ev) SPJ_CUDA(cudaEventCreate(&e));
}

Workspace::~Workspace() {
  if (stream) cudaStreamSynchronize(stream);
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  // DevBufs free on their own streams; make sure those frees are issued
  // before the stream goes away
  probe = DeviceGeoms();
  dsc = DecodeScratch();
  psc = ProbeScratch();
  boxes_tmp.release();
  cand_build.release();
  cand_probe.release();
  flags.release();
  out_build.release();
  out_probe.release();
  scan_tmp.release();
  slots.release();
  arena.release();
  rqueue.release();
  status.release();
  wkb_data.release();
  wkb_offsets.release();
  wkb_validity.release();
  if (stream) {
    cudaStreamSynchronize(stream);
    if (own_stream) cudaStreamDestroy(stream);
  }
}

JoinEngine::JoinEngine(int device, EngineConfig cfg) : device_(device), cfg_(cfg) {
  SPJ_CUDA(cudaStreamCreateWithFlags(&bs_, cudaStreamNonBlocking));
}

JoinEngine::~JoinEngine() {
  // the build-side buffers free on bs_: release them before bs_ goes away
  cudaStreamSynchronize(bs_);
  bg_ = DeviceGeoms();
  bsc_ = DecodeScratch();
  bvh_ = Lbvh();
  bsplit_ = PointSplit();
  cudaStreamSynchronize(bs_);
  cudaStreamDestroy(bs_);
}

void JoinEngine::build(const WkbDeviceColumn& col) {
  built_ = false;
  cudaStream_t s = bs_;
  decode_wkb(col, bg_, bsc_, false, s);
  if (bg_.nrings > 0) build_band_index(bg_, bsc_, s);
  bg_.has_grid = false;
  if (bg_.nrings > 0 && cfg_.cell_grid) build_cell_grid(bg_, bsc_, s);
  bg_.grid_rings = cfg_.grid_rings;
  if (bg_.nrings > 0) build_ring_flags(bg_, s);
  const uint32_t leaf = cfg_.leaf_size ? cfg_.leaf_size : (bg_.all_points ? 16u : 4u);
  build_lbvh(bg_.box.as<float4>(), bg_.n, leaf, bvh_, s);
  split_points();
  SPJ_CUDA(cudaStreamSynchronize(s));
  built_ = true;
}

void JoinEngine::split_points() {
  bsplit_.n = 0;
  if (cfg_.fuse_dwithin && bg_.all_points && bvh_.nprims > 0) build_point_split(bg_.pt.as<double2>(), bg_.n, bvh_, bsplit_, bs_);
}

void JoinEngine::reindex(uint32_t leaf_size) {
  SPJ_CHECK(built_, "reindex before the build side was finished");
  cfg_.leaf_size = leaf_size;
  build_lbvh(bg_.box.as<float4>(), bg_.n, leaf_size, bvh_, bs_);
  split_points();
  SPJ_CUDA(cudaStreamSynchronize(bs_));
}

static inline float ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

uint64_t JoinEngine::probe(Workspace& ws, const WkbDeviceColumn& col, int predicate,
                           double distance, uint32_t probe_base, const uint32_t** d_build,
                           const uint32_t** d_probe, const double* d_row) {
  SPJ_CHECK(built_, "probe called before the build side was finished");
  SPJ_CHECK(predicate == kPredDWithin || (predicate >= 0 && predicate <= 7),
            "unknown predicate code " + std::to_string(predicate));
  SPJ_CHECK(col.n >= 0 && (uint64_t)col.n + probe_base <= 0xFFFFFFFFull,
            "probe row ids exceed 32 bits");
  if (predicate == kPredDWithin && d_row == nullptr)
    SPJ_CHECK(distance >= 0 && !std::isnan(distance),
              "ST_DWithin distance must be a non-negative number");
  cudaStream_t s = ws.stream;
  const bool prof = cfg_.profile;
  uint64_t launches = 0;
  if (prof) SPJ_CUDA(cudaEventRecord(ws.ev[0], s));

  const bool hint = ws.last_probe_points;
  decode_wkb(col, ws.probe, ws.dsc, hint, s);
  launches += ws.probe.all_points && hint ? 1 : 17;
  ws.last_probe_points = ws.probe.all_points;
  const uint32_t n = ws.probe.n;
  if (prof) SPJ_CUDA(cudaEventRecord(ws.ev[1], s));

  const float4* boxes = ws.probe.box.as<float4>();
  if (predicate == kPredDWithin) {
    ws.boxes_tmp.reserve(((size_t)n + 1) * sizeof(float4), s);
    expand_boxes(ws.probe.view(), distance, d_row, ws.boxes_tmp.as<float4>(), s);
    boxes = ws.boxes_tmp.as<float4>();
    launches++;
  }
  const LbvhView tv = bvh_.view();
  const uint32_t* order = nullptr;
  if (cfg_.probe_order > 0 || (cfg_.probe_order == 0 && n >= kOrderMinRows)) {
    order = probe_order(tv, boxes, n, ws.psc, s);
    if (order) launches += 21;  // keys + 4 radix passes (histogram, 3-kernel scan, scatter)
  }
  if (predicate == kPredDWithin && cfg_.fuse_dwithin && cfg_.refine_form == kFastF32 &&
      ws.probe.all_points && bsplit_.n == bvh_.nprims && bvh_.nprims > 0) {
    // point build and probe sides: the distance test runs inside the
    // traversal, no candidate pairs are materialized
    reset_status(ws.status, s);
    ws.psc.counts.reserve(((size_t)n + 1) * 4, s);
    ws.psc.offsets.reserve(((size_t)n + 1) * 8, s);
    const double2* ppt = ws.probe.pt.as<double2>();
    // result slots per probe, kept by the counting pass (bounded memory)
    uint32_t K = cfg_.dwithin_slots;
    while (K > 0 && (uint64_t)n * K * 4 > kMaxSlotBytes) K >>= 1;
    uint32_t* slots = nullptr;
    DwithinArena arena;
    if (K > 0) {
      ws.slots.reserve((size_t)n * K * 4 + 16, s);
      slots = ws.slots.as<uint32_t>();
      if (cfg_.dwithin_arena == 1 || (cfg_.dwithin_arena == 2 && order == nullptr)) {
        // 16 B cursor, n heads, then chunks of the slots' size in total
        const uint64_t chunks =
            std::max<uint64_t>(1024, (uint64_t)n * K / kArenaChunkWords);
        const size_t head_bytes = ((size_t)n * 4 + 127) & ~(size_t)127;
        ws.arena.reserve(128 + head_bytes + chunks * kArenaChunkWords * 4, s);
        uint8_t* base = ws.arena.as<uint8_t>();
        arena.cursor = reinterpret_cast<unsigned long long*>(base);
        arena.head = reinterpret_cast<uint32_t*>(base + 128);
        arena.words = reinterpret_cast<uint32_t*>(base + 128 + head_bytes);
        arena.chunks = (uint32_t)std::min<uint64_t>(chunks, 0xFFFFFFF0ull);
        SPJ_CUDA(cudaMemsetAsync(arena.cursor, 0, 8, s));
      }
    }
    dwithin_count(tv, bsplit_, boxes, ppt, n, distance, order, ws.psc.counts.as<uint32_t>(),
                  ws.status.as<DeviceStatus>(), s, slots, K, arena, d_row);
    scan_u32_u64(ws.psc.counts.as<uint32_t>(), ws.psc.offsets.as<uint64_t>(), n, ws.psc.tmp, s);
    uint64_t total = 0;
    DeviceStatus hst;
    SPJ_CUDA(cudaMemcpyAsync(&total, ws.psc.offsets.as<uint64_t>() + n, 8,
                             cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaMemcpyAsync(&hst, ws.status.get(), sizeof hst, cudaMemcpyDeviceToHost, s));
    SPJ_CUDA(cudaStreamSynchronize(s));
    check_traversal(tv, s);
    if (prof) SPJ_CUDA(cudaEventRecord(ws.ev[2], s));
    ws.out_build.reserve((total + 1) * 4, s);
    ws.out_probe.reserve((total + 1) * 4, s);
    dwithin_scatter(tv, bsplit_, boxes, ppt, n, distance, order, ws.psc.offsets.as<uint64_t>(),
                    probe_base, ws.out_build.as<uint32_t>(), ws.out_probe.as<uint32_t>(), total,
                    s, ws.psc.counts.as<uint32_t>(), slots, K, arena, d_row);
    launches += 5 + (arena.words ? 1 : 0);
    if (prof) {
      SPJ_CUDA(cudaEventRecord(ws.ev[3], s));
      SPJ_CUDA(cudaEventRecord(ws.ev[4], s));
    }
    SPJ_CUDA(cudaStreamSynchronize(s));
    {
      std::lock_guard<std::mutex> lk(stats_mu_);
      stats_.calls++;
      stats_.probe_rows += n;
      stats_.candidates += hst.counters[1];
      stats_.results += total;
      stats_.escalations += hst.counters[0];
      stats_.pairs_evaluated += hst.counters[1];
      stats_.kernel_launches += launches;
      stats_.probe_bytes +=
          (uint64_t)col.data_len + (uint64_t)(col.n + 1) * (col.offsets64 ? 8 : 4);
      if (prof) {
        stats_.ms_decode += ev_ms(ws.ev[0], ws.ev[1]);
        stats_.ms_filter += ev_ms(ws.ev[1], ws.ev[2]);
        stats_.ms_refine += ev_ms(ws.ev[2], ws.ev[3]);
        stats_.ms_compact += ev_ms(ws.ev[3], ws.ev[4]);
      }
    }
    *d_build = ws.out_build.as<uint32_t>();
    *d_probe = ws.out_probe.as<uint32_t>();
    return total;
  }
  const uint64_t m = probe_count(tv, boxes, n, ws.psc, s, order);  // syncs
  SPJ_CHECK(m < (1ull << 34), "candidate pair count too large");
  ws.cand_build.reserve((m + 1) * 4, s);
  ws.cand_probe.reserve((m + 1) * 4, s);
  probe_scatter(tv, boxes, n, ws.psc, probe_base, ws.cand_build.as<uint32_t>(),
                ws.cand_probe.as<uint32_t>(), s, order);
  launches += 5;
  const uint32_t* cperm = nullptr;
  bool build_major = false;
  if (cfg_.candidate_order == 2 ||
      (cfg_.candidate_order == 3 && predicate != kPredDWithin && !bg_.all_points &&
       m >= kBuildMajorMin)) {
    // (auto, 3: the order pays when consecutive pairs re-read one build
    // geometry's vertices and band index from cache; a point build row is
    // 16 bytes with nothing to re-read, distance candidates are cheap to
    // test, and small candidate sets do not repay the sort)
    cperm = build_major_order(ws.cand_build.as<uint32_t>(), ws.cand_probe.as<uint32_t>(), m,
                              probe_base, bg_.n, order, n,
                              order_tile_count(cfg_.order_tiles, m), ws.psc, s);
    if (cperm) {
      // Morton list with its build rows (counts gather, scan, k_cand_perm) and
      // one radix pass per 8 bits of the build row; else rank, keys and 4 passes
      int bits = 1;
      while (bits < 32 && (bg_.n - 1) >> bits) bits++;
      launches += order && bits <= 24 ? 5 + 5 * ((bits + 7) / 8) : 22;
    }
    build_major = cperm != nullptr;
  }
  if (prof) SPJ_CUDA(cudaEventRecord(ws.ev[2], s));

  reset_status(ws.status, s);
  ws.flags.reserve(m + 1, s);
  uint32_t *rq = nullptr, *rqn = nullptr;
  const int mb = refine_blocks(cfg_.refine_min_blocks, build_major,
                               predicate == kIntersects || predicate == kDisjoint);
  const bool split = cfg_.refine_split == 1 || cfg_.refine_split == 3 ||
                     (cfg_.refine_split == 2 && !build_major);
  if (split && cfg_.refine_form == kFastF32 && predicate != kPredDWithin) {
    ws.rqueue.reserve((m + 2) * 4, s);
    rq = ws.rqueue.as<uint32_t>();
    rqn = rq + m + 1;
  }
  const GeomsView bv = bg_.view(), pv = ws.probe.view();
  if (predicate == kPredDWithin)
    refine_dwithin(bv, pv, ws.cand_build.as<uint32_t>(), ws.cand_probe.as<uint32_t>(), m,
                   probe_base, distance, cfg_.refine_form, ws.flags.as<uint8_t>(),
                   ws.status.as<DeviceStatus>(), s, cperm, d_row);
  else
    refine_relation(bv, pv, ws.cand_build.as<uint32_t>(), ws.cand_probe.as<uint32_t>(), m,
                    probe_base, predicate, cfg_.refine_form, ws.flags.as<uint8_t>(),
                    ws.status.as<DeviceStatus>(), s, nullptr, cperm, mb, rq, rqn,
                    cfg_.refine_split == 3);
  launches += rq ? 2 : 1;
  if (prof) SPJ_CUDA(cudaEventRecord(ws.ev[3], s));

  // compaction: tile counts and their scan, then the survivors tile by tile
  ws.scan_tmp.reserve(compact_sums_bytes((int64_t)m), s);
  uint64_t* sums = ws.scan_tmp.as<uint64_t>();
  compact_count(ws.flags.as<uint8_t>(), (int64_t)m, sums, s);
  uint64_t total = 0;
  DeviceStatus hst;
  SPJ_CUDA(cudaMemcpyAsync(&total, sums + compact_tiles((int64_t)m), 8, cudaMemcpyDeviceToHost,
                           s));
  SPJ_CUDA(cudaMemcpyAsync(&hst, ws.status.get(), sizeof hst, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  if (hst.first_bad != ~0ull) {
    throw Error(std::string("refine: ") + status_message((uint32_t)(hst.first_bad >> 40)));
  }
  ws.out_build.reserve((total + 1) * 4, s);
  ws.out_probe.reserve((total + 1) * 4, s);
  compact_pairs_tiles(ws.cand_build.as<uint32_t>(), ws.cand_probe.as<uint32_t>(),
                      ws.flags.as<uint8_t>(), (int64_t)m, sums, ws.out_build.as<uint32_t>(),
                      ws.out_probe.as<uint32_t>(), total, s);
  launches += 3;
  if (prof) SPJ_CUDA(cudaEventRecord(ws.ev[4], s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  {
    std::lock_guard<std::mutex> lk(stats_mu_);
    stats_.calls++;
    stats_.probe_rows += n;
    stats_.candidates += m;
    stats_.results += total;
    stats_.escalations += hst.counters[0];
    stats_.pairs_evaluated += hst.counters[1];
    stats_.kernel_launches += launches;
    stats_.probe_bytes += (uint64_t)col.data_len + (uint64_t)(col.n + 1) * (col.offsets64 ? 8 : 4);
    if (prof) {
      stats_.ms_decode += ev_ms(ws.ev[0], ws.ev[1]);
      stats_.ms_filter += ev_ms(ws.ev[1], ws.ev[2]);
      stats_.ms_refine += ev_ms(ws.ev[2], ws.ev[3]);
      stats_.ms_compact += ev_ms(ws.ev[3], ws.ev[4]);
    }
  }
  *d_build = ws.out_build.as<uint32_t>();
  *d_probe = ws.out_probe.as<uint32_t>();
  return total;
}

uint64_t JoinEngine::refine_pairs(Workspace& ws, const GeomsView& pv, const uint32_t* cb,
                                  const uint32_t* cp, uint64_t m, int predicate,
                                  double distance) {
  SPJ_CHECK(built_, "refine called before the build side was finished");
  cudaStream_t s = ws.stream;
  reset_status(ws.status, s);
  ws.flags.reserve(m + 1, s);
  const GeomsView bv = bg_.view();
  if (predicate == kPredDWithin)
    refine_dwithin(bv, pv, cb, cp, m, 0, distance, cfg_.refine_form, ws.flags.as<uint8_t>(),
                   ws.status.as<DeviceStatus>(), s);
  else
    refine_relation(bv, pv, cb, cp, m, 0, predicate, cfg_.refine_form, ws.flags.as<uint8_t>(),
                    ws.status.as<DeviceStatus>(), s, nullptr, nullptr,
                    refine_blocks(cfg_.refine_min_blocks, false));
  ws.scan_tmp.reserve(compact_sums_bytes((int64_t)m), s);
  uint64_t* sums = ws.scan_tmp.as<uint64_t>();
  compact_count(ws.flags.as<uint8_t>(), (int64_t)m, sums, s);
  uint64_t total = 0;
  DeviceStatus hst;
  SPJ_CUDA(cudaMemcpyAsync(&total, sums + compact_tiles((int64_t)m), 8, cudaMemcpyDeviceToHost,
                           s));
  SPJ_CUDA(cudaMemcpyAsync(&hst, ws.status.get(), sizeof hst, cudaMemcpyDeviceToHost, s));
  SPJ_CUDA(cudaStreamSynchronize(s));
  if (hst.first_bad != ~0ull)
    throw Error(std::string("refine: ") + status_message((uint32_t)(hst.first_bad >> 40)));
  ws.out_build.reserve((total + 1) * 4, s);
  ws.out_probe.reserve((total + 1) * 4, s);
  compact_pairs_tiles(cb, cp, ws.flags.as<uint8_t>(), (int64_t)m, sums,
                      ws.out_build.as<uint32_t>(), ws.out_probe.as<uint32_t>(), total, s);
  SPJ_CUDA(cudaStreamSynchronize(s));
  {
    std::lock_guard<std::mutex> lk(stats_mu_);
    stats_.candidates += m;
    stats_.results += total;
    stats_.escalations += hst.counters[0];
    stats_.pairs_evaluated += hst.counters[1];
  }
  return total;
}

JoinStats JoinEngine::stats() {
  std::lock_guard<std::mutex> lk(stats_mu_);
  return stats_;
}

void JoinEngine::reset_stats() {
  std::lock_guard<std::mutex> lk(stats_mu_);
  stats_ = JoinStats();
}

WkbDeviceColumn stage_column(Workspace& ws, const HostWkbColumn& col, uint64_t* bytes) {
  cudaStream_t s = ws.stream;
  WkbDeviceColumn d;
  d.n = col.n;
  d.offsets64 = col.offsets64;
  const size_t osz = col.offsets64 ? 8 : 4;
  int64_t base, end;
  if (col.n == 0) {
    base = end = 0;
  } else if (col.offsets64) {
    base = reinterpret_cast<const int64_t*>(col.offsets)[0];
    end = reinterpret_cast<const int64_t*>(col.offsets)[col.n];
  } else {
    base = reinterpret_cast<const int32_t*>(col.offsets)[0];
    end = reinterpret_cast<const int32_t*>(col.offsets)[col.n];
  }
  SPJ_CHECK(base >= 0 && end >= base, "invalid Arrow offsets");
  const int64_t base4 = base & ~int64_t(3);
  ws.wkb_offsets.reserve((size_t)(col.n + 1) * osz, s);
  ws.wkb_data.reserve((size_t)(end - base4) + 16, s);
  if (col.n >= 0 && col.offsets)
    SPJ_CUDA(cudaMemcpyAsync(ws.wkb_offsets.get(), col.offsets, (size_t)(col.n + 1) * osz,
                             cudaMemcpyHostToDevice, s));
  if (end > base4)
    SPJ_CUDA(cudaMemcpyAsync(ws.wkb_data.get(), col.data + base4, (size_t)(end - base4),
                             cudaMemcpyHostToDevice, s));
  uint64_t b = (uint64_t)(col.n + 1) * osz + (uint64_t)(end - base4);
  if (col.validity) {
    const int64_t b0 = col.validity_offset >> 3;
    const int64_t b1 = (col.validity_offset + col.n + 7) >> 3;
    ws.wkb_validity.reserve((size_t)(b1 - b0) + 1, s);
    SPJ_CUDA(cudaMemcpyAsync(ws.wkb_validity.get(), col.validity + b0, (size_t)(b1 - b0),
                             cudaMemcpyHostToDevice, s));
    d.validity = ws.wkb_validity.as<uint8_t>();
    d.validity_offset = col.validity_offset & 7;
    b += (uint64_t)(b1 - b0);
  }
  d.offsets = ws.wkb_offsets.get();
  // offsets index the caller's data buffer; shift the device pointer so the
  // same offsets land in the staged copy (which starts at base4)
  d.data = ws.wkb_data.as<uint8_t>() - base4;
  d.data_len = (uint64_t)end;
  if (bytes) *bytes = b;
  return d;
}

}  // namespace spj
