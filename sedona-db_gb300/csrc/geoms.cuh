// geoms.cuh — device-resident geometry columns (structure of arrays in HBM).
//
// One decoded Arrow WKB column becomes:
//   kind[n]                 u8   0 empty/null, 1 point, 3 polygon, 6 multipolygon
//   pt[n]                   f64x2 the point of a point row (NaN otherwise)
//   box[n]                  f32x4 (xmin, ymin, xmax, ymax) filter box, NaN = empty;
//                           points round to nearest (degenerate box), everything
//                           else is rounded outward
//                           (rust/sedona-spatial-join-gpu/src/join_provider.rs:109-141,
//                            rust/sedona-spatial-join/src/utils/bounds.rs:147-162)
//   row_part[n+1]           u32  row -> polygons (parts)
//   part_ring[nparts+1]     u32  part -> rings (ring 0 of a part is its shell)
//   ring_vtx[nrings+1]      u32  ring -> vertices; every ring stores its points
//                           plus one extra copy of its first point, so segment i
//                           is (v[i], v[i+1]) for i < nsegs (the layout tg builds,
//                           c/sedona-tg/src/tg/tg.c:2210-2221)
//   ring_nsegs[nrings]      i32  tg num_segments (tg.c:2124-2134)
//   ring_rect[nrings]       f64x4 exact vertex bounds of the ring
//   xy[nverts]              f64x2 vertices (16 B, one 128-bit load each)
//   xy32[nverts]            f32x2 the same vertices rounded to nearest
//   row_flags[n]            u8   bit 0: a multipolygon row had parts without
//                           rings (those parts are not stored; tg keeps them
//                           as empty children, which a polygon covering the
//                           row must also cover, tg.c:5872-5897)
//   ring_flags[nrings]      u8   tg's ring flags (tg.c:1910-2113): bit 0
//                           convex, bit 1 clockwise, bit 7 set once computed
//                           (build_ring_flags; absent for columns that did
//                           not need them, in which case the relate code
//                           computes a ring's flags where it uses them)
// and, for a build side that is refined against, a per-ring y-band edge index
// (band_*), see refine.cu, and a per-ring cell grid (grid_*): a G x G grid
// over the ring's rect whose clean cells (no edge touches the closed cell)
// carry the ring's inside / outside status (used by point-in-ring tests), see
// cellgrid.cu.
#pragma once
#include "common.cuh"

namespace spj {

enum GeomKind : uint8_t { kEmpty = 0, kPoint = 1, kPolygon = 3, kMultiPolygon = 6 };

struct GeomsView {
  uint32_t n = 0;
  uint32_t nparts = 0, nrings = 0, nverts = 0;
  const uint8_t* kind = nullptr;
  const double2* pt = nullptr;
  const float4* box = nullptr;
  const uint32_t* row_part = nullptr;
  const uint32_t* part_ring = nullptr;
  const uint32_t* ring_vtx = nullptr;
  const int32_t* ring_nsegs = nullptr;
  const Rect64* ring_rect = nullptr;
  const float4* ring_rect32 = nullptr;  // the same rect rounded to nearest
  const double2* xy = nullptr;
  const float2* xy32 = nullptr;
  const uint8_t* row_flags = nullptr;   // nullptr: no row had empty parts
  const uint8_t* ring_flags = nullptr;  // nullptr: not computed
  // y-band edge index (nullptr when not built)
  const uint32_t* ring_bands = nullptr;  // nrings+1: start of each ring's band_off slice
  const uint32_t* band_off = nullptr;    // per ring: nb+1 offsets into band_edges
  const uint16_t* band_edges = nullptr;  // edge index within the ring
  // the same entries' f32 segments (a.x, a.y, b.x, b.y): the FP32 tiers read
  // one 16-byte word per entry instead of an index and then two vertices
  const float4* band_seg = nullptr;
  const float2* band_param = nullptr;    // per ring: (y origin, bands per unit y)
  // cell grid (nullptr when not built): per ring (status offset, G; G = 0 for
  // no grid), (x0, y0, w, h) with cell (i, j) = [x0 + i w, x0 + (i+1) w] x
  // [y0 + j h, y0 + (j+1) h] in f32 arithmetic, and one status byte per cell
  // (0 mixed, 1 inside, 2 outside)
  const uint2* grid_meta = nullptr;
  const float4* grid_rect = nullptr;
  const uint8_t* grid_status = nullptr;
  // ring-ring and ring-in-ring tests may answer from the cells that hold the
  // other ring's box (when they are all clean and alike)
  bool grid_rings = false;
};

struct DeviceGeoms {
  uint32_t n = 0, nparts = 0, nrings = 0, nverts = 0;
  bool all_points = false;  // every non-empty row is a point
  bool any_points = false;
  bool any_polys = false;
  DevBuf kind, pt, box, row_part, part_ring, ring_vtx, ring_nsegs, ring_rect, ring_rect32, xy,
      xy32;
  DevBuf row_flags, ring_flags;
  bool has_row_flags = false, has_ring_flags = false;
  DevBuf ring_bands, band_off, band_edges, band_seg, band_param;
  bool has_bands = false;
  DevBuf grid_meta, grid_rect, grid_status;
  bool has_grid = false;
  bool grid_rings = false;

  GeomsView view() const {
    GeomsView v;
    v.n = n;
    v.nparts = nparts;
    v.nrings = nrings;
    v.nverts = nverts;
    v.kind = kind.as<uint8_t>();
    v.pt = pt.as<double2>();
    v.box = box.as<float4>();
    v.row_part = row_part.as<uint32_t>();
    v.part_ring = part_ring.as<uint32_t>();
    v.ring_vtx = ring_vtx.as<uint32_t>();
    v.ring_nsegs = ring_nsegs.as<int32_t>();
    v.ring_rect = ring_rect.as<Rect64>();
    v.ring_rect32 = ring_rect32.as<float4>();
    v.xy = xy.as<double2>();
    v.xy32 = xy32.as<float2>();
    if (has_row_flags) v.row_flags = row_flags.as<uint8_t>();
    if (has_ring_flags) v.ring_flags = ring_flags.as<uint8_t>();
    if (has_bands) {
      v.ring_bands = ring_bands.as<uint32_t>();
      v.band_off = band_off.as<uint32_t>();
      v.band_edges = band_edges.as<uint16_t>();
      v.band_seg = band_seg.as<float4>();
      v.band_param = band_param.as<float2>();
    }
    if (has_grid) {
      v.grid_meta = grid_meta.as<uint2>();
      v.grid_rect = grid_rect.as<float4>();
      v.grid_status = grid_status.as<uint8_t>();
      v.grid_rings = grid_rings;
    }
    return v;
  }
  size_t device_bytes() const {
    return kind.size() + pt.size() + box.size() + row_part.size() + part_ring.size() +
           ring_vtx.size() + ring_nsegs.size() + ring_rect.size() + ring_rect32.size() +
           xy.size() + xy32.size() + row_flags.size() + ring_flags.size() +
           ring_bands.size() + band_off.size() + band_edges.size() + band_seg.size() +
           band_param.size() +
           grid_meta.size() + grid_rect.size() + grid_status.size();
  }
};

// A WKB column whose buffers are already on the device.
struct WkbDeviceColumn {
  int64_t n = 0;
  const void* offsets = nullptr;  // int32 or int64, n+1 entries
  bool offsets64 = false;
  const uint8_t* data = nullptr;
  uint64_t data_len = 0;
  const uint8_t* validity = nullptr;  // LSB bitmap or nullptr
  int64_t validity_offset = 0;        // Arrow array offset applied to validity bits
};

struct DecodeScratch {
  DevBuf counts, scans, ring_src, tmp, status;
};

// Decode a device WKB column into `out`.  points_hint: the caller expects a
// point column; the single-kernel point path is used and the call falls back
// to the general path when a non-point row shows up.  Throws spj::Error on
// malformed WKB (message names the first bad row).
void decode_wkb(const WkbDeviceColumn& col, DeviceGeoms& out, DecodeScratch& scratch,
                bool points_hint, cudaStream_t s);

// tg's convex / clockwise flags of every ring (ring_flags); cheap, but only
// the polygon-polygon relations other than intersects read them.
void build_ring_flags(DeviceGeoms& g, cudaStream_t s);

// Build the per-ring y-band edge index used by the banded refine kernels.
void build_band_index(DeviceGeoms& g, DecodeScratch& scratch, cudaStream_t s);

// Build the per-ring cell grids (after the band index): rings with at least
// kGridMinSegs segments get a G x G grid, G = clamp(2 ceil(sqrt(nsegs)), 8, 32).
constexpr int kGridMinSegs = 12;
void build_cell_grid(DeviceGeoms& g, DecodeScratch& scratch, cudaStream_t s);

// Reads the device status word; throws with a message if a kernel failed.
void check_status(DevBuf& status, cudaStream_t s, const char* what);
void reset_status(DevBuf& status, cudaStream_t s);

}  // namespace spj
