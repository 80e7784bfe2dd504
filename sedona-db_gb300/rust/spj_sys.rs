// spj_sys.rs — Rust bindings of include/spj_gb300.h (the entry points this
// library adds beyond the reference's gpuspatial_c.h), for the
// sedona-libgpuspatial crate (c/sedona-libgpuspatial/src/), beside its
// bindgen output for gpuspatial_c.h (libgpuspatial_glue_bindgen.rs).
//
// Not compiled in this repository (there is no Rust toolchain here); the
// declarations mirror include/spj_gb300.h field for field, and a maintainer
// may equally generate them with bindgen from that header.
#![allow(non_camel_case_types, dead_code)]

use std::ffi::{c_char, c_int, c_void, CStr};
use std::ptr;

use arrow::ffi::{FFI_ArrowArray, FFI_ArrowSchema};

use crate::libgpuspatial_glue_bindgen::GpuSpatialRuntime;

pub const SPJ_PREDICATE_DWITHIN: i32 = 100;
pub const SPJ_REFINE_PLAIN_F64: i32 = 0;
pub const SPJ_REFINE_FAST_F32: i32 = 1;
const ENOSPC: c_int = 28;

#[repr(C)]
pub struct SpjJoinConfig {
    pub runtime: *const GpuSpatialRuntime,
    pub leaf_size: u32,
    pub refine_form: i32,
    pub profile: i32,
    pub probe_order: i32,
}

#[repr(C)]
pub struct SpjKnnConfig {
    pub runtime: *const GpuSpatialRuntime,
    pub leaf_size: u32,
    pub refine_form: i32,
}

#[repr(C)]
pub struct SpjJoin {
    _private: [u8; 0],
}
#[repr(C)]
pub struct SpjKnn {
    _private: [u8; 0],
}

pub type PairCallback =
    unsafe extern "C" fn(build: *const u32, probe: *const u32, len: u64, ud: *mut c_void) -> c_int;

extern "C" {
    pub fn SpjJoinCreate(config: *const SpjJoinConfig, out: *mut *mut SpjJoin) -> c_int;
    pub fn SpjJoinRelease(join: *mut SpjJoin);
    pub fn SpjJoinLastError(join: *mut SpjJoin) -> *const c_char;
    pub fn SpjJoinSetOption(join: *mut SpjJoin, key: *const c_char, value: i64) -> c_int;
    pub fn SpjJoinPushBuildArrow(
        join: *mut SpjJoin,
        schema: *const FFI_ArrowSchema,
        array: *const FFI_ArrowArray,
    ) -> c_int;
    pub fn SpjJoinFinishBuild(join: *mut SpjJoin) -> c_int;
    pub fn SpjJoinSetProbeDistances(
        join: *mut SpjJoin,
        distances: *const f64,
        n: u64,
        device: i32,
    ) -> c_int;
    pub fn SpjJoinProbeArrow(
        join: *mut SpjJoin,
        schema: *const FFI_ArrowSchema,
        array: *const FFI_ArrowArray,
        predicate: i32,
        distance: f64,
        probe_base: u32,
        callback: PairCallback,
        user_data: *mut c_void,
    ) -> c_int;

    pub fn SpjKnnCreate(config: *const SpjKnnConfig, out: *mut *mut SpjKnn) -> c_int;
    pub fn SpjKnnRelease(knn: *mut SpjKnn);
    pub fn SpjKnnLastError(knn: *mut SpjKnn) -> *const c_char;
    pub fn SpjKnnBuild(knn: *mut SpjKnn, xy: *const f64, n: u64) -> c_int;
    pub fn SpjKnnQueryArrow(
        knn: *mut SpjKnn,
        schema: *const FFI_ArrowSchema,
        array: *const FFI_ArrowArray,
        k: u32,
        include_tie_breakers: i32,
        offsets: *mut u64,
        out_idx: *mut u32,
        out_dist: *mut f64,
        capacity: u64,
        total: *mut u64,
    ) -> c_int;
}

fn message(p: *const c_char) -> String {
    if p.is_null() {
        return String::new();
    }
    unsafe { CStr::from_ptr(p) }.to_string_lossy().into_owned()
}

/// The fused build / probe / refine join over the device: probe WKB in,
/// refined (build, probe) pairs out, with no host work between filter and
/// refine.  One object serves one thread at a time; the provider keeps one
/// per probe partition (a pool), all built from the same build batches.
pub struct SpjJoinHandle {
    raw: *mut SpjJoin,
}
unsafe impl Send for SpjJoinHandle {}

impl SpjJoinHandle {
    pub fn try_new(runtime: *const GpuSpatialRuntime) -> Result<Self, String> {
        let cfg = SpjJoinConfig {
            runtime,
            leaf_size: 0,
            refine_form: SPJ_REFINE_FAST_F32,
            profile: 0,
            probe_order: 0,
        };
        let mut raw = ptr::null_mut();
        if unsafe { SpjJoinCreate(&cfg, &mut raw) } != 0 {
            return Err("SpjJoinCreate failed".into());
        }
        Ok(Self { raw })
    }

    fn check(&self, rc: c_int, what: &str) -> Result<(), String> {
        if rc == 0 {
            Ok(())
        } else {
            Err(format!("{what}: {}", message(unsafe { SpjJoinLastError(self.raw) })))
        }
    }

    pub fn set_option(&mut self, key: &CStr, value: i64) -> Result<(), String> {
        let rc = unsafe { SpjJoinSetOption(self.raw, key.as_ptr(), value) };
        self.check(rc, "SpjJoinSetOption")
    }

    pub fn push_build(
        &mut self,
        schema: &FFI_ArrowSchema,
        array: &FFI_ArrowArray,
    ) -> Result<(), String> {
        let rc = unsafe { SpjJoinPushBuildArrow(self.raw, schema, array) };
        self.check(rc, "SpjJoinPushBuildArrow")
    }

    pub fn finish_build(&mut self) -> Result<(), String> {
        let rc = unsafe { SpjJoinFinishBuild(self.raw) };
        self.check(rc, "SpjJoinFinishBuild")
    }

    /// ST_DWithin distance column for the next probe (None: the scalar).
    pub fn set_probe_distances(&mut self, d: Option<&[f64]>) -> Result<(), String> {
        let (p, n) = d.map_or((ptr::null(), 0), |d| (d.as_ptr(), d.len() as u64));
        let rc = unsafe { SpjJoinSetProbeDistances(self.raw, p, n, 0) };
        self.check(rc, "SpjJoinSetProbeDistances")
    }

    /// Refined pairs of one probe batch; probe ids are offset by probe_base.
    pub fn probe(
        &mut self,
        schema: &FFI_ArrowSchema,
        array: &FFI_ArrowArray,
        predicate: i32,
        distance: f64,
        probe_base: u32,
        build_out: &mut Vec<u32>,
        probe_out: &mut Vec<u32>,
    ) -> Result<(), String> {
        struct Sink<'a> {
            b: &'a mut Vec<u32>,
            p: &'a mut Vec<u32>,
        }
        unsafe extern "C" fn collect(b: *const u32, p: *const u32, n: u64, ud: *mut c_void) -> c_int {
            let sink = &mut *(ud as *mut Sink);
            let n = n as usize;
            if n > 0 {
                sink.b.extend_from_slice(std::slice::from_raw_parts(b, n));
                sink.p.extend_from_slice(std::slice::from_raw_parts(p, n));
            }
            0
        }
        let mut sink = Sink { b: build_out, p: probe_out };
        let rc = unsafe {
            SpjJoinProbeArrow(
                self.raw,
                schema,
                array,
                predicate,
                distance,
                probe_base,
                collect,
                &mut sink as *mut Sink as *mut c_void,
            )
        };
        self.check(rc, "SpjJoinProbeArrow")
    }
}

impl Drop for SpjJoinHandle {
    fn drop(&mut self) {
        unsafe { SpjJoinRelease(self.raw) }
    }
}

/// KNN over a point build side (SpjKnn*).
pub struct SpjKnnHandle {
    raw: *mut SpjKnn,
}
unsafe impl Send for SpjKnnHandle {}

impl SpjKnnHandle {
    pub fn try_new(runtime: *const GpuSpatialRuntime, build_xy: &[f64]) -> Result<Self, String> {
        let cfg = SpjKnnConfig { runtime, leaf_size: 0, refine_form: SPJ_REFINE_FAST_F32 };
        let mut raw = ptr::null_mut();
        if unsafe { SpjKnnCreate(&cfg, &mut raw) } != 0 {
            return Err("SpjKnnCreate failed".into());
        }
        let h = Self { raw };
        let rc = unsafe { SpjKnnBuild(raw, build_xy.as_ptr(), (build_xy.len() / 2) as u64) };
        if rc != 0 {
            return Err(format!("SpjKnnBuild: {}", message(unsafe { SpjKnnLastError(raw) })));
        }
        Ok(h)
    }

    /// Per probe row i: (build row, distance) pairs in
    /// out[offsets[i]..offsets[i + 1]], the k nearest and, with
    /// include_tie_breakers, the ties within 1e-9 of the k-th distance.
    pub fn query(
        &mut self,
        schema: &FFI_ArrowSchema,
        array: &FFI_ArrowArray,
        rows: usize,
        k: u32,
        include_tie_breakers: bool,
    ) -> Result<(Vec<u64>, Vec<u32>, Vec<f64>), String> {
        let mut offsets = vec![0u64; rows + 1];
        let mut cap = rows * k as usize + 16;
        loop {
            let mut idx = vec![0u32; cap];
            let mut dist = vec![0f64; cap];
            let mut total = 0u64;
            let rc = unsafe {
                SpjKnnQueryArrow(
                    self.raw,
                    schema,
                    array,
                    k,
                    include_tie_breakers as i32,
                    offsets.as_mut_ptr(),
                    idx.as_mut_ptr(),
                    dist.as_mut_ptr(),
                    cap as u64,
                    &mut total,
                )
            };
            if rc == ENOSPC {
                cap = total as usize;
                continue;
            }
            if rc != 0 {
                return Err(format!("SpjKnnQueryArrow: {}", message(unsafe { SpjKnnLastError(self.raw) })));
            }
            idx.truncate(total as usize);
            dist.truncate(total as usize);
            return Ok((offsets, idx, dist));
        }
    }
}

impl Drop for SpjKnnHandle {
    fn drop(&mut self) {
        unsafe { SpjKnnRelease(self.raw) }
    }
}

// ---------------------------------------------------------------------------
// GeoParquet -> device, result materialisation and the partitioned join
// (include/spj_gb300.h): the readers and operators of sedona-geoparquet and
// sedona-spatial-join call these in place of their CPU paths.

/// An Arrow binary / large_binary column whose buffers are in device memory.
#[repr(C)]
#[derive(Clone, Copy)]
pub struct SpjDeviceWkb {
    pub length: i64,
    pub offsets: *const c_void,
    pub offsets_are_64bit: i32,
    pub data: *const u8,
    pub data_length: u64,
    pub validity: *const u8,
    pub validity_offset: i64,
}

/// A WKB column (Arrow binary / large_binary layout) in host memory.
#[repr(C)]
pub struct SpjHostWkb {
    pub length: i64,
    pub offsets: *const c_void,
    pub offsets_are_64bit: i32,
    pub data: *const u8,
    pub validity: *const u8,
    pub validity_offset: i64,
}

#[repr(C)]
pub struct SpjParquet {
    _private: [u8; 0],
}

#[repr(C)]
pub struct SpjParquetWriteOptions {
    pub compression: i32,
    pub page_version: i32,
    pub row_group_rows: i64,
    pub page_bytes: i64,
}

#[repr(C)]
pub struct SpjPartitionOptions {
    pub num_partitions: u32,
    pub sample_rows: u32,
    pub build_budget_bytes: u64,
    pub seed: u64,
    pub host_gather: i32,
    pub record_layout: i32,
}

#[repr(C)]
#[derive(Default)]
pub struct SpjPartitionStats {
    pub partitions: u32,
    pub passes: u32,
    pub build_rows_max: u64,
    pub probe_rows_multi: u64,
    pub probe_rows_none: u64,
    pub probe_rows_probed: u64,
    pub pairs: u64,
    pub ms_boxes: f64,
    pub ms_partition: f64,
    pub ms_passes: f64,
    pub direct_host_reads: i32,
}

pub const SPJ_NULL_INDEX: u32 = 0xFFFF_FFFF;

extern "C" {
    pub fn SpjJoinBuildDevice(join: *mut SpjJoin, column: *const SpjDeviceWkb) -> c_int;

    pub fn SpjParquetOpen(path: *const c_char, out: *mut *mut SpjParquet) -> c_int;
    pub fn SpjParquetRelease(file: *mut SpjParquet);
    pub fn SpjParquetLastError(file: *mut SpjParquet) -> *const c_char;
    pub fn SpjParquetInfo(
        file: *mut SpjParquet,
        num_rows: *mut i64,
        num_row_groups: *mut i32,
        num_columns: *mut i32,
    ) -> c_int;
    pub fn SpjParquetColumnName(file: *mut SpjParquet, i: i32, buf: *mut c_char, cap: u64) -> c_int;
    pub fn SpjParquetRowGroupRows(file: *mut SpjParquet, row_group: i32, rows: *mut i64) -> c_int;
    pub fn SpjParquetReadWkb(
        file: *mut SpjParquet,
        column: *const c_char,
        rg_begin: i32,
        rg_end: i32,
        device: i32,
        out: *mut SpjDeviceWkb,
    ) -> c_int;
    pub fn SpjParquetWriteWkb(
        path: *const c_char,
        column: *const c_char,
        length: i64,
        offsets: *const c_void,
        offsets_are_64bit: i32,
        data: *const u8,
        validity: *const u8,
        validity_offset: i64,
        options: *const SpjParquetWriteOptions,
    ) -> c_int;

    pub fn SpjMaterializeLastError() -> *const c_char;
    pub fn SpjGatherFixed(
        d_values: *const c_void,
        width: u32,
        n_values: u64,
        d_idx: *const u32,
        n: u64,
        d_out: *mut c_void,
        stream: *mut c_void,
    ) -> c_int;
    pub fn SpjGatherValidity(
        d_validity: *const u8,
        validity_offset: i64,
        n_values: u64,
        d_idx: *const u32,
        n: u64,
        d_out_bitmap: *mut u8,
        null_count: *mut u64,
        stream: *mut c_void,
    ) -> c_int;
    pub fn SpjGatherBinary(
        d_offsets: *const c_void,
        offsets_are_64bit: i32,
        d_data: *const u8,
        n_values: u64,
        d_idx: *const u32,
        n: u64,
        d_out_offsets: *mut i64,
        d_out_data: *mut u8,
        capacity: u64,
        out_bytes: *mut u64,
        stream: *mut c_void,
    ) -> c_int;
    pub fn SpjVisitedMark(
        d_bitmap: *mut u32,
        n_rows: u64,
        d_idx: *const u32,
        n: u64,
        stream: *mut c_void,
    ) -> c_int;
    pub fn SpjVisitedCollect(
        d_bitmap: *const u32,
        n_rows: u64,
        visited: i32,
        d_out_idx: *mut u32,
        capacity: u64,
        count: *mut u64,
        stream: *mut c_void,
    ) -> c_int;

    pub fn SpjJoinPartitioned(
        join: *mut SpjJoin,
        build: *const SpjHostWkb,
        probe: *const SpjHostWkb,
        predicate: i32,
        distance: f64,
        options: *const SpjPartitionOptions,
        callback: PairCallback,
        user_data: *mut c_void,
        stats: *mut SpjPartitionStats,
    ) -> c_int;
}

/// A GeoParquet file opened for device reads (sedona-geoparquet's
/// file_opener.rs reads the geometry column through this instead of
/// arrow-rs when the scan feeds a GPU join).
pub struct SpjParquetFile {
    raw: *mut SpjParquet,
}

impl SpjParquetFile {
    pub fn open(path: &CStr) -> Result<Self, String> {
        let mut raw = ptr::null_mut();
        let rc = unsafe { SpjParquetOpen(path.as_ptr(), &mut raw) };
        if rc != 0 {
            return Err(format!("SpjParquetOpen: {}", message(unsafe { SpjParquetLastError(ptr::null_mut()) })));
        }
        Ok(Self { raw })
    }

    /// Row groups [rg_begin, rg_end) of a WKB column (None: the primary
    /// geometry column) as a device column, valid until the next read.
    pub fn read_wkb(
        &mut self,
        column: Option<&CStr>,
        rg_begin: i32,
        rg_end: i32,
        device: i32,
    ) -> Result<SpjDeviceWkb, String> {
        let mut out = SpjDeviceWkb {
            length: 0,
            offsets: ptr::null(),
            offsets_are_64bit: 1,
            data: ptr::null(),
            data_length: 0,
            validity: ptr::null(),
            validity_offset: 0,
        };
        let col = column.map_or(ptr::null(), |c| c.as_ptr());
        let rc = unsafe { SpjParquetReadWkb(self.raw, col, rg_begin, rg_end, device, &mut out) };
        if rc != 0 {
            return Err(format!("SpjParquetReadWkb: {}", message(unsafe { SpjParquetLastError(self.raw) })));
        }
        Ok(out)
    }
}

impl Drop for SpjParquetFile {
    fn drop(&mut self) {
        unsafe { SpjParquetRelease(self.raw) }
    }
}
