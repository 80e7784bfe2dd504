// materialize.cuh — device gathers shared by the result materialisation
// entry points and the partitioned join's passes.
#pragma once
#include "common.cuh"
#include "geoms.cuh"

namespace spj {

// Rows idx[0..n) of a binary column (its offsets / data may be device memory
// or host memory the device can read) into a device large_binary column:
// out_off (n + 1 int64) and out_data; returns the data bytes.  Indices must
// be < col.n.  Synchronizes s.
uint64_t gather_binary(const WkbDeviceColumn& col, const uint32_t* d_idx, uint64_t n,
                       DevBuf& out_off, DevBuf& out_data, DevBuf& scratch_len,
                       DevBuf& scratch_pos, DevBuf& scan_tmp, cudaStream_t s);

// out[i] = values[idx[i]] for 8-byte values (indices < n_values).
void gather_u64(const uint64_t* values, uint64_t n_values, const uint32_t* d_idx, uint64_t n,
                uint64_t* out, cudaStream_t s);

}  // namespace spj
