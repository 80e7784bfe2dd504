// parquet.cuh — GeoParquet WKB columns: the file metadata parsed on the host
// (Thrift compact protocol, the Parquet format's own footer encoding), the
// page table of the selected column chunks, and the device decode.
//
// The reference reads GeoParquet through arrow-rs on the CPU
// (rust/sedona-geoparquet/src/file_opener.rs:125-210 opens the file and plans
// row groups; metadata.rs:382-460 takes the geometry columns from the "geo"
// key) and then parses every WKB value again on the CPU
// (EvaluatedGeometryArray, rust/sedona-spatial-join/src/operand_evaluator.rs).
// Here only the footer and the page headers are read on the host; the chunk
// bytes go to HBM in one copy and every page is decompressed and decoded
// there into the Arrow large_binary layout the WKB decode kernel reads.
#pragma once
#include <functional>
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"

namespace spj {
namespace pq {

// Parquet enums (parquet.thrift)
enum PhysType { kBoolean = 0, kInt32 = 1, kInt64 = 2, kInt96 = 3, kFloat = 4, kDouble = 5,
                kByteArray = 6, kFixedLenByteArray = 7 };
enum Repetition { kRequired = 0, kOptional = 1, kRepeated = 2 };
enum Codec { kUncompressed = 0, kSnappy = 1 };
enum Encoding { kPlain = 0, kPlainDictionary = 2, kRle = 3, kRleDictionary = 8 };
enum PageType { kDataPage = 0, kIndexPage = 1, kDictionaryPage = 2, kDataPageV2 = 3 };

struct SchemaElement {
  int type = -1;
  int repetition = -1;
  int num_children = 0;
  std::string name;
};

struct ColumnChunk {
  int type = -1;
  int codec = 0;
  std::vector<std::string> path;
  int64_t num_values = 0;
  int64_t total_compressed = 0;
  int64_t data_page_offset = -1;
  int64_t dictionary_page_offset = -1;
};

struct RowGroup {
  int64_t num_rows = 0;
  std::vector<ColumnChunk> columns;
};

struct Leaf {
  std::string name;  // dotted path
  int type = -1;
  int max_def = 0, max_rep = 0;
  bool top_level = false;
};

struct FileMeta {
  int64_t num_rows = 0;
  std::vector<SchemaElement> schema;
  std::vector<RowGroup> row_groups;
  std::vector<std::pair<std::string, std::string>> kv;
  std::string created_by;
  std::vector<Leaf> leaves;       // schema leaves in column order
  std::string primary_column;     // from the "geo" key ("" when absent)
  std::vector<std::pair<std::string, std::string>> geo_encodings;  // column -> encoding
};

// Parses the footer (FileMetaData) from the last `tail_len` bytes of a file
// of `file_len` bytes.  Returns the tail length it needs when the tail is
// too short (0 when parsed).  Throws spj::Error on a malformed file.
uint64_t parse_footer(const uint8_t* tail, uint64_t tail_len, uint64_t file_len, FileMeta& out);

// One page of a column chunk, located in the staging buffer.
struct PageInfo {
  uint64_t src = 0;        // offset of the stored page bytes (after its header)
  uint64_t dst = 0;        // offset of the decompressed bytes in the page buffer
  uint64_t first_row = 0;  // data pages: column row of the page's first value
  uint32_t src_size = 0, raw_size = 0;
  uint32_t num_values = 0;
  uint32_t lvl_bytes = 0;  // v2: definition + repetition level bytes (never compressed)
  uint32_t def_len = 0;    // v2: definition level bytes
  int32_t dict = -1;       // the chunk's dictionary (index into the dictionary table)
  uint8_t kind = 0;        // 0 dictionary, 1 data v1, 2 data v2
  uint8_t codec = 0;
  uint8_t encoding = 0;
  uint8_t max_def = 0;
  uint8_t in_src = 0;      // not compressed: decoded straight from the staging buffer
  uint8_t pad[3] = {};
};
static_assert(sizeof(PageInfo) == 56, "PageInfo layout");

// Walks the page headers of one column chunk held at buf[begin, end) and
// appends its pages (data pages numbered from *row on).  The chunk's
// dictionary, if it has one, gets the id dict_index (its page and the data
// pages that use it carry it); returns whether it had one.
bool walk_pages(const uint8_t* buf, uint64_t begin, uint64_t end, int codec, int max_def,
                int dict_index, uint64_t* row, std::vector<PageInfo>& pages);
// The same walk with the bytes fetched on demand: bytes_at(pos) gives the
// chunk's bytes from position pos on, at least the page header there (a
// header cut short throws "truncated thrift structure").  header_pos, when
// given, receives each page's header position.
using HeaderBytes = std::function<std::pair<const uint8_t*, const uint8_t*>(uint64_t)>;
bool walk_pages(const HeaderBytes& bytes_at, uint64_t begin, uint64_t end, int codec,
                int max_def, int dict_index, uint64_t* row, std::vector<PageInfo>& pages,
                std::vector<uint64_t>* header_pos);

// Snappy block compression (the published format: a varint length, then
// literal and copy elements); used by the writer.
void snappy_compress(const uint8_t* in, size_t n, std::string& out);

struct WriteOptions {
  int compression = 1;  // 0 none, 1 snappy
  int page_version = 1;
  int64_t row_group_rows = 1 << 20;
  int64_t page_bytes = 1 << 20;
};

// Writes a GeoParquet file with one optional BYTE_ARRAY WKB column.
void write_wkb(const char* path, const char* column, int64_t n, const void* offsets,
               bool offsets64, const uint8_t* data, const uint8_t* validity,
               int64_t validity_offset, const WriteOptions& opt);

}  // namespace pq
}  // namespace spj
