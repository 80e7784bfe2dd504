// parquet_meta.cu — host side of the GeoParquet path: the Thrift compact
// protocol (the encoding of Parquet's footer and page headers), the footer
// and page-header parsers, the "geo" metadata (a small JSON reader), a
// Snappy block compressor and a GeoParquet writer for WKB columns.
//
// Field ids and enum values follow the Parquet format's parquet.thrift;
// the "geo" key and its primary_column / columns.<name>.encoding members
// follow the GeoParquet specification as the reference reads them
// (rust/sedona-geoparquet/src/metadata.rs:283-330, 382-460).
#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstring>

#include "parquet.cuh"

namespace spj {
namespace pq {
namespace {

// ---------------------------------------------------------------------------
// Thrift compact protocol

enum TType { kTStop = 0, kTTrue = 1, kTFalse = 2, kTByte = 3, kTI16 = 4, kTI32 = 5, kTI64 = 6,
             kTDouble = 7, kTBinary = 8, kTList = 9, kTSet = 10, kTMap = 11, kTStruct = 12 };

constexpr int kMaxDepth = 32;

struct TIn {
  const uint8_t* p;
  const uint8_t* end;

  void need(uint64_t n) const {
    if ((uint64_t)(end - p) < n) throw Error("parquet: truncated thrift structure");
  }
  uint8_t byte() {
    need(1);
    return *p++;
  }
  uint64_t varint() {
    uint64_t v = 0;
    for (int sh = 0;; sh += 7) {
      if (sh > 63) throw Error("parquet: thrift varint too long");
      const uint8_t b = byte();
      v |= (uint64_t)(b & 0x7f) << sh;
      if (!(b & 0x80)) return v;
    }
  }
  int64_t zigzag() {
    const uint64_t v = varint();
    return (int64_t)(v >> 1) ^ -(int64_t)(v & 1);
  }
  std::string binary() {
    const uint64_t n = varint();
    need(n);
    std::string s(reinterpret_cast<const char*>(p), n);
    p += n;
    return s;
  }
  void skip(int type, int depth);
};

// on_field(id, type) reads the field and returns true, or returns false to
// have it skipped
template <class F>
void read_struct(TIn& in, F&& on_field, int depth = 0) {
  if (depth > kMaxDepth) throw Error("parquet: thrift nesting too deep");
  int16_t last = 0;
  for (;;) {
    const uint8_t h = in.byte();
    if (h == kTStop) return;
    const int type = h & 0x0f;
    const int delta = h >> 4;
    const int16_t id = delta ? (int16_t)(last + delta) : (int16_t)in.zigzag();
    last = id;
    if (!on_field(id, type)) in.skip(type, depth + 1);
  }
}

// calls elem(element type) once per element
template <class F>
void read_list(TIn& in, F&& elem) {
  const uint8_t h = in.byte();
  uint64_t n = h >> 4;
  const int et = h & 0x0f;
  if (n == 15) n = in.varint();
  if (n > (uint64_t)(in.end - in.p)) throw Error("parquet: thrift list longer than its input");
  for (uint64_t i = 0; i < n; i++) elem(et);
}

void TIn::skip(int type, int depth) {
  if (depth > kMaxDepth) throw Error("parquet: thrift nesting too deep");
  switch (type) {
    case kTTrue:
    case kTFalse:
      return;  // a struct field's bool lives in its type nibble
    case kTByte:
      need(1);
      p += 1;
      return;
    case kTI16:
    case kTI32:
    case kTI64:
      varint();
      return;
    case kTDouble:
      need(8);
      p += 8;
      return;
    case kTBinary: {
      const uint64_t n = varint();
      need(n);
      p += n;
      return;
    }
    case kTList:
    case kTSet:
      read_list(*this, [&](int et) {
        if (et == kTTrue || et == kTFalse) {  // a list's bools take one byte each
          need(1);
          p += 1;
        } else {
          skip(et, depth + 1);
        }
      });
      return;
    case kTMap: {
      const uint64_t n = varint();
      if (n == 0) return;
      const uint8_t kv = byte();
      for (uint64_t i = 0; i < n; i++) {
        skip(kv >> 4, depth + 1);
        skip(kv & 0x0f, depth + 1);
      }
      return;
    }
    case kTStruct:
      read_struct(*this, [](int16_t, int) { return false; }, depth + 1);
      return;
    default:
      throw Error("parquet: unknown thrift type " + std::to_string(type));
  }
}

int32_t as_i32(TIn& in) {
  const int64_t v = in.zigzag();
  if (v < INT32_MIN || v > INT32_MAX) throw Error("parquet: i32 field out of range");
  return (int32_t)v;
}

struct TOut {
  std::string b;
  std::vector<int16_t> last{0};

  void byte(uint8_t v) { b.push_back((char)v); }
  void varint(uint64_t v) {
    while (v >= 0x80) {
      byte((uint8_t)(v | 0x80));
      v >>= 7;
    }
    byte((uint8_t)v);
  }
  void zigzag(int64_t v) { varint(((uint64_t)v << 1) ^ (uint64_t)(v >> 63)); }
  void field(int16_t id, int type) {
    const int d = id - last.back();
    if (d > 0 && d <= 15) {
      byte((uint8_t)((d << 4) | type));
    } else {
      byte((uint8_t)type);
      zigzag(id);
    }
    last.back() = id;
  }
  void i16(int16_t id, int16_t v) {
    field(id, kTI16);
    zigzag(v);
  }
  void i32(int16_t id, int32_t v) {
    field(id, kTI32);
    zigzag(v);
  }
  void i64(int16_t id, int64_t v) {
    field(id, kTI64);
    zigzag(v);
  }
  void str(int16_t id, const std::string& s) {
    field(id, kTBinary);
    varint(s.size());
    b += s;
  }
  void boolean(int16_t id, bool v) { field(id, v ? kTTrue : kTFalse); }
  void list(int16_t id, int etype, size_t n) {
    field(id, kTList);
    if (n < 15) {
      byte((uint8_t)((n << 4) | etype));
    } else {
      byte((uint8_t)(0xf0 | etype));
      varint(n);
    }
  }
  void begin(int16_t id) {  // a struct field
    field(id, kTStruct);
    last.push_back(0);
  }
  void begin_elem() { last.push_back(0); }  // a struct element of a list
  void end() {
    byte(kTStop);
    last.pop_back();
  }
};

// ---------------------------------------------------------------------------
// FileMetaData

void parse_schema_element(TIn& in, SchemaElement& e) {
  read_struct(in, [&](int16_t id, int t) {
    if (id == 1 && t == kTI32) e.type = as_i32(in);
    else if (id == 3 && t == kTI32) e.repetition = as_i32(in);
    else if (id == 4 && t == kTBinary) e.name = in.binary();
    else if (id == 5 && t == kTI32) e.num_children = as_i32(in);
    else return false;
    return true;
  });
}

void parse_column_meta(TIn& in, ColumnChunk& c) {
  read_struct(in, [&](int16_t id, int t) {
    if (id == 1 && t == kTI32) {
      c.type = as_i32(in);
    } else if (id == 3 && t == kTList) {
      read_list(in, [&](int et) {
        if (et != kTBinary) throw Error("parquet: path_in_schema is not a string list");
        c.path.push_back(in.binary());
      });
    } else if (id == 4 && t == kTI32) {
      c.codec = as_i32(in);
    } else if (id == 5 && t == kTI64) {
      c.num_values = in.zigzag();
    } else if (id == 7 && t == kTI64) {
      c.total_compressed = in.zigzag();
    } else if (id == 9 && t == kTI64) {
      c.data_page_offset = in.zigzag();
    } else if (id == 11 && t == kTI64) {
      c.dictionary_page_offset = in.zigzag();
    } else {
      return false;
    }
    return true;
  });
}

void parse_row_group(TIn& in, RowGroup& g) {
  read_struct(in, [&](int16_t id, int t) {
    if (id == 1 && t == kTList) {
      read_list(in, [&](int et) {
        if (et != kTStruct) throw Error("parquet: row group columns are not structs");
        ColumnChunk c;
        bool has_meta = false;
        read_struct(in, [&](int16_t cid, int ct) {
          if (cid == 1 && ct == kTBinary) {
            if (!in.binary().empty())
              throw Error("parquet: column chunks in other files are not supported");
            return true;
          }
          if (cid == 3 && ct == kTStruct) {
            parse_column_meta(in, c);
            has_meta = true;
            return true;
          }
          return false;
        });
        if (!has_meta) throw Error("parquet: column chunk without metadata");
        g.columns.push_back(std::move(c));
      });
    } else if (id == 3 && t == kTI64) {
      g.num_rows = in.zigzag();
    } else {
      return false;
    }
    return true;
  });
}

// ---------------------------------------------------------------------------
// JSON (just enough for the "geo" metadata)

struct JVal {
  enum Kind { kNull, kBool, kNum, kStr, kArr, kObj } kind = kNull;
  std::string s;
  std::vector<std::pair<std::string, JVal>> obj;
  std::vector<JVal> arr;
  const JVal* get(const char* k) const {
    for (auto& kv : obj)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
};

struct JParser {
  const char* p;
  const char* end;
  int depth = 0;

  [[noreturn]] void bad() { throw Error("parquet: malformed \"geo\" metadata JSON"); }
  void ws() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
  }
  bool lit(const char* w) {
    const size_t n = strlen(w);
    if ((size_t)(end - p) >= n && memcmp(p, w, n) == 0) {
      p += n;
      return true;
    }
    return false;
  }
  static void utf8(std::string& o, uint32_t c) {
    if (c < 0x80) {
      o.push_back((char)c);
    } else if (c < 0x800) {
      o.push_back((char)(0xc0 | (c >> 6)));
      o.push_back((char)(0x80 | (c & 0x3f)));
    } else if (c < 0x10000) {
      o.push_back((char)(0xe0 | (c >> 12)));
      o.push_back((char)(0x80 | ((c >> 6) & 0x3f)));
      o.push_back((char)(0x80 | (c & 0x3f)));
    } else {
      o.push_back((char)(0xf0 | (c >> 18)));
      o.push_back((char)(0x80 | ((c >> 12) & 0x3f)));
      o.push_back((char)(0x80 | ((c >> 6) & 0x3f)));
      o.push_back((char)(0x80 | (c & 0x3f)));
    }
  }
  uint32_t hex4() {
    if (end - p < 4) bad();
    uint32_t v = 0;
    for (int i = 0; i < 4; i++) {
      const char c = *p++;
      v <<= 4;
      if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
      else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
      else bad();
    }
    return v;
  }
  std::string str() {
    if (p >= end || *p != '"') bad();
    p++;
    std::string o;
    while (p < end && *p != '"') {
      if (*p != '\\') {
        o.push_back(*p++);
        continue;
      }
      if (++p >= end) bad();
      const char e = *p++;
      switch (e) {
        case '"': o.push_back('"'); break;
        case '\\': o.push_back('\\'); break;
        case '/': o.push_back('/'); break;
        case 'b': o.push_back('\b'); break;
        case 'f': o.push_back('\f'); break;
        case 'n': o.push_back('\n'); break;
        case 'r': o.push_back('\r'); break;
        case 't': o.push_back('\t'); break;
        case 'u': {
          uint32_t c = hex4();
          if (c >= 0xd800 && c < 0xdc00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
            p += 2;
            const uint32_t lo = hex4();
            if (lo < 0xdc00 || lo >= 0xe000) bad();
            c = 0x10000 + ((c - 0xd800) << 10) + (lo - 0xdc00);
          }
          utf8(o, c);
          break;
        }
        default: bad();
      }
    }
    if (p >= end) bad();
    p++;
    return o;
  }
  JVal value() {
    if (++depth > 64) bad();
    ws();
    JVal v;
    if (p >= end) bad();
    if (*p == '{') {
      p++;
      v.kind = JVal::kObj;
      ws();
      if (p < end && *p == '}') {
        p++;
      } else {
        for (;;) {
          ws();
          std::string k = str();
          ws();
          if (p >= end || *p != ':') bad();
          p++;
          JVal member = value();
          v.obj.emplace_back(std::move(k), std::move(member));
          ws();
          if (p < end && *p == ',') {
            p++;
            continue;
          }
          if (p < end && *p == '}') {
            p++;
            break;
          }
          bad();
        }
      }
    } else if (*p == '[') {
      p++;
      v.kind = JVal::kArr;
      ws();
      if (p < end && *p == ']') {
        p++;
      } else {
        for (;;) {
          v.arr.push_back(value());
          ws();
          if (p < end && *p == ',') {
            p++;
            continue;
          }
          if (p < end && *p == ']') {
            p++;
            break;
          }
          bad();
        }
      }
    } else if (*p == '"') {
      v.kind = JVal::kStr;
      v.s = str();
    } else if (lit("true") || lit("false")) {
      v.kind = JVal::kBool;
    } else if (lit("null")) {
      v.kind = JVal::kNull;
    } else {
      const char* s = p;
      while (p < end && ((*p >= '0' && *p <= '9') || *p == '+' || *p == '-' || *p == '.' ||
                         *p == 'e' || *p == 'E'))
        p++;
      if (p == s) bad();
      v.kind = JVal::kNum;
      v.s.assign(s, p);
    }
    depth--;
    return v;
  }
};

void read_geo(FileMeta& m) {
  for (auto& kv : m.kv) {
    if (kv.first != "geo") continue;
    JParser jp{kv.second.data(), kv.second.data() + kv.second.size()};
    const JVal root = jp.value();
    if (root.kind != JVal::kObj) throw Error("parquet: \"geo\" metadata is not an object");
    if (const JVal* pc = root.get("primary_column"))
      if (pc->kind == JVal::kStr) m.primary_column = pc->s;
    if (const JVal* cols = root.get("columns"))
      if (cols->kind == JVal::kObj)
        for (auto& c : cols->obj) {
          std::string enc = "WKB";
          if (const JVal* e = c.second.get("encoding"))
            if (e->kind == JVal::kStr) enc = e->s;
          m.geo_encodings.emplace_back(c.first, enc);
        }
  }
}

void collect_leaves(FileMeta& m, size_t& i, const std::string& prefix, int def, int rep,
                    int depth) {
  if (i >= m.schema.size()) throw Error("parquet: schema shorter than its children counts");
  if (depth > 64) throw Error("parquet: schema nesting too deep");
  const SchemaElement& e = m.schema[i++];
  if (e.repetition == kOptional) def++;
  if (e.repetition == kRepeated) {
    def++;
    rep++;
  }
  const std::string name = prefix.empty() ? e.name : prefix + "." + e.name;
  if (e.num_children > 0) {
    for (int c = 0; c < e.num_children; c++) collect_leaves(m, i, name, def, rep, depth + 1);
  } else {
    Leaf l;
    l.name = name;
    l.type = e.type;
    l.max_def = def;
    l.max_rep = rep;
    l.top_level = depth == 1;
    m.leaves.push_back(l);
  }
}

uint32_t le32(const uint8_t* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

}  // namespace

uint64_t parse_footer(const uint8_t* tail, uint64_t tail_len, uint64_t file_len, FileMeta& out) {
  if (file_len < 12 || tail_len < 8) throw Error("parquet: file too short");
  if (memcmp(tail + tail_len - 4, "PAR1", 4) != 0)
    throw Error("parquet: missing PAR1 magic at the end of the file");
  const uint64_t flen = le32(tail + tail_len - 8);
  if (flen + 12 > file_len) throw Error("parquet: footer length exceeds the file");
  if (flen + 8 > tail_len) return flen + 8;
  TIn in{tail + tail_len - 8 - flen, tail + tail_len - 8};
  FileMeta m;
  read_struct(in, [&](int16_t id, int t) {
    if (id == 2 && t == kTList) {
      read_list(in, [&](int et) {
        if (et != kTStruct) throw Error("parquet: schema is not a struct list");
        m.schema.emplace_back();
        parse_schema_element(in, m.schema.back());
      });
    } else if (id == 3 && t == kTI64) {
      m.num_rows = in.zigzag();
    } else if (id == 4 && t == kTList) {
      read_list(in, [&](int et) {
        if (et != kTStruct) throw Error("parquet: row groups are not structs");
        m.row_groups.emplace_back();
        parse_row_group(in, m.row_groups.back());
      });
    } else if (id == 5 && t == kTList) {
      read_list(in, [&](int et) {
        if (et != kTStruct) throw Error("parquet: key/value metadata is not a struct list");
        std::string k, v;
        read_struct(in, [&](int16_t kid, int kt) {
          if (kid == 1 && kt == kTBinary) k = in.binary();
          else if (kid == 2 && kt == kTBinary) v = in.binary();
          else return false;
          return true;
        });
        m.kv.emplace_back(std::move(k), std::move(v));
      });
    } else if (id == 6 && t == kTBinary) {
      m.created_by = in.binary();
    } else {
      return false;
    }
    return true;
  });
  if (m.schema.empty()) throw Error("parquet: empty schema");
  size_t i = 1;
  for (int c = 0; c < m.schema[0].num_children; c++) collect_leaves(m, i, "", 0, 0, 1);
  for (auto& g : m.row_groups)
    if (g.columns.size() != m.leaves.size())
      throw Error("parquet: a row group's column count differs from the schema's leaves");
  read_geo(m);
  out = std::move(m);
  return 0;
}

// ---------------------------------------------------------------------------
// page headers

bool walk_pages(const uint8_t* buf, uint64_t begin, uint64_t end, int codec, int max_def,
                int dict_index, uint64_t* row, std::vector<PageInfo>& pages) {
  return walk_pages(
      [buf, end](uint64_t pos) { return std::make_pair(buf + pos, buf + end); }, begin, end,
      codec, max_def, dict_index, row, pages, nullptr);
}

bool walk_pages(const HeaderBytes& bytes_at, uint64_t begin, uint64_t end, int codec,
                int max_def, int dict_index, uint64_t* row, std::vector<PageInfo>& pages,
                std::vector<uint64_t>* header_pos) {
  if (codec != kUncompressed && codec != kSnappy)
    throw Error("parquet: compression codec " + std::to_string(codec) +
                " is not supported (UNCOMPRESSED and SNAPPY are)");
  if (max_def > 1) throw Error("parquet: nested columns are not supported");
  uint64_t pos = begin;
  bool has_dict = false, seen_data = false;
  while (pos < end) {
    const auto hb = bytes_at(pos);
    TIn in{hb.first, hb.second};
    int type = -1;
    int32_t usize = -1, csize = -1;
    int32_t nvals = -1, enc = -1, def_enc = kRle, nnulls = 0, def_len = 0, rep_len = 0;
    bool v2_compressed = true;
    auto data_v1 = [&](int16_t f, int ft) {
      if (f == 1 && ft == kTI32) nvals = as_i32(in);
      else if (f == 2 && ft == kTI32) enc = as_i32(in);
      else if (f == 3 && ft == kTI32) def_enc = as_i32(in);
      else return false;
      return true;
    };
    auto dict_hdr = [&](int16_t f, int ft) {
      if (f == 1 && ft == kTI32) nvals = as_i32(in);
      else if (f == 2 && ft == kTI32) enc = as_i32(in);
      else return false;
      return true;
    };
    auto data_v2 = [&](int16_t f, int ft) {
      if (f == 1 && ft == kTI32) nvals = as_i32(in);
      else if (f == 2 && ft == kTI32) nnulls = as_i32(in);
      else if (f == 4 && ft == kTI32) enc = as_i32(in);
      else if (f == 5 && ft == kTI32) def_len = as_i32(in);
      else if (f == 6 && ft == kTI32) rep_len = as_i32(in);
      else if (f == 7 && (ft == kTTrue || ft == kTFalse)) v2_compressed = ft == kTTrue;
      else return false;
      return true;
    };
    read_struct(in, [&](int16_t id, int t) {
      if (id == 1 && t == kTI32) type = as_i32(in);
      else if (id == 2 && t == kTI32) usize = as_i32(in);
      else if (id == 3 && t == kTI32) csize = as_i32(in);
      else if (id == 5 && t == kTStruct) read_struct(in, data_v1, 1);
      else if (id == 7 && t == kTStruct) read_struct(in, dict_hdr, 1);
      else if (id == 8 && t == kTStruct) read_struct(in, data_v2, 1);
      else return false;
      return true;
    });
    const uint64_t hdr = (uint64_t)(in.p - hb.first);
    if (usize < 0 || csize < 0) throw Error("parquet: page header without sizes");
    const uint64_t src = pos + hdr;
    if (src + (uint64_t)csize > end) throw Error("parquet: page runs past its column chunk");
    const uint64_t page_pos = pos;
    pos = src + (uint64_t)csize;
    if (type == kIndexPage) continue;
    if (type != kDataPage && type != kDataPageV2 && type != kDictionaryPage)
      throw Error("parquet: unknown page type " + std::to_string(type));
    if (nvals < 0 || enc < 0) throw Error("parquet: page header without its page fields");
    PageInfo pg;
    pg.src = src;
    pg.src_size = (uint32_t)csize;
    pg.raw_size = (uint32_t)usize;
    pg.num_values = (uint32_t)nvals;
    pg.codec = (uint8_t)codec;
    pg.encoding = (uint8_t)enc;
    pg.max_def = (uint8_t)max_def;
    if (type == kDictionaryPage) {
      if (seen_data || has_dict) throw Error("parquet: dictionary page after other pages");
      if (enc != kPlain && enc != kPlainDictionary)
        throw Error("parquet: dictionary page encoding " + std::to_string(enc));
      pg.kind = 0;
      pg.dict = dict_index;
      has_dict = true;
    } else {
      seen_data = true;
      if (enc != kPlain && enc != kPlainDictionary && enc != kRleDictionary)
        throw Error("parquet: data page encoding " + std::to_string(enc) +
                    " is not supported (PLAIN and the dictionary encodings are)");
      if (enc != kPlain && !has_dict)
        throw Error("parquet: dictionary-encoded page without a dictionary");
      pg.dict = enc == kPlain ? -1 : dict_index;
      pg.first_row = *row;
      *row += (uint64_t)nvals;
      if (type == kDataPage) {
        if (max_def > 0 && def_enc != kRle)
          throw Error("parquet: definition levels are not RLE encoded");
        pg.kind = 1;
      } else {
        if (rep_len != 0) throw Error("parquet: repetition levels in a flat column");
        if (def_len < 0 || def_len > csize || def_len > usize)
          throw Error("parquet: bad level lengths in a v2 page header");
        if (max_def == 0 && (def_len != 0 || nnulls != 0))
          throw Error("parquet: levels in a required column");
        pg.kind = 2;
        pg.lvl_bytes = (uint32_t)def_len;
        pg.def_len = (uint32_t)def_len;
        if (!v2_compressed) pg.codec = kUncompressed;
      }
    }
    pg.in_src = pg.codec == kUncompressed;
    if (pg.in_src && pg.raw_size != pg.src_size)
      throw Error("parquet: stored page whose sizes differ");
    pages.push_back(pg);
    if (header_pos) header_pos->push_back(page_pos);
  }
  if (pos != end) throw Error("parquet: column chunk size disagrees with its pages");
  return has_dict;
}

// ---------------------------------------------------------------------------
// Snappy block compression: greedy matching over 64 KiB blocks with a hash
// table of 4-byte sequences (multiplicative hashing by 2^32 / golden ratio).

namespace {

void put_varint(std::string& o, uint64_t v) {
  while (v >= 0x80) {
    o.push_back((char)(v | 0x80));
    v >>= 7;
  }
  o.push_back((char)v);
}

void emit_literal(std::string& o, const uint8_t* s, size_t len) {
  if (len == 0) return;
  const uint64_t m = len - 1;
  if (m < 60) {
    o.push_back((char)(m << 2));
  } else {
    const int nb = m < (1u << 8) ? 1 : m < (1u << 16) ? 2 : m < (1u << 24) ? 3 : 4;
    o.push_back((char)((59 + nb) << 2));
    for (int i = 0; i < nb; i++) o.push_back((char)(m >> (8 * i)));
  }
  o.append(reinterpret_cast<const char*>(s), len);
}

void emit_copy(std::string& o, uint32_t off, size_t len) {
  while (len) {
    size_t l = len > 64 ? 64 : len;
    if (len > 64 && len - 64 < 4) l = len - 4;  // leave a tail of 4 or more
    if (l >= 4 && l <= 11 && off < 2048) {
      o.push_back((char)(1 | ((l - 4) << 2) | ((off >> 8) << 5)));
      o.push_back((char)(off & 0xff));
    } else {
      o.push_back((char)(2 | ((l - 1) << 2)));
      o.push_back((char)(off & 0xff));
      o.push_back((char)(off >> 8));
    }
    len -= l;
  }
}

}  // namespace

void snappy_compress(const uint8_t* in, size_t n, std::string& out) {
  out.clear();
  put_varint(out, n);
  constexpr size_t kBlock = 1 << 16;
  constexpr int kHashBits = 14;
  std::vector<int32_t> table(1 << kHashBits);
  for (size_t b0 = 0; b0 < n; b0 += kBlock) {
    const size_t b1 = std::min(n, b0 + kBlock);
    std::fill(table.begin(), table.end(), -1);
    size_t ip = b0, lit = b0;
    while (ip + 4 <= b1) {
      uint32_t v;
      memcpy(&v, in + ip, 4);
      const uint32_t h = (v * 2654435761u) >> (32 - kHashBits);
      const int32_t cand = table[h];
      table[h] = (int32_t)(ip - b0);
      if (cand >= 0) {
        const size_t c = b0 + (size_t)cand;
        uint32_t w;
        memcpy(&w, in + c, 4);
        if (w == v) {
          size_t len = 4;
          while (ip + len < b1 && in[c + len] == in[ip + len]) len++;
          emit_literal(out, in + lit, ip - lit);
          emit_copy(out, (uint32_t)(ip - c), len);
          ip += len;
          lit = ip;
          continue;
        }
      }
      ip++;
    }
    emit_literal(out, in + lit, b1 - lit);
  }
}

// ---------------------------------------------------------------------------
// writer

namespace {

// RLE runs (bit width 1) of the definition levels of rows [r0, r1)
template <class Valid>
std::string def_levels(Valid&& valid, int64_t r0, int64_t r1) {
  std::string o;
  int64_t r = r0;
  while (r < r1) {
    const bool v = valid(r);
    int64_t e = r + 1;
    while (e < r1 && valid(e) == v) e++;
    put_varint(o, (uint64_t)(e - r) << 1);
    o.push_back((char)(v ? 1 : 0));
    r = e;
  }
  return o;
}

void put_le32(std::string& o, uint32_t v) {
  for (int i = 0; i < 4; i++) o.push_back((char)(v >> (8 * i)));
}

struct FileOut {
  int fd = -1;
  uint64_t pos = 0;
  explicit FileOut(const char* path) {
    fd = ::open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) throw Error(std::string("parquet: cannot create ") + path);
  }
  ~FileOut() {
    if (fd >= 0) ::close(fd);
  }
  void write(const void* p, size_t n) {
    const char* c = static_cast<const char*>(p);
    while (n) {
      const ssize_t w = ::write(fd, c, n);
      if (w <= 0) throw Error("parquet: write failed");
      c += w;
      n -= (size_t)w;
      pos += (uint64_t)w;
    }
  }
  void write(const std::string& s) { write(s.data(), s.size()); }
};

std::string json_escape(const std::string& s) {
  std::string o;
  for (unsigned char c : s) {
    if (c == '"' || c == '\\') {
      o.push_back('\\');
      o.push_back((char)c);
    } else if (c < 0x20) {
      char b[8];
      snprintf(b, sizeof b, "\\u%04x", c);
      o += b;
    } else {
      o.push_back((char)c);
    }
  }
  return o;
}

}  // namespace

void write_wkb(const char* path, const char* column, int64_t n, const void* offsets,
               bool offsets64, const uint8_t* data, const uint8_t* validity,
               int64_t validity_offset, const WriteOptions& opt) {
  SPJ_CHECK(path && column && *column, "null path or column name");
  SPJ_CHECK(n >= 0 && (n == 0 || offsets), "null offsets");
  SPJ_CHECK(opt.compression == 0 || opt.compression == 1, "compression must be 0 or 1");
  SPJ_CHECK(opt.page_version == 1 || opt.page_version == 2, "page_version must be 1 or 2");
  SPJ_CHECK(opt.row_group_rows > 0 && opt.page_bytes > 0, "sizes must be positive");
  auto off = [&](int64_t i) -> uint64_t {
    return offsets64 ? (uint64_t) static_cast<const int64_t*>(offsets)[i]
                     : (uint64_t)(uint32_t) static_cast<const int32_t*>(offsets)[i];
  };
  auto valid = [&](int64_t i) {
    if (!validity) return true;
    const int64_t b = validity_offset + i;
    return ((validity[b >> 3] >> (b & 7)) & 1) != 0;
  };
  FileOut f(path);
  f.write("PAR1", 4);
  struct ChunkOut {
    int64_t rows, start, usize, csize;
  };
  std::vector<ChunkOut> chunks;
  std::string body, values, comp, lv;
  for (int64_t g0 = 0; g0 < n; g0 += opt.row_group_rows) {
    const int64_t g1 = std::min(n, g0 + opt.row_group_rows);
    ChunkOut ck{g1 - g0, (int64_t)f.pos, 0, 0};
    for (int64_t r = g0; r < g1;) {
      // one page: rows until page_bytes of values (at least one row)
      values.clear();
      int64_t e = r, nulls = 0;
      while (e < g1 && (e == r || (int64_t)values.size() < opt.page_bytes)) {
        if (valid(e)) {
          const uint64_t s = off(e), t = off(e + 1);
          SPJ_CHECK(t >= s, "offsets decrease at row " + std::to_string(e));
          SPJ_CHECK(t - s < (1ull << 32), "value larger than 4 GiB at row " + std::to_string(e));
          put_le32(values, (uint32_t)(t - s));
          values.append(reinterpret_cast<const char*>(data + s), t - s);
        } else {
          nulls++;
        }
        e++;
      }
      lv = def_levels(valid, r, e);
      uint64_t usize, csize;
      if (opt.page_version == 1) {
        body.clear();
        put_le32(body, (uint32_t)lv.size());
        body += lv;
        body += values;
        usize = body.size();
        if (opt.compression) {
          snappy_compress(reinterpret_cast<const uint8_t*>(body.data()), body.size(), comp);
          body.swap(comp);
        }
        csize = body.size();
      } else {
        if (opt.compression)
          snappy_compress(reinterpret_cast<const uint8_t*>(values.data()), values.size(), comp);
        else
          comp = values;
        body = lv + comp;
        usize = lv.size() + values.size();
        csize = body.size();
      }
      SPJ_CHECK(usize < (1ull << 31) && csize < (1ull << 31), "page larger than 2 GiB");
      TOut h;
      h.i32(1, opt.page_version == 1 ? kDataPage : kDataPageV2);
      h.i32(2, (int32_t)usize);
      h.i32(3, (int32_t)csize);
      if (opt.page_version == 1) {
        h.begin(5);
        h.i32(1, (int32_t)(e - r));
        h.i32(2, kPlain);
        h.i32(3, kRle);
        h.i32(4, kRle);
        h.end();
      } else {
        h.begin(8);
        h.i32(1, (int32_t)(e - r));
        h.i32(2, (int32_t)nulls);
        h.i32(3, (int32_t)(e - r));
        h.i32(4, kPlain);
        h.i32(5, (int32_t)lv.size());
        h.i32(6, 0);
        h.boolean(7, opt.compression != 0);
        h.end();
      }
      h.byte(kTStop);
      f.write(h.b);
      f.write(body);
      ck.usize += (int64_t)(h.b.size() + usize);
      ck.csize += (int64_t)(h.b.size() + csize);
      r = e;
    }
    chunks.push_back(ck);
  }
  // footer (FileMetaData)
  TOut m;
  m.i32(1, 1);
  m.list(2, kTStruct, 2);
  m.begin_elem();
  m.str(4, "schema");
  m.i32(5, 1);
  m.end();
  m.begin_elem();
  m.i32(1, kByteArray);
  m.i32(3, kOptional);
  m.str(4, column);
  m.end();
  m.i64(3, n);
  m.list(4, kTStruct, chunks.size());
  int16_t ordinal = 0;
  for (auto& ck : chunks) {
    m.begin_elem();
    m.list(1, kTStruct, 1);
    m.begin_elem();
    m.i64(2, ck.start);
    m.begin(3);
    m.i32(1, kByteArray);
    m.list(2, kTI32, 2);
    m.zigzag(kPlain);
    m.zigzag(kRle);
    m.list(3, kTBinary, 1);
    m.varint(strlen(column));
    m.b += column;
    m.i32(4, opt.compression ? kSnappy : kUncompressed);
    m.i64(5, ck.rows);
    m.i64(6, ck.usize);
    m.i64(7, ck.csize);
    m.i64(9, ck.start);
    m.end();
    m.end();
    m.i64(2, ck.usize);
    m.i64(3, ck.rows);
    m.i64(5, ck.start);
    m.i64(6, ck.csize);
    m.i16(7, ordinal++);
    m.end();
  }
  const std::string col = json_escape(column);
  const std::string geo = "{\"version\": \"1.1.0\", \"primary_column\": \"" + col +
                          "\", \"columns\": {\"" + col +
                          "\": {\"encoding\": \"WKB\", \"geometry_types\": []}}}";
  m.list(5, kTStruct, 1);
  m.begin_elem();
  m.str(1, "geo");
  m.str(2, geo);
  m.end();
  m.str(6, "sedona-db_gb300 GeoParquet writer");
  m.byte(kTStop);
  f.write(m.b);
  std::string tail;
  put_le32(tail, (uint32_t)m.b.size());
  tail += "PAR1";
  f.write(tail);
}

}  // namespace pq
}  // namespace spj
