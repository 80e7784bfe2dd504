/*
 * spj_parquet.c — CPU oracle for the GeoParquet read path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the device reader
 * (SpjParquetReadWkb).  Only tests/ and bench.py's cpu_baseline / reference
 * legs load it.
 *
 * The reference reads GeoParquet through the `parquet` crate (arrow-rs,
 * version 57.3.0 in the reference's Cargo.lock:4595-4596; a third-party
 * dependency that is not part of the reference tree), from
 * rust/sedona-geoparquet/src/file_opener.rs.  This file restates what that
 * reader does for a flat BYTE_ARRAY column, from the published Parquet format
 * (parquet.thrift field ids, the Thrift compact protocol, RLE / bit-packed
 * hybrid levels, PLAIN and dictionary encodings, data pages v1 and v2) and
 * the published Snappy block format, one page after another on one thread.
 * It is pinned against pyarrow (Arrow's C++ reader) on the committed fixtures
 * and on the reference's own GeoParquet test files.
 */
#include <setjmp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "spj_oracle.h"

typedef struct {
  const uint8_t* p;
  const uint8_t* end;
  jmp_buf* fail;
} rd_t;

static void need(rd_t* r, uint64_t n) {
  if ((uint64_t)(r->end - r->p) < n) longjmp(*r->fail, 1);
}
static uint8_t rbyte(rd_t* r) {
  need(r, 1);
  return *r->p++;
}
static uint64_t rvarint(rd_t* r) {
  uint64_t v = 0;
  for (int sh = 0; sh < 64; sh += 7) {
    uint8_t b = rbyte(r);
    v |= (uint64_t)(b & 0x7f) << sh;
    if (!(b & 0x80)) return v;
  }
  longjmp(*r->fail, 1);
}
static int64_t rzz(rd_t* r) {
  uint64_t v = rvarint(r);
  return (int64_t)(v >> 1) ^ -(int64_t)(v & 1);
}
static void rbin(rd_t* r, const uint8_t** s, uint64_t* n) {
  *n = rvarint(r);
  need(r, *n);
  *s = r->p;
  r->p += *n;
}

/* Thrift compact: field headers and skipping */
static int rfield(rd_t* r, int16_t* last, int16_t* id) {
  uint8_t h = rbyte(r);
  if (h == 0) return -1;
  int d = h >> 4;
  *id = d ? (int16_t)(*last + d) : (int16_t)rzz(r);
  *last = *id;
  return h & 0x0f;
}
static void rskip(rd_t* r, int t, int depth);
static void rskip_struct(rd_t* r, int depth) {
  int16_t last = 0, id;
  int t;
  while ((t = rfield(r, &last, &id)) >= 0) rskip(r, t, depth + 1);
}
static void rskip(rd_t* r, int t, int depth) {
  if (depth > 32) longjmp(*r->fail, 1);
  const uint8_t* s;
  uint64_t n;
  switch (t) {
    case 1: case 2: return;
    case 3: need(r, 1); r->p++; return;
    case 4: case 5: case 6: rvarint(r); return;
    case 7: need(r, 8); r->p += 8; return;
    case 8: rbin(r, &s, &n); return;
    case 9: case 10: {
      uint8_t h = rbyte(r);
      uint64_t cnt = h >> 4;
      int et = h & 15;
      if (cnt == 15) cnt = rvarint(r);
      for (uint64_t i = 0; i < cnt; i++) {
        if (et == 1 || et == 2) { need(r, 1); r->p++; } else rskip(r, et, depth + 1);
      }
      return;
    }
    case 11: {
      uint64_t cnt = rvarint(r);
      if (!cnt) return;
      uint8_t kv = rbyte(r);
      for (uint64_t i = 0; i < cnt; i++) { rskip(r, kv >> 4, depth + 1); rskip(r, kv & 15, depth + 1); }
      return;
    }
    case 12: rskip_struct(r, depth); return;
    default: longjmp(*r->fail, 1);
  }
}
static uint64_t rlist(rd_t* r, int* et) {
  uint8_t h = rbyte(r);
  uint64_t cnt = h >> 4;
  *et = h & 15;
  if (cnt == 15) cnt = rvarint(r);
  if (cnt > (uint64_t)(r->end - r->p)) longjmp(*r->fail, 1);
  return cnt;
}

typedef struct {
  int type, rep, nchild;
  char name[256];
} sel_t;
typedef struct {
  int64_t num_values, total_compressed, data_off, dict_off;
  int codec, type;
} chunk_t;

typedef struct {
  /* growing outputs */
  int64_t* off;
  uint8_t* data;
  uint8_t* valid;
  int64_t n, cap_rows;
  uint64_t nbytes, cap_bytes;
} out_t;

static void out_row(out_t* o, const uint8_t* v, uint32_t len, int ok, jmp_buf* fail) {
  if (o->n + 1 >= o->cap_rows) {
    o->cap_rows = o->cap_rows ? o->cap_rows * 2 : 1024;
    o->off = realloc(o->off, sizeof(int64_t) * (size_t)(o->cap_rows + 1));
    o->valid = realloc(o->valid, (size_t)o->cap_rows);
    if (!o->off || !o->valid) longjmp(*fail, 2);
  }
  if (ok && len) {
    if (o->nbytes + len > o->cap_bytes) {
      while (o->nbytes + len > o->cap_bytes) o->cap_bytes = o->cap_bytes ? o->cap_bytes * 2 : 4096;
      o->data = realloc(o->data, o->cap_bytes);
      if (!o->data) longjmp(*fail, 2);
    }
    memcpy(o->data + o->nbytes, v, len);
    o->nbytes += len;
  }
  o->valid[o->n] = (uint8_t)ok;
  o->n++;
  o->off[o->n] = (int64_t)o->nbytes;
}

/* Snappy block decompression (one element after another). */
static int unsnap(const uint8_t* in, uint64_t n, uint8_t* out, uint64_t out_n) {
  const uint8_t* ip = in;
  const uint8_t* end = in + n;
  uint64_t ulen = 0;
  for (int sh = 0;; sh += 7) {
    if (ip >= end || sh > 35) return -1;
    uint8_t b = *ip++;
    ulen |= (uint64_t)(b & 0x7f) << sh;
    if (!(b & 0x80)) break;
  }
  if (ulen != out_n) return -1;
  uint64_t op = 0;
  while (ip < end) {
    uint8_t tag = *ip++;
    uint64_t len, off;
    switch (tag & 3) {
      case 0:
        len = (uint64_t)(tag >> 2) + 1;
        if (len > 60) {
          int nb = (int)len - 60;
          if (end - ip < nb) return -1;
          len = 0;
          for (int b = 0; b < nb; b++) len |= (uint64_t)ip[b] << (8 * b);
          len += 1;
          ip += nb;
        }
        if ((uint64_t)(end - ip) < len || op + len > out_n) return -1;
        memcpy(out + op, ip, len);
        ip += len;
        op += len;
        continue;
      case 1:
        if (end - ip < 1) return -1;
        len = ((tag >> 2) & 7) + 4;
        off = ((uint64_t)(tag >> 5) << 8) | ip[0];
        ip += 1;
        break;
      case 2:
        if (end - ip < 2) return -1;
        len = (uint64_t)(tag >> 2) + 1;
        off = ip[0] | ((uint64_t)ip[1] << 8);
        ip += 2;
        break;
      default:
        if (end - ip < 4) return -1;
        len = (uint64_t)(tag >> 2) + 1;
        off = ip[0] | ((uint64_t)ip[1] << 8) | ((uint64_t)ip[2] << 16) | ((uint64_t)ip[3] << 24);
        ip += 4;
        break;
    }
    if (off == 0 || off > op || op + len > out_n) return -1;
    for (uint64_t i = 0; i < len; i++) out[op + i] = out[op - off + i];  /* byte order repeats */
    op += len;
  }
  return op == out_n ? 0 : -1;
}

/* RLE / bit-packed hybrid: count values of width bw into vals */
static int rle_hybrid(const uint8_t* p, const uint8_t* end, int bw, uint32_t count, uint32_t* vals) {
  uint32_t i = 0;
  int vb = (bw + 7) / 8;
  while (i < count) {
    uint64_t h = 0;
    for (int sh = 0;; sh += 7) {
      if (p >= end || sh > 63) return -1;
      uint8_t b = *p++;
      h |= (uint64_t)(b & 0x7f) << sh;
      if (!(b & 0x80)) break;
    }
    if (h & 1) {
      uint64_t nv = (h >> 1) * 8;
      if (nv == 0) return -1;
      for (uint64_t k = 0; k < nv && i < count; k++, i++) {
        uint32_t v = 0;
        for (int b = 0; b < bw; b++) {
          uint64_t bit = k * (uint64_t)bw + (uint64_t)b;
          if (p + bit / 8 >= end) return -1;
          v |= (uint32_t)((p[bit / 8] >> (bit % 8)) & 1) << b;
        }
        vals[i] = v;
      }
      uint64_t nb = (h >> 1) * (uint64_t)bw;
      p = (uint64_t)(end - p) < nb ? end : p + nb;
    } else {
      uint64_t run = h >> 1;
      if (run == 0 || end - p < vb) return -1;
      uint32_t v = 0;
      for (int b = 0; b < vb; b++) v |= (uint32_t)p[b] << (8 * b);
      p += vb;
      for (uint64_t k = 0; k < run && i < count; k++) vals[i++] = v;
    }
  }
  return 0;
}

static uint32_t le32(const uint8_t* p) {
  return p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

/* find "primary_column": "<name>" in the geo JSON */
static int geo_primary(const uint8_t* s, uint64_t n, char* name, size_t cap) {
  const char key[] = "\"primary_column\"";
  for (uint64_t i = 0; i + sizeof key - 1 <= n; i++) {
    if (memcmp(s + i, key, sizeof key - 1)) continue;
    uint64_t j = i + sizeof key - 1;
    while (j < n && (s[j] == ' ' || s[j] == ':' || s[j] == '\n' || s[j] == '\t')) j++;
    if (j >= n || s[j] != '"') return -1;
    j++;
    size_t k = 0;
    while (j < n && s[j] != '"' && k + 1 < cap) {
      if (s[j] == '\\' && j + 1 < n) j++;
      name[k++] = (char)s[j++];
    }
    name[k] = 0;
    return 0;
  }
  return -1;
}

typedef struct {
  uint8_t* file;
  long flen;
  uint8_t* page;
  uint32_t* lv;
  uint32_t* ix;
  uint64_t* dict_off;
  uint32_t* dict_len;
  uint8_t* dict_store;
  sel_t* schema;
  chunk_t* chunks;
  int64_t* group_rows;
  out_t o;
  const char* why;
} pctx_t;

#define FAIL(msg) do { c->why = (msg); longjmp(*fail, 1); } while (0)

/* Every step that can fail runs here.  All allocations live in *c (heap
 * memory), so the caller frees them after a longjmp out of this function. */
static void parse_file(pctx_t* c, jmp_buf* fail, const char* column) {
  const uint8_t* file = c->file;
  const long flen = c->flen;
  if (flen < 12 || memcmp(file + flen - 4, "PAR1", 4)) FAIL("not a Parquet file");
  uint32_t mlen = le32(file + flen - 8);
  if ((uint64_t)mlen + 12 > (uint64_t)flen) FAIL("footer length exceeds the file");
  rd_t r = {file + flen - 8 - mlen, file + flen - 8, fail};
  int nschema = 0, ngroups = 0, ncols_total = 0, chunk_cap = 0;
  int16_t last = 0, id;
  int t;
  char primary[256] = {0};
  while ((t = rfield(&r, &last, &id)) >= 0) {
    if (id == 2 && t == 9) {
      int et;
      uint64_t cnt = rlist(&r, &et);
      c->schema = calloc(cnt ? cnt : 1, sizeof(sel_t));
      if (!c->schema) longjmp(*fail, 2);
      for (uint64_t i = 0; i < cnt; i++) {
        sel_t* e = &c->schema[nschema++];
        e->type = e->rep = -1;
        int16_t l2 = 0, f2;
        int t2;
        while ((t2 = rfield(&r, &l2, &f2)) >= 0) {
          const uint8_t* sp;
          uint64_t n;
          if (f2 == 1 && t2 == 5) e->type = (int)rzz(&r);
          else if (f2 == 3 && t2 == 5) e->rep = (int)rzz(&r);
          else if (f2 == 5 && t2 == 5) e->nchild = (int)rzz(&r);
          else if (f2 == 4 && t2 == 8) {
            rbin(&r, &sp, &n);
            size_t k = n < sizeof e->name - 1 ? n : sizeof e->name - 1;
            memcpy(e->name, sp, k);
            e->name[k] = 0;
          } else rskip(&r, t2, 1);
        }
      }
    } else if (id == 4 && t == 9) {
      int et;
      uint64_t cnt = rlist(&r, &et);
      c->group_rows = calloc(cnt ? cnt : 1, sizeof(int64_t));
      if (!c->group_rows) longjmp(*fail, 2);
      for (uint64_t g = 0; g < cnt; g++) {
        int16_t l2 = 0, f2;
        int t2;
        while ((t2 = rfield(&r, &l2, &f2)) >= 0) {
          if (f2 == 1 && t2 == 9) {
            int et2;
            uint64_t nc = rlist(&r, &et2);
            for (uint64_t k = 0; k < nc; k++) {
              if (ncols_total == chunk_cap) {
                chunk_cap = chunk_cap ? chunk_cap * 2 : 16;
                chunk_t* grown = realloc(c->chunks, sizeof(chunk_t) * (size_t)chunk_cap);
                if (!grown) longjmp(*fail, 2);
                c->chunks = grown;
              }
              chunk_t* ck = &c->chunks[ncols_total++];
              memset(ck, 0, sizeof *ck);
              ck->dict_off = -1;
              int16_t l3 = 0, f3;
              int t3;
              while ((t3 = rfield(&r, &l3, &f3)) >= 0) {
                if (f3 == 3 && t3 == 12) {
                  int16_t l4 = 0, f4;
                  int t4;
                  while ((t4 = rfield(&r, &l4, &f4)) >= 0) {
                    if (f4 == 1 && t4 == 5) ck->type = (int)rzz(&r);
                    else if (f4 == 4 && t4 == 5) ck->codec = (int)rzz(&r);
                    else if (f4 == 5 && t4 == 6) ck->num_values = rzz(&r);
                    else if (f4 == 7 && t4 == 6) ck->total_compressed = rzz(&r);
                    else if (f4 == 9 && t4 == 6) ck->data_off = rzz(&r);
                    else if (f4 == 11 && t4 == 6) ck->dict_off = rzz(&r);
                    else rskip(&r, t4, 2);
                  }
                } else rskip(&r, t3, 2);
              }
            }
          } else if (f2 == 3 && t2 == 6) {
            c->group_rows[g] = rzz(&r);
          } else rskip(&r, t2, 1);
        }
        ngroups++;
      }
    } else if (id == 5 && t == 9) {
      int et;
      uint64_t cnt = rlist(&r, &et);
      for (uint64_t i = 0; i < cnt; i++) {
        int16_t l2 = 0, f2;
        int t2;
        const uint8_t *k = NULL, *v = NULL;
        uint64_t kn = 0, vn = 0;
        while ((t2 = rfield(&r, &l2, &f2)) >= 0) {
          if (f2 == 1 && t2 == 8) rbin(&r, &k, &kn);
          else if (f2 == 2 && t2 == 8) rbin(&r, &v, &vn);
          else rskip(&r, t2, 1);
        }
        if (k && kn == 3 && !memcmp(k, "geo", 3) && v) geo_primary(v, vn, primary, sizeof primary);
      }
    } else {
      rskip(&r, t, 0);
    }
  }
  if (nschema < 1) FAIL("empty schema");
  /* the column: a direct child of the root with no children */
  const char* want = column ? column : primary;
  int col = -1, leaf = 0, max_def = 0;
  int i = 1;
  for (int ch = 0; ch < c->schema[0].nchild && i < nschema; ch++) {
    int pending = 1, first = i, leaves_here = 0;
    while (pending > 0 && i < nschema) {
      pending--;
      if (c->schema[i].nchild > 0) pending += c->schema[i].nchild;
      else leaves_here++;
      i++;
    }
    if (c->schema[first].nchild == 0 && !strcmp(c->schema[first].name, want)) {
      if (c->schema[first].rep == 2 || c->schema[first].type != 6) FAIL("unsupported column");
      col = leaf;
      max_def = c->schema[first].rep == 1 ? 1 : 0;
    }
    leaf += leaves_here;
  }
  const int leaf_cols = leaf;
  if (col < 0) FAIL("no such column");
  if (ncols_total != ngroups * leaf_cols) FAIL("row group column counts differ from the schema");
  for (int g = 0; g < ngroups; g++) {
    chunk_t* ck = &c->chunks[g * leaf_cols + col];
    if (ck->codec != 0 && ck->codec != 1) FAIL("unsupported codec");
    int64_t start = ck->data_off;
    if (ck->dict_off > 0 && ck->dict_off < start) start = ck->dict_off;
    if (start < 4 || ck->total_compressed < 0 || start + ck->total_compressed > flen)
      FAIL("column chunk outside the file");
    const uint8_t* p = file + start;
    const uint8_t* cend = p + ck->total_compressed;
    uint64_t ndict = 0;
    int have_dict = 0;
    int64_t rows_left = c->group_rows[g];
    while (p < cend) {
      rd_t h = {p, cend, fail};
      int16_t l2 = 0, f2;
      int t2, ptype = -1, nvals = -1, enc = -1, def_len = 0, rep_len = 0, v2c = 1;
      int64_t usize = -1, csize = -1;
      while ((t2 = rfield(&h, &l2, &f2)) >= 0) {
        if (f2 == 1 && t2 == 5) ptype = (int)rzz(&h);
        else if (f2 == 2 && t2 == 5) usize = rzz(&h);
        else if (f2 == 3 && t2 == 5) csize = rzz(&h);
        else if ((f2 == 5 || f2 == 7 || f2 == 8) && t2 == 12) {
          int16_t l3 = 0, f3;
          int t3;
          while ((t3 = rfield(&h, &l3, &f3)) >= 0) {
            if (f3 == 1 && t3 == 5) nvals = (int)rzz(&h);
            else if (f2 != 8 && f3 == 2 && t3 == 5) enc = (int)rzz(&h);
            else if (f2 == 8 && f3 == 4 && t3 == 5) enc = (int)rzz(&h);
            else if (f2 == 8 && f3 == 5 && t3 == 5) def_len = (int)rzz(&h);
            else if (f2 == 8 && f3 == 6 && t3 == 5) rep_len = (int)rzz(&h);
            else if (f2 == 8 && f3 == 7 && (t3 == 1 || t3 == 2)) v2c = t3 == 1;
            else rskip(&h, t3, 2);
          }
        } else rskip(&h, t2, 1);
      }
      if (usize < 0 || csize < 0 || csize > cend - h.p) FAIL("page runs past its chunk");
      const uint8_t* body = h.p;
      p = h.p + csize;
      if (ptype == 1) continue;
      if (nvals < 0 || enc < 0 || rep_len != 0 || def_len < 0 || def_len > csize ||
          def_len > usize)
        FAIL("bad page header");
      const int lvl = ptype == 3 ? def_len : 0;
      const int comp = ck->codec == 1 && (ptype != 3 || v2c);
      uint8_t* page = malloc((size_t)usize + 1);
      if (!page) longjmp(*fail, 2);
      free(c->page);
      c->page = page;
      memcpy(page, body, (size_t)lvl);
      if (comp) {
        if (unsnap(body + lvl, (uint64_t)(csize - lvl), page + lvl, (uint64_t)(usize - lvl)))
          FAIL("malformed Snappy data");
      } else {
        if (usize != csize) FAIL("stored page whose sizes differ");
        memcpy(page + lvl, body + lvl, (size_t)(usize - lvl));
      }
      if (ptype == 2) {
        /* dictionary: keep its bytes and the entries' spans */
        free(c->dict_store);
        c->dict_store = page;
        c->page = NULL;
        ndict = (uint64_t)nvals;
        free(c->dict_off);
        free(c->dict_len);
        c->dict_off = malloc(sizeof(uint64_t) * (ndict + 1));
        c->dict_len = malloc(sizeof(uint32_t) * (ndict + 1));
        if (!c->dict_off || !c->dict_len) longjmp(*fail, 2);
        uint64_t q = 0;
        for (uint64_t k = 0; k < ndict; k++) {
          if (q + 4 > (uint64_t)usize) FAIL("malformed dictionary page");
          uint32_t l = le32(c->dict_store + q);
          if (q + 4 + l > (uint64_t)usize) FAIL("malformed dictionary page");
          c->dict_off[k] = q + 4;
          c->dict_len[k] = l;
          q += 4 + l;
        }
        have_dict = 1;
        continue;
      }
      if (ptype != 0 && ptype != 3) FAIL("unknown page type");
      /* definition levels */
      free(c->lv);
      c->lv = malloc(sizeof(uint32_t) * ((size_t)nvals + 1));
      if (!c->lv) longjmp(*fail, 2);
      uint32_t* lv = c->lv;
      const uint8_t* vp = page;
      const uint8_t* pend = page + usize;
      if (max_def == 0) {
        for (int k = 0; k < nvals; k++) lv[k] = 1;
      } else if (ptype == 0) {
        if (usize < 4 || le32(page) > (uint64_t)usize - 4) FAIL("malformed levels");
        uint32_t L = le32(page);
        if (rle_hybrid(page + 4, page + 4 + L, 1, (uint32_t)nvals, lv)) FAIL("malformed levels");
        vp = page + 4 + L;
      } else {
        if (rle_hybrid(page, page + def_len, 1, (uint32_t)nvals, lv)) FAIL("malformed levels");
        vp = page + lvl;
      }
      uint32_t m = 0;
      for (int k = 0; k < nvals; k++) m += lv[k] ? 1 : 0;
      if (enc == 0) {
        for (int k = 0; k < nvals; k++) {
          if (!lv[k]) {
            out_row(&c->o, NULL, 0, 0, fail);
            continue;
          }
          if (pend - vp < 4) FAIL("PLAIN values run past the page");
          uint32_t l = le32(vp);
          if ((uint64_t)(pend - vp - 4) < l) FAIL("PLAIN values run past the page");
          out_row(&c->o, vp + 4, l, 1, fail);
          vp += 4 + l;
        }
      } else if (enc == 2 || enc == 8) {
        if (!have_dict) FAIL("dictionary-encoded page without a dictionary");
        free(c->ix);
        c->ix = malloc(sizeof(uint32_t) * ((size_t)m + 1));
        if (!c->ix) longjmp(*fail, 2);
        if (m) {
          if (pend - vp < 1 || vp[0] > 32) FAIL("malformed dictionary indices");
          if (rle_hybrid(vp + 1, pend, vp[0], m, c->ix)) FAIL("malformed dictionary indices");
        }
        uint32_t k2 = 0;
        for (int k = 0; k < nvals; k++) {
          if (!lv[k]) {
            out_row(&c->o, NULL, 0, 0, fail);
            continue;
          }
          uint32_t d = c->ix[k2++];
          if (d >= ndict) FAIL("dictionary index out of range");
          out_row(&c->o, c->dict_store + c->dict_off[d], c->dict_len[d], 1, fail);
        }
      } else {
        FAIL("unsupported encoding");
      }
      rows_left -= nvals;
    }
    if (rows_left != 0) FAIL("page values disagree with the row group's rows");
  }
}

int spjo_parquet_read(const char* path, const char* column, int64_t* n_rows, int64_t** offsets,
                      uint8_t** data, uint8_t** valid, char* err, int errcap) {
  pctx_t* c = calloc(1, sizeof(pctx_t));
  if (!c) {
    snprintf(err, errcap, "out of memory");
    return -1;
  }
  int rc = 0;
  FILE* f = fopen(path, "rb");
  if (!f) {
    snprintf(err, errcap, "cannot open %s", path);
    free(c);
    return -1;
  }
  fseek(f, 0, SEEK_END);
  c->flen = ftell(f);
  fseek(f, 0, SEEK_SET);
  c->file = malloc(c->flen > 0 ? (size_t)c->flen : 1);
  if (!c->file || c->flen < 0 || fread(c->file, 1, (size_t)c->flen, f) != (size_t)c->flen) {
    snprintf(err, errcap, "cannot read %s", path);
    rc = -1;
  }
  fclose(f);
  jmp_buf fail;
  if (rc == 0) {
    c->why = "malformed Parquet file";
    int code = setjmp(fail);
    if (code == 0) {
      parse_file(c, &fail, column);
      if (!c->o.off) {
        c->o.off = calloc(1, sizeof(int64_t));
        c->o.valid = malloc(1);
      }
      c->o.off[0] = 0;
      *n_rows = c->o.n;
      *offsets = c->o.off;
      *data = c->o.data ? c->o.data : malloc(1);
      *valid = c->o.valid;
      c->o.off = NULL;
      c->o.data = NULL;
      c->o.valid = NULL;
    } else {
      snprintf(err, errcap, "%s", code == 2 ? "out of memory" : c->why);
      rc = -1;
    }
  }
  free(c->file);
  free(c->page);
  free(c->lv);
  free(c->ix);
  free(c->dict_off);
  free(c->dict_len);
  free(c->dict_store);
  free(c->schema);
  free(c->chunks);
  free(c->group_rows);
  free(c->o.off);
  free(c->o.data);
  free(c->o.valid);
  free(c);
  return rc;
}
