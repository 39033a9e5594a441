// gb_parquet.cu — Parquet row groups straight into the GROUP BY on GB300.
//
// Host: the footer and every page header are parsed from the file bytes
// (thrift compact protocol) into a page index — the GPU-side restatement of
// ParquetReader's metadata walk (src/storage/parquet.cpp:92-184 ThriftRd,
// 187-382 / 1107-1366 metadata, 385-470 page headers, 2475-2706
// ReadColumnInto's page loop).
//
// Device, per batch of row groups:
//   k_pq_runs   one CTA per dictionary-encoded data page: the page is staged in
//               shared memory and its RLE / bit-packed run headers are walked
//               into a run table (RleDecoder::FetchRun, parquet.cpp:485-512).
//   k_pq_views  per row chunk: each column's pages over the chunk and the run
//               window of the dictionary column the scan stages (searched for
//               every chunk in parallel before the scan).
//   k_pq_scan   row chunks: every needed column is decoded at each row — PLAIN
//               values loaded in place from the page, dictionary indices
//               located through the run table and bit-unpacked from the page
//               (RleDecoder::Next / NextBatch, parquet.cpp:514-608) then
//               gathered from the dictionary page (DecodeDataPageTyped,
//               parquet.cpp:2119-2210; an index past the dictionary yields 0)
//               — the scan filter is evaluated on the decoded values
//               (BuildTypedKeepMask, physical_planner.cpp:505-720) and the
//               passing rows are compacted into typed columns.
//   The compacted columns then go through the ordinary aggregation ingest.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "gb_zstd.h"
#include "gb_agg_host.h"
#include "gb_kernels.cuh"

namespace gb {

// ------------------------------------------------------------ thrift reader
struct TReader {
    const uint8_t *p;
    size_t n, pos;
    bool bad = false;
    TReader(const uint8_t *p_, size_t n_, size_t pos_ = 0) : p(p_), n(n_), pos(pos_) {}
    uint8_t byte() {
        if (pos >= n) {
            bad = true;
            return 0;
        }
        return p[pos++];
    }
    uint64_t varint() {
        uint64_t v = 0;
        for (int sh = 0; sh < 64; sh += 7) {
            uint8_t b = byte();
            v |= (uint64_t)(b & 0x7f) << sh;
            if (!(b & 0x80) || bad) return v;
        }
        bad = true;
        return v;
    }
    int64_t zz() {
        uint64_t v = varint();
        return (int64_t)(v >> 1) ^ -(int64_t)(v & 1);
    }
    // next field of the current struct; false at STOP
    bool field(int &fid, int &type, int &last) {
        uint8_t b = byte();
        if (bad || b == 0) return false;
        type = b & 0x0f;
        int delta = b >> 4;
        fid = delta ? last + delta : (int)(int16_t)zz();
        last = fid;
        return true;
    }
    void list_header(int &etype, uint64_t &size) {
        uint8_t b = byte();
        etype = b & 0x0f;
        size = (b >> 4) == 15 ? varint() : (b >> 4);
    }
    std::string binary() {
        uint64_t len = varint();
        if (bad || pos + len > n) {
            bad = true;
            return std::string();
        }
        std::string s((const char *)p + pos, (size_t)len);
        pos += len;
        return s;
    }
    void skip(int type, int depth = 0) {
        if (depth > 32) {
            bad = true;
            return;
        }
        switch (type) {
        case 1:
        case 2: break;  // bool in the field header
        case 3: byte(); break;
        case 4:
        case 5:
        case 6: varint(); break;
        case 7: pos += 8; break;
        case 8: {
            uint64_t len = varint();
            pos += len;
            break;
        }
        case 9:
        case 10: {
            int et;
            uint64_t sz;
            list_header(et, sz);
            for (uint64_t i = 0; i < sz && !bad; i++) skip(et, depth + 1);
            break;
        }
        case 11: {
            uint64_t sz = varint();
            if (sz) {
                uint8_t kv = byte();
                for (uint64_t i = 0; i < sz && !bad; i++) {
                    skip(kv >> 4, depth + 1);
                    skip(kv & 0x0f, depth + 1);
                }
            }
            break;
        }
        case 12: {
            int fid, t, last = 0;
            while (field(fid, t, last)) skip(t, depth + 1);
            break;
        }
        default: bad = true;
        }
        if (pos > n) bad = true;
    }
};

}  // namespace gb

using namespace gb;

// ----------------------------------------------------------- host structures
struct PqPage {
    int32_t kind;        // 0 PLAIN, 1 dictionary indices
    int32_t col;         // file column
    uint32_t rg;
    uint32_t first_row;  // within the row group
    uint32_t n_values;   // entries, NULLs included (rows of a flat column)
    uint32_t bytes;      // bytes of the encoded values
    uint64_t off;        // offset of the encoded values in the file
    uint64_t def_off = 0;    // OPTIONAL column: its definition levels (RLE/bit-packed, bit width 1)
    uint32_t def_bytes = 0;  // 0: REQUIRED column (no levels)
    // a page of a compressed (SNAPPY) column chunk: where its bytes are in the
    // file; off / def_off above are then offsets in the batch's decompressed
    // image (set per batch)
    uint64_t src_off = 0;    // compressed values (page v1: the whole payload)
    uint32_t src_bytes = 0;
    uint32_t raw_bytes = 0;  // their uncompressed size
    uint32_t lvl_copy = 0;   // page v2: level bytes stored uncompressed before them
    uint8_t lvl_pending = 0; // page v1 of an OPTIONAL column: the level length is inside the compressed bytes
    uint8_t stored = 0;      // page v2 with is_compressed = false: values copied, not inflated
};

struct PqChunk {
    int64_t num_values = 0;
    uint64_t start = 0, size = 0;  // byte range of the column chunk
    int32_t codec = 0;
    int64_t dict_off = -1;  // dictionary payload offset (-1 = none)
    uint32_t dict_n = 0;
    uint32_t dict_bytes = 0;  // dictionary payload bytes (uncompressed)
    uint64_t dict_src = 0;    // compressed chunk: the dictionary page's compressed bytes in the file
    uint32_t dict_src_bytes = 0;
    // column statistics (zone map): raw min / max bytes, Statistics fields
    // 5/6 (min_value/max_value) over the deprecated 2/1 (min/max)
    bool has_stats = false;
    std::string stat_min, stat_max;
    uint32_t page_begin = 0, page_end = 0;  // into pages (data pages only)
};

struct PqColumn {
    std::string name;
    int32_t ptype = -1;  // parquet physical type
    int32_t gtype = 0;   // gb_type (0 = unsupported)
    int32_t repetition = 0;
    int32_t width = 0;   // bytes per PLAIN value (0: BYTE_ARRAY)
    bool plain_strings = false;  // a BYTE_ARRAY column with PLAIN data pages
};

struct gb_pq_file {
    const uint8_t *host = nullptr;
    uint64_t size = 0;
    std::vector<PqColumn> cols;
    std::vector<uint64_t> rg_rows;
    std::vector<std::vector<PqChunk>> chunks;  // [rg][col]
    std::vector<PqPage> pages;
    uint64_t num_rows = 0;
    bool compressed = false;  // some column chunk is SNAPPY-compressed
    void *dev = nullptr;  // device copy of the file (gb_pq_upload)
    // page index of the uploaded file, built on the GPU by the first
    // device-resident scan and kept with the file (like Parquet's offset
    // index): every page's descriptor and every dictionary page's run table
    std::mutex idx_mu;
    bool idx_ready = false;
    void *idx_pages = nullptr, *idx_runs = nullptr, *idx_page_runs = nullptr;
    std::vector<uint32_t> idx_col_pages;  // [(rg * n_cols + col) * 2] = {begin, end}
    // device buffers of gb_pq_dict_sum, kept (grow-only) for the next call
    std::mutex ds_mu;
    void *ds_buf[11] = {};
    size_t ds_cap[11] = {};
};

static gb_status pq_corrupt(const char *what) {
    set_error("malformed Parquet: %s", what);
    return GB_ERR_CORRUPT;
}

static gb_status parse_footer(gb_pq_file *f) {
    const uint8_t *b = f->host;
    const uint64_t n = f->size;
    if (n < 12 || memcmp(b, "PAR1", 4) != 0 || memcmp(b + n - 4, "PAR1", 4) != 0) return pq_corrupt("magic");
    uint32_t flen;
    memcpy(&flen, b + n - 8, 4);
    if ((uint64_t)flen + 12 > n) return pq_corrupt("footer length");
    TReader r(b, n - 8, n - 8 - flen);
    int fid, type, last = 0;
    std::vector<PqColumn> schema;
    while (r.field(fid, type, last)) {
        if (fid == 2 && type == 9) {  // schema
            int et;
            uint64_t sz;
            r.list_header(et, sz);
            for (uint64_t i = 0; i < sz && !r.bad; i++) {
                PqColumn c;
                int nchild = 0, conv = -1, int_bits = 0;
                bool int_signed = true;
                int f2, t2, l2 = 0;
                while (r.field(f2, t2, l2)) {
                    if (f2 == 1 && t2 == 5) c.ptype = (int)r.zz();
                    else if (f2 == 3 && t2 == 5) c.repetition = (int)r.zz();
                    else if (f2 == 4 && t2 == 8) c.name = r.binary();
                    else if (f2 == 5 && t2 == 5) nchild = (int)r.zz();
                    else if (f2 == 6 && t2 == 5) conv = (int)r.zz();
                    else if (f2 == 10 && t2 == 12) {  // LogicalType union
                        int f3, t3, l3 = 0;
                        while (r.field(f3, t3, l3)) {
                            if (f3 == 10 && t3 == 12) {  // INTEGER
                                int f4, t4, l4 = 0;
                                while (r.field(f4, t4, l4)) {
                                    if (f4 == 1 && t4 == 3) int_bits = (int8_t)r.byte();
                                    else if (f4 == 2 && (t4 == 1 || t4 == 2)) int_signed = t4 == 1;  // isSigned
                                    else r.skip(t4);
                                }
                            } else r.skip(t3);
                        }
                    } else r.skip(t2);
                }
                if (i == 0) continue;  // root
                if (nchild > 0) {
                    set_error("nested Parquet schemas are not supported on the GPU path");
                    return GB_ERR_UNSUPPORTED;
                }
                // unsigned integers (converted types UINT_8..UINT_64, or a
                // LogicalType INTEGER with isSigned = false): 8- and 16-bit
                // values fit an INTEGER; 32- and 64-bit values (and their
                // statistics, which Parquet orders unsigned) do not fit the
                // signed types, so those columns are refused
                const bool uns = (conv >= 11 && conv <= 14) || (int_bits != 0 && !int_signed);
                const int ubits = conv == 11 ? 8 : conv == 12 ? 16 : conv == 13 ? 32 : conv == 14 ? 64 : int_bits;
                switch (c.ptype) {
                case 1:
                    if (uns) c.gtype = ubits <= 16 ? GB_T_INTEGER : 0;
                    else c.gtype = (conv == 16 || int_bits == 16) ? GB_T_SMALLINT : GB_T_INTEGER;
                    c.width = 4;
                    break;
                case 2: c.gtype = uns ? 0 : GB_T_BIGINT; c.width = 8; break;
                case 5: c.gtype = GB_T_DOUBLE; c.width = 8; break;
                case 6: c.gtype = GB_T_VARCHAR; c.width = 0; break;  // BYTE_ARRAY (UTF8 or not)
                default: c.gtype = 0; c.width = 0; break;
                }
                schema.push_back(c);
            }
        } else if (fid == 3 && type == 6) {
            f->num_rows = (uint64_t)r.zz();
        } else if (fid == 4 && type == 9) {  // row groups
            int et;
            uint64_t sz;
            r.list_header(et, sz);
            for (uint64_t g = 0; g < sz && !r.bad; g++) {
                std::vector<PqChunk> cc;
                uint64_t rows = 0;
                int f2, t2, l2 = 0;
                while (r.field(f2, t2, l2)) {
                    if (f2 == 1 && t2 == 9) {
                        int et2;
                        uint64_t sz2;
                        r.list_header(et2, sz2);
                        for (uint64_t c = 0; c < sz2 && !r.bad; c++) {
                            PqChunk ch;
                            int64_t data_off = -1, dict_off = -1, comp = 0;
                            int f3, t3, l3 = 0;
                            while (r.field(f3, t3, l3)) {
                                if (f3 == 3 && t3 == 12) {  // ColumnMetaData
                                    int f4, t4, l4 = 0;
                                    while (r.field(f4, t4, l4)) {
                                        if (f4 == 4 && t4 == 5) ch.codec = (int)r.zz();
                                        else if (f4 == 5 && t4 == 6) ch.num_values = r.zz();
                                        else if (f4 == 7 && t4 == 6) comp = r.zz();
                                        else if (f4 == 9 && t4 == 6) data_off = r.zz();
                                        else if (f4 == 11 && t4 == 6) dict_off = r.zz();
                                        else if (f4 == 12 && t4 == 12) {  // Statistics
                                            int f5, t5, l5 = 0;
                                            while (r.field(f5, t5, l5)) {
                                                if ((f5 == 1 || f5 == 5) && t5 == 8) {
                                                    ch.stat_max = r.binary();
                                                    ch.has_stats = true;
                                                } else if ((f5 == 2 || f5 == 6) && t5 == 8) {
                                                    ch.stat_min = r.binary();
                                                    ch.has_stats = true;
                                                } else r.skip(t5);
                                            }
                                        }
                                        else r.skip(t4);
                                    }
                                } else r.skip(t3);
                            }
                            int64_t start = (dict_off >= 0 && dict_off < data_off) ? dict_off : data_off;
                            if (start < 0 || comp < 0 || (uint64_t)(start + comp) > n) return pq_corrupt("column chunk range");
                            ch.start = (uint64_t)start;
                            ch.size = (uint64_t)comp;
                            cc.push_back(ch);
                        }
                    } else if (f2 == 3 && t2 == 6) {
                        rows = (uint64_t)r.zz();
                    } else r.skip(t2);
                }
                f->chunks.push_back(cc);
                f->rg_rows.push_back(rows);
            }
        } else {
            r.skip(type);
        }
    }
    if (r.bad) return pq_corrupt("footer thrift");
    if (schema.empty()) return pq_corrupt("schema has no columns");
    uint64_t total = 0;
    for (uint64_t rows : f->rg_rows) total += rows;
    if (total != f->num_rows) return pq_corrupt("row-group rows do not add up to num_rows");
    f->cols = schema;
    for (auto &cc : f->chunks)
        if (cc.size() != f->cols.size()) return pq_corrupt("row group column count");
    return GB_OK;
}

// Walk one column chunk's page headers.
static gb_status parse_pages(gb_pq_file *f, uint32_t rg, uint32_t col) {
    PqChunk &ch = f->chunks[rg][col];
    uint64_t pos = ch.start, end = ch.start + ch.size;
    uint32_t row = 0;
    ch.page_begin = (uint32_t)f->pages.size();
    // a flat OPTIONAL column (maximum definition level 1) prefixes every data
    // page's values with its definition levels (ReadDefLevels,
    // parquet.cpp:1879-1981): page v1 as a 4-byte length + RLE/bit-packed
    // hybrid, page v2 as the hybrid alone, its length in the page header
    const bool opt = f->cols[col].repetition == 1;
    while (pos < end) {
        TReader r(f->host, end, pos);
        int fid, type, last = 0;
        int ptype = -1, enc = -1, version = 0;
        int64_t csize = -1, usize = -1, nvals = -1, dict_n = -1, def_len = 0, rep_len = 0;
        bool v2_compressed = true;
        while (r.field(fid, type, last)) {
            if (fid == 1 && type == 5) ptype = (int)r.zz();
            else if (fid == 2 && type == 5) usize = r.zz();
            else if (fid == 3 && type == 5) csize = r.zz();
            else if ((fid == 5 || fid == 8) && type == 12) {  // data page v1 / v2
                version = fid == 5 ? 1 : 2;
                int f2, t2, l2 = 0;
                while (r.field(f2, t2, l2)) {
                    if (f2 == 1 && t2 == 5) nvals = r.zz();
                    else if (fid == 5 && f2 == 2 && t2 == 5) enc = (int)r.zz();
                    else if (fid == 8 && f2 == 4 && t2 == 5) enc = (int)r.zz();
                    else if (fid == 8 && f2 == 5 && t2 == 5) def_len = r.zz();
                    else if (fid == 8 && f2 == 6 && t2 == 5) rep_len = r.zz();
                    else if (fid == 8 && f2 == 7 && (t2 == 1 || t2 == 2)) v2_compressed = t2 == 1;  // is_compressed
                    else r.skip(t2);
                }
                if (rep_len || (def_len && !opt)) {
                    set_error("Parquet levels on a non-OPTIONAL or repeated column are not supported");
                    return GB_ERR_UNSUPPORTED;
                }
            } else if (fid == 7 && type == 12) {
                int f2, t2, l2 = 0;
                while (r.field(f2, t2, l2)) {
                    if (f2 == 1 && t2 == 5) dict_n = r.zz();
                    else r.skip(t2);
                }
            } else r.skip(type);
        }
        if (r.bad || csize < 0 || r.pos + (uint64_t)csize > end) return pq_corrupt("page header");
        const uint64_t payload = r.pos;
        const uint64_t next_page = payload + (uint64_t)csize;
        const bool comp = ch.codec != 0;
        if (comp && (usize < 0 || usize > (int64_t)0x7fffffff)) return pq_corrupt("uncompressed page size");
        if (ptype == 2) {
            if (dict_n < 0) return pq_corrupt("dictionary page header");
            ch.dict_off = (int64_t)payload;
            ch.dict_n = (uint32_t)dict_n;
            ch.dict_bytes = (uint32_t)csize;
            if (comp) {  // decompressed into the batch's image; its offset is set there
                ch.dict_src = payload;
                ch.dict_src_bytes = (uint32_t)csize;
                ch.dict_bytes = (uint32_t)usize;
                csize = usize;  // the checks below bound the uncompressed values
            }
            if ((uint64_t)dict_n * f->cols[col].width > (uint64_t)csize) return pq_corrupt("dictionary size");
            // BYTE_ARRAY: a 4-byte length before every value
            if (f->cols[col].gtype == GB_T_VARCHAR && (uint64_t)dict_n * 4 > (uint64_t)csize)
                return pq_corrupt("dictionary size");
        } else if (ptype == 0 || ptype == 3) {
            if (nvals < 0) return pq_corrupt("data page header");
            PqPage pg;
            pg.col = (int32_t)col;
            pg.rg = rg;
            pg.first_row = row;
            pg.n_values = (uint32_t)nvals;
            pg.bytes = (uint32_t)csize;
            pg.off = payload;
            if (comp) {
                // page v1: levels and values are compressed together; page v2:
                // its levels are stored as is, then the (compressed) values
                const uint64_t lv = version == 2 ? (uint64_t)def_len : 0;
                if (lv > (uint64_t)csize || (version == 2 && (uint64_t)usize < lv)) return pq_corrupt("page sizes");
                pg.lvl_copy = (uint32_t)lv;
                pg.src_off = payload + lv;
                pg.src_bytes = (uint32_t)((uint64_t)csize - lv);
                pg.raw_bytes = (uint32_t)((uint64_t)usize - lv);
                pg.stored = version == 2 && !v2_compressed;
                if (pg.stored && pg.src_bytes != pg.raw_bytes) return pq_corrupt("page sizes");
                pg.lvl_pending = opt && version == 1;
                pg.def_bytes = (uint32_t)lv;  // v1 OPTIONAL: known once inflated
                if (opt && version == 2 && lv == 0 && nvals > 0) return pq_corrupt("definition levels");
                pg.bytes = pg.raw_bytes;  // values bytes (v1 OPTIONAL: less its levels, set per batch)
                csize = usize;
            } else if (opt) {
                uint64_t lv;
                if (version == 1) {
                    if (csize < 4) return pq_corrupt("definition levels");
                    uint32_t l4;
                    memcpy(&l4, f->host + payload, 4);
                    pg.def_off = payload + 4;
                    lv = 4 + (uint64_t)l4;
                    pg.def_bytes = l4;
                } else {
                    if (def_len < 0) return pq_corrupt("definition levels");
                    pg.def_off = payload;
                    lv = (uint64_t)def_len;
                    pg.def_bytes = (uint32_t)def_len;
                }
                if (lv > (uint64_t)csize || (pg.def_bytes == 0 && nvals > 0)) return pq_corrupt("definition levels");
                pg.off = payload + lv;
                pg.bytes = (uint32_t)((uint64_t)csize - lv);
            }
            if (enc == 0) {
                pg.kind = 0;
                // with NULLs only the defined values are stored: their count
                // is checked on the GPU once the levels are decoded
                if (!opt && (uint64_t)nvals * f->cols[col].width > (uint64_t)csize) return pq_corrupt("PLAIN page size");
                if (f->cols[col].gtype == GB_T_VARCHAR) f->cols[col].plain_strings = true;
            } else if (enc == 2 || enc == 8) {
                pg.kind = 1;
                if (pg.bytes < 1 && !(opt && nvals > 0)) return pq_corrupt("dictionary-index page");
            } else {
                set_error("Parquet encoding %d is not supported on the GPU path", enc);
                return GB_ERR_UNSUPPORTED;
            }
            f->pages.push_back(pg);
            row += (uint32_t)nvals;
        }
        pos = next_page;
    }
    ch.page_end = (uint32_t)f->pages.size();
    if (row != f->rg_rows[rg]) return pq_corrupt("page values do not add up to the row group");
    return GB_OK;
}

// ================================================================= kernels
struct DPage {
    uint64_t off;       // offset of the encoded values in the device file
    uint64_t dict_off;  // dictionary payload offset
    uint64_t dict_ids;  // VARCHAR: device address of the dictionary's string ids (0: fixed-width values)
    uint64_t dict_match;  // VARCHAR: per dictionary entry, 1 = passes the string predicates (0: none)
    uint64_t def_off;   // definition levels (OPTIONAL column; def_bytes = 0: REQUIRED)
    uint32_t first_row, n_values, bytes, dict_n;  // n_values: entries, NULLs included
    uint32_t run_base, run_cap;          // run-table slice of the dictionary indices
    uint32_t def_run_base, def_run_cap;  // run-table slice of the definition levels
    uint32_t def_bytes;
    int32_t kind, width;
    uint32_t pad;
};

struct DRun {
    uint32_t start;  // first entry of the run within its stream
    uint32_t off;    // payload byte of the packed values (0xffffffff = RLE)
    uint32_t cnt;
    uint32_t val;    // RLE value
    uint32_t nn;     // definition levels: defined entries before the run
};

// One RLE/bit-packed hybrid stream for the run walk: the dictionary indices
// of a data page (bit width in its first byte) or the definition levels of
// an OPTIONAL column's data page (bit width 1).  Per page, page_runs holds
// PQ_PR words: {index runs, index bit width, level runs, defined entries}.
#define PQ_PR 4
struct RunJob {
    uint64_t off;       // stream offset in the device file
    uint32_t bytes;     // stream bytes
    uint32_t n_values;  // entries to decode (an upper bound for indices)
    uint32_t run_base, run_cap;
    uint32_t page;      // index into pages / page_runs
    uint32_t levels;    // 1: definition levels
};

#define PQ_WIN 16384
#define PQ_LEVEL_RUN 512  // bit-packed level runs are split at this many entries (bounds the popcount)

// One CTA per stream: windows of the payload are staged in shared memory and
// thread 0 walks the run headers (RleDecoder::FetchRun, parquet.cpp:476-540).
// A level stream's runs also carry the defined entries before them, and its
// bit-packed runs are split every PQ_LEVEL_RUN entries so that a row's
// position among the defined values needs at most PQ_LEVEL_RUN / 64 words of
// popcount.  For a level stream, the page's defined entries must fit its
// values (PLAIN: width bytes each); anything else sets ERR_CORRUPT.
__global__ void k_pq_runs(const uint8_t *file, const DPage *pages, const RunJob *jobs, DRun *runs,
                          uint32_t *page_runs, Ctl *ctl) {
    __shared__ uint8_t win[PQ_WIN + 16];
    __shared__ uint64_t s_pos;   // stream position of the walk
    __shared__ uint32_t s_vals, s_runs, s_done, s_bw, s_nn;
    const RunJob J = jobs[blockIdx.x];
    if (threadIdx.x == 0) {
        s_vals = 0;
        s_runs = 0;
        s_nn = 0;
        s_done = 0;
        s_pos = 0;
        if (J.levels) {
            s_bw = 1;
        } else if (J.bytes == 0) {  // no encoded values (a page of NULLs only)
            s_bw = 0;
            s_done = 1;
        } else {
            s_bw = file[J.off];
            s_pos = 1;
            if (s_bw > 32) {
                atomicOr(&ctl->err, (u32)ERR_CORRUPT);
                s_done = 1;
            }
        }
    }
    __syncthreads();
    while (!s_done) {
        const uint64_t w0 = s_pos;
        const uint64_t wn = min((uint64_t)PQ_WIN, (uint64_t)J.bytes - w0);
        for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) win[i] = file[J.off + w0 + i];
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t bw = s_bw;
            const uint32_t vb = (bw + 7) / 8;
            uint64_t pos = w0;
            uint32_t vals = s_vals, nr = s_runs, nn = s_nn;
            bool done = false, err = false;
            while (!done) {
                if (vals >= J.n_values || pos >= J.bytes) {
                    done = true;
                    break;
                }
                // a header (<= 10 bytes) plus an RLE value must lie inside the window
                if (pos + 16 > w0 + wn && w0 + wn < J.bytes) break;
                uint64_t hdr = 0;
                int sh = 0;
                uint64_t q = pos;
                for (;;) {
                    if (q >= J.bytes || sh > 35) {
                        err = true;
                        break;
                    }
                    const uint8_t b = win[q - w0];
                    q++;
                    hdr |= (uint64_t)(b & 0x7f) << sh;
                    if (!(b & 0x80)) break;
                    sh += 7;
                }
                if (err) break;
                if (hdr & 1) {
                    const uint64_t cnt = min((hdr >> 1) * 8, (uint64_t)(J.n_values - vals));
                    const uint64_t plen = (hdr >> 1) * (uint64_t)bw;
                    uint64_t have = cnt;
                    bool trunc = false;
                    if (q + plen > J.bytes) {
                        // truncated packed run: the reference decodes what is there
                        // and leaves the rest unset (RleDecoder::NextBatch refill)
                        have = min(cnt, ((uint64_t)J.bytes - q) * 8 / (bw ? bw : 1));
                        trunc = true;
                    }
                    // level runs split every PQ_LEVEL_RUN entries (byte aligned: 512 bits)
                    for (uint64_t e0 = 0; e0 < have && !err; e0 += (J.levels ? PQ_LEVEL_RUN : have)) {
                        DRun rn;
                        rn.start = vals + (uint32_t)e0;
                        rn.off = (uint32_t)(q + (J.levels ? e0 / 8 : 0));
                        rn.cnt = (uint32_t)min(have - e0, (uint64_t)(J.levels ? PQ_LEVEL_RUN : have));
                        rn.val = 0;
                        rn.nn = nn;
                        if (J.levels) {
                            // defined entries of this piece: popcount of its bits
                            // (read from the file: a run may extend past the window)
                            uint32_t c = 0;
                            for (uint32_t b = 0; b < rn.cnt; b += 8) {
                                uint32_t byte = __ldg(file + J.off + rn.off + b / 8);
                                if (rn.cnt - b < 8) byte &= (1u << (rn.cnt - b)) - 1u;
                                c += __popc(byte);
                            }
                            nn += c;
                        }
                        if (rn.cnt) {
                            if (nr >= J.run_cap) {
                                err = true;
                                break;
                            }
                            runs[J.run_base + nr] = rn;
                            nr++;
                        }
                    }
                    vals += (uint32_t)have;
                    q += plen;
                    if (trunc) done = true;
                } else {
                    const uint64_t cnt = hdr >> 1;
                    if (q + vb > J.bytes) {
                        done = true;
                        break;
                    }
                    uint32_t v = 0;
                    for (uint32_t b = 0; b < vb; b++) v |= (uint32_t)win[q - w0 + b] << (8 * b);
                    q += vb;
                    DRun rn;
                    rn.start = vals;
                    rn.off = 0xffffffffu;
                    rn.cnt = (uint32_t)min(cnt, (uint64_t)(J.n_values - vals));
                    rn.val = v;
                    rn.nn = nn;
                    if (J.levels) {
                        if (v > 1) {  // a flat OPTIONAL column has levels 0 and 1
                            err = true;
                            break;
                        }
                        nn += v ? rn.cnt : 0u;
                    }
                    if (rn.cnt) {
                        if (nr >= J.run_cap) {
                            err = true;
                            break;
                        }
                        runs[J.run_base + nr] = rn;
                        nr++;
                        vals += rn.cnt;
                    }
                }
                pos = q;
            }
            if (err) {
                atomicOr(&ctl->err, (u32)ERR_CORRUPT);
                done = true;
            }
            s_pos = pos;
            s_vals = vals;
            s_runs = nr;
            s_nn = nn;
            s_done = done;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        uint32_t *pr = page_runs + (u64)PQ_PR * J.page;
        if (J.levels) {
            const DPage &pg = pages[J.page];
            pr[2] = s_runs;
            pr[3] = s_nn;
            // the defined entries are the stored values: they must fit
            if (s_vals < pg.n_values || (pg.kind == 0 && (u64)s_nn * (u64)pg.width > pg.bytes))
                atomicOr(&ctl->err, (u32)ERR_CORRUPT);
        } else {
            pr[0] = s_runs;
            pr[1] = s_bw;
        }
    }
}


// ------------------------------------------------- VARCHAR dictionary pages
// A BYTE_ARRAY dictionary page holds its values PLAIN: a 4-byte little-endian
// length, then the bytes, per value (ReadDictionaryPage / the VARCHAR branch
// of DecodeDataPageTyped, parquet.cpp:2340-2471, 2229-2331), and so does a
// PLAIN BYTE_ARRAY data page (its defined values only; parquet.cpp:
// 1742-1854).  A batch's dictionary strings and PLAIN-page strings are
// compacted into one offsets + bytes array and encoded once into the
// handle's string dictionary; a dictionary-encoded data page's indices then
// gather string ids, and value j of a PLAIN page is its page's entry j.
struct DDict {
    uint64_t off;           // payload offset in the device file
    uint64_t entry_base;    // index of the page's first value in the batch's entries
    uint64_t compact_base;  // its first byte in the compacted strings
    uint32_t n, bytes;      // values, payload bytes
};

// One CTA per dictionary page: windows of the payload are staged in shared
// memory and thread 0 walks the length prefixes, writing each value's source
// address and compacted offset.  Every length is checked against the
// payload, and the walk must end exactly at the payload's end; anything else
// sets ERR_CORRUPT (and the host stops before using the entries).
// counts != nullptr (a PLAIN page, whose value count the levels decide): d.n
// only bounds the values, nothing is written but counts[page], and the walk
// ends at the payload's end.
__global__ void k_pq_dict_walk(const uint8_t *file, const DDict *dicts, u64 *src, int64_t *offs, Ctl *ctl,
                               uint32_t *counts) {
    __shared__ uint8_t win[PQ_WIN];
    __shared__ u64 s_pos;
    __shared__ uint32_t s_i;
    __shared__ int s_state;  // 0 walking, 1 done, 2 corrupt
    const DDict d = dicts[blockIdx.x];
    if (threadIdx.x == 0) {
        s_pos = 0;
        s_i = 0;
        s_state = d.n == 0 ? (d.bytes == 0 ? 1 : 2) : 0;
    }
    __syncthreads();
    // each window moves the walk by at least one value: n + 1 windows suffice
    for (u64 round = 0; round <= (u64)d.n && s_state == 0; round++) {
        const u64 w0 = s_pos;
        const u64 wn = min((u64)PQ_WIN, (u64)d.bytes - w0);
        for (u64 k = threadIdx.x; k < wn; k += blockDim.x) win[k] = file[d.off + w0 + k];
        __syncthreads();
        if (threadIdx.x == 0) {
            u64 pos = w0;
            uint32_t i = s_i;
            int state = 0;
            while (i < d.n) {
                if (counts && pos == d.bytes) break;  // every value of the payload walked
                if (pos + 4 > w0 + wn) {
                    if (pos + 4 > d.bytes) state = 2;  // no room for the length
                    break;
                }
                const uint8_t *q = win + (pos - w0);
                const uint32_t len = (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) |
                                     ((uint32_t)q[3] << 24);
                if ((u64)len > (u64)d.bytes - pos - 4) {
                    state = 2;  // the value runs past the payload
                    break;
                }
                if (!counts) {
                    src[d.entry_base + i] = d.off + pos + 4;
                    offs[d.entry_base + i] = (int64_t)(d.compact_base + pos - 4 * (u64)i);
                }
                pos += 4 + (u64)len;
                i++;
            }
            if (state == 0 && (i == d.n || (counts && pos == d.bytes))) state = pos == d.bytes ? 1 : 2;
            if (state == 0 && pos == w0) state = 2;  // no progress (cannot happen with a valid window)
            s_pos = pos;
            s_i = i;
            s_state = state;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && s_state != 1) atomicOr(&ctl->err, (u32)ERR_CORRUPT);
    if (threadIdx.x == 0 && counts) counts[blockIdx.x] = s_i;
}

// Copy each dictionary value's bytes to its compacted offset (the walk has
// checked every range against its page).
__global__ void k_pq_dict_copy(const uint8_t *file, const u64 *src, const int64_t *offs, u64 n, uint8_t *out) {
    for (u64 e = blockIdx.x * (u64)blockDim.x + threadIdx.x; e < n; e += (u64)gridDim.x * blockDim.x) {
        const uint8_t *a = file + src[e];
        uint8_t *b = out + offs[e];
        const int64_t len = offs[e + 1] - offs[e];
        for (int64_t k = 0; k < len; k++) b[k] = a[k];
    }
}

// Locate the page of `col` holding row r of the chunk's row group:
// pages [pb, pe) are sorted by first_row.
__device__ __forceinline__ uint32_t find_page(const DPage *pages, uint32_t pb, uint32_t pe, uint32_t r) {
    uint32_t lo = pb, hi = pe;  // last page with first_row <= r
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (pages[mid].first_row <= r) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Decode one value of a page at value index i (as int64 / double bits).
// `bw` bits (bw <= 32) starting at bit `bit` of the byte string at p, read
// with aligned 8-byte loads of the words that hold them.
__device__ __forceinline__ uint32_t load_bits(const uint8_t *p, u64 bit, uint32_t bw) {
    const uintptr_t a = (uintptr_t)p + (uintptr_t)(bit >> 3);
    const u64 *w = (const u64 *)(a & ~(uintptr_t)7);
    const uint32_t sh = (uint32_t)(a & 7) * 8 + (uint32_t)(bit & 7);  // bit offset within *w
    u64 v = __ldg(w) >> sh;
    if (sh + bw > 64) v |= __ldg(w + 1) << (64 - sh);
    return (uint32_t)(v & (bw >= 32 ? 0xffffffffull : ((1ull << bw) - 1ull)));
}

// A PLAIN value at any byte address: aligned loads of the words that hold
// its bytes, joined by a funnel shift (a misaligned 4- or 8-byte load would
// fault).  The words read hold bytes of the value only.
__device__ __forceinline__ u64 load_plain(const uint8_t *p, int width) {
    const uintptr_t a = (uintptr_t)p;
    if (width == 4) {
        const uint32_t *w = (const uint32_t *)(a & ~(uintptr_t)3);
        const uint32_t sh = (uint32_t)(a & 3) * 8;
        const uint32_t lo = __ldg(w);
        const uint32_t v = sh ? __funnelshift_r(lo, __ldg(w + 1), sh) : lo;
        return (u64)(i64)(int32_t)v;
    }
    const u64 *w = (const u64 *)(a & ~(uintptr_t)7);
    const uint32_t sh = (uint32_t)(a & 7) * 8;
    const u64 lo = __ldg(w);
    return sh ? ((lo >> sh) | (__ldg(w + 1) << (64 - sh))) : lo;
}

// 64 bits starting at bit `bit` of p (LSB first): the aligned words that hold
// them, joined by a funnel shift.
__device__ __forceinline__ u64 load64_bits(const uint8_t *p, u64 bit) {
    const uintptr_t a = (uintptr_t)p + (uintptr_t)(bit >> 3);
    const u64 *w = (const u64 *)(a & ~(uintptr_t)7);
    const uint32_t sh = (uint32_t)(a & 7) * 8 + (uint32_t)(bit & 7);  // < 64
    const u64 lo = __ldg(w);
    return sh ? ((lo >> sh) | (__ldg(w + 1) << (64 - sh))) : lo;
}

// Entry i of a page: is it defined (not NULL), and if so its index j among
// the page's stored values (the defined entries before it).  A REQUIRED
// column's entries are all defined (j = i).
__device__ __forceinline__ bool level_at(const uint8_t *file, const DPage &pg, const DRun *runs,
                                         const uint32_t *page_runs, uint32_t pidx, uint32_t i, uint32_t &j) {
    j = i;
    if (pg.def_bytes == 0) return true;
    const uint32_t nr = page_runs[PQ_PR * pidx + 2];
    const DRun *rr = runs + pg.def_run_base;
    if (nr == 0) return false;
    uint32_t lo = 0, hi = nr;  // last run with start <= i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (rr[mid].start <= i) lo = mid;
        else hi = mid;
    }
    const DRun rn = rr[lo];
    if (i < rn.start || i >= rn.start + rn.cnt) return false;  // past the decoded levels (corrupt page)
    const uint32_t d = i - rn.start;
    if (rn.off == 0xffffffffu) {
        j = rn.nn + (rn.val ? d : 0u);
        return rn.val != 0;
    }
    // a bit-packed piece (<= PQ_LEVEL_RUN entries): popcount of the bits before d
    const uint8_t *bp = file + pg.def_off + rn.off;
    uint32_t c = 0;
    for (uint32_t w = 0; w + 64 <= d; w += 64) c += __popcll(load64_bits(bp, w));
    const u64 tail = load64_bits(bp, d & ~63u);
    const uint32_t r = d & 63u;
    if (r) c += __popcll(tail & ((1ull << r) - 1ull));
    j = rn.nn + c;
    return (tail >> r) & 1ull;
}

// Value i of page pg; for a VARCHAR page `match` asks for its entry's
// string-predicate flag instead of its string id.
__device__ __forceinline__ u64 decode_at(const uint8_t *file, const DPage &pg, const DRun *runs,
                                         const uint32_t *page_runs, uint32_t pidx, uint32_t i, bool match = false) {
    if (pg.kind == 0) {
        if (pg.dict_ids) {  // a PLAIN BYTE_ARRAY page: value i is entry i of its walked strings
            if (i >= pg.dict_n) return match ? 0ull : ~0ull;  // more defined rows than values: NULL id
            if (match) return pg.dict_match ? (u64)__ldg((const uint8_t *)pg.dict_match + i) : 1ull;
            return (u64)__ldg((const long long *)pg.dict_ids + i);
        }
        return load_plain(file + pg.off + (u64)i * pg.width, pg.width);
    }
    const uint32_t nr = page_runs[PQ_PR * pidx], bw = page_runs[PQ_PR * pidx + 1];
    const DRun *rr = runs + pg.run_base;
    uint32_t lo = 0, hi = nr;  // last run with start <= i
    if (nr == 0) return 0;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (rr[mid].start <= i) lo = mid;
        else hi = mid;
    }
    const DRun rn = rr[lo];
    uint32_t idx;
    if (i >= rn.start + rn.cnt) {
        idx = 0xffffffffu;  // past the decoded values (truncated page): left unset → 0
    } else if (rn.off == 0xffffffffu) {
        idx = rn.val;
    } else {
        idx = load_bits(file + pg.off + rn.off, (u64)(i - rn.start) * bw, bw);
    }
    if (idx >= pg.dict_n) return pg.dict_ids ? (match ? 0ull : ~0ull) : 0;  // out of range: the reference's 0 (VARCHAR: NULL id)
    if (pg.dict_ids) {
        if (match) return pg.dict_match ? (u64)__ldg((const uint8_t *)pg.dict_match + idx) : 1ull;
        return (u64)__ldg((const long long *)pg.dict_ids + idx);
    }
    return load_plain(file + pg.dict_off + (u64)idx * pg.width, pg.width);
}

struct PqChunkArg {
    uint32_t rg;          // index into the batch's row groups
    uint32_t row0, nrows; // rows [row0, row0 + nrows) of the row group
};

struct PqScan {
    int32_t n_cols;
    int32_t out_type[GB_MAX_COLS];   // gb_type of each compacted output column
    int32_t n_filters;
    int32_t id_col;                  // the VARCHAR key's string-id column (-1: none); a NULL key is id -1
    int32_t str_match;               // 1: the VARCHAR key has string predicates (pages' dict_match)
    Filter filters[GB_MAX_FILTERS];
    void *out[GB_MAX_COLS];
    uint64_t *out_valid[GB_MAX_COLS];  // validity words of an OPTIONAL column's output (all ones on entry)
    u64 out_cap;
};

// Row chunks of one batch.  Pass 1 decodes only the filter columns and keeps
// a row flag; pass 2 decodes the needed columns of the surviving rows only
// (late materialisation) into the compacted output.
// col_pages[2 * (rg * n_cols + c)] = {page begin, page end} in `pages`.
#define PQ_CHUNK 4096
__device__ __forceinline__ u64 decode_col(const uint8_t *file, const DPage *pages, const DRun *runs,
                                          const uint32_t *page_runs, const uint32_t *col_pages, int n_cols,
                                          uint32_t rg, int c, uint32_t r, bool &valid, bool match = false) {
    const uint32_t pb = col_pages[2 * (rg * n_cols + c)], pe = col_pages[2 * (rg * n_cols + c) + 1];
    const uint32_t pi = find_page(pages, pb, pe, r);
    const DPage &pg = pages[pi];
    uint32_t j;
    valid = level_at(file, pg, runs, page_runs, pi, r - pg.first_row, j);
    return valid ? decode_at(file, pg, runs, page_runs, pi, j, match) : 0;
}

// Per chunk, shared memory holds each column's pages that overlap the chunk
// (PQ_MAXP at most; more falls back to the global page search) and, for the
// first dictionary-encoded column, the runs of those pages that overlap the
// chunk (PQ_MAXR at most; more falls back to the global run search), so a
// row's decode searches a few shared entries instead of global arrays.
#define PQ_MAXP 8
#define PQ_MAXR 1024


#define PQ_FASTC 4  // columns of a chunk decoded by the straight-line path

struct PqChunkView {
    uint32_t np[GB_MAX_COLS];              // pages overlapping the chunk (0 = fallback)
    uint32_t pfirst[GB_MAX_COLS][PQ_MAXP];  // their first rows
    uint32_t pidx[GB_MAX_COLS][PQ_MAXP];    // their page indices
    int32_t dcol;                           // dictionary column with staged runs (-1: none)
    uint32_t fast;                          // 1: every column REQUIRED in one page, PLAIN fixed-width or dcol
    uint32_t rlo[PQ_MAXP];                  // first run of each page of dcol in the run table
    uint32_t rbeg[PQ_MAXP], rcnt[PQ_MAXP];  // staged run windows per page of dcol
};

// A chunk's view as k_pq_views writes it (u32 words, n_cols columns):
// [0] dcol, [1] fast, [2, 2 + n_cols) np, then per column pfirst[PQ_MAXP] and
// pidx[PQ_MAXP], then rlo, rbeg, rcnt [PQ_MAXP] each.
__host__ __device__ __forceinline__ uint32_t pq_view_words(int n_cols) {
    return 2u + (uint32_t)n_cols * (1u + 2u * PQ_MAXP) + 3u * PQ_MAXP;
}

__device__ __forceinline__ uint32_t run_search(const DRun *rr, uint32_t lo, uint32_t hi, uint32_t i) {
    while (hi - lo > 1) {  // last run with start <= i
        const uint32_t mid = (lo + hi) >> 1;
        if (rr[mid].start <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Value i of dictionary page pg, its run found in `rr[lo, hi)`.
__device__ __forceinline__ u64 dict_value(const uint8_t *file, const DPage &pg, const DRun *rr, uint32_t lo,
                                          uint32_t hi, uint32_t bw, uint32_t i, bool match = false) {
    if (hi <= lo) return 0;
    const DRun rn = rr[run_search(rr, lo, hi, i)];
    uint32_t idx;
    if (i < rn.start || i >= rn.start + rn.cnt) {
        idx = 0xffffffffu;  // past the decoded values (truncated page): left unset → 0
    } else if (rn.off == 0xffffffffu) {
        idx = rn.val;
    } else {
        idx = load_bits(file + pg.off + rn.off, (u64)(i - rn.start) * bw, bw);
    }
    if (idx >= pg.dict_n) return pg.dict_ids ? (match ? 0ull : ~0ull) : 0;  // out of range: the reference's 0 (VARCHAR: NULL id)
    if (pg.dict_ids) {
        if (match) return pg.dict_match ? (u64)__ldg((const uint8_t *)pg.dict_match + idx) : 1ull;
        return (u64)__ldg((const long long *)pg.dict_ids + idx);
    }
    return load_plain(file + pg.dict_off + (u64)idx * pg.width, pg.width);
}

// Row r (row-group relative) of column c through the chunk's staged view;
// valid = false for a NULL entry of an OPTIONAL column.
__device__ __forceinline__ u64 decode_staged(const uint8_t *file, const DPage *pages, const DRun *runs,
                                             const uint32_t *page_runs, const uint32_t *col_pages, int n_cols,
                                             uint32_t rg, int c, uint32_t r, const PqChunkView &V,
                                             const DRun *srun, bool &valid, bool match = false) {
    const uint32_t np = V.np[c];
    if (np == 0) return decode_col(file, pages, runs, page_runs, col_pages, n_cols, rg, c, r, valid, match);
    uint32_t k = 0;
    while (k + 1 < np && V.pfirst[c][k + 1] <= r) k++;
    const uint32_t pi = V.pidx[c][k];
    const DPage &pg = pages[pi];
    uint32_t j;
    valid = level_at(file, pg, runs, page_runs, pi, r - pg.first_row, j);
    if (!valid) return 0;
    if (pg.kind != 0 && c == V.dcol)  // (staged runs: REQUIRED columns only, j = i)
        return dict_value(file, pg, srun + V.rbeg[k], 0, V.rcnt[k], page_runs[PQ_PR * pi + 1], j, match);
    return decode_at(file, pg, runs, page_runs, pi, j, match);
}

// One thread per chunk: each column's pages overlapping the chunk (a
// fallback to per-row page search past PQ_MAXP pages), the first dictionary
// column whose runs the scan stages in shared memory with each page's run
// window (none past PQ_MAXR runs), and whether the chunk takes the
// straight-line decode.  Every chunk's searches run here in parallel, before
// the scan, instead of in one thread of each scan block while it waits.
__global__ void k_pq_views(const DPage *pages, const DRun *runs, const uint32_t *page_runs,
                           const uint32_t *col_pages, const PqChunkArg *chunks, uint32_t n_chunks, int n_cols,
                           int id_col, uint32_t *views) {
    const uint32_t W = pq_view_words(n_cols);
    for (uint32_t ci = blockIdx.x * blockDim.x + threadIdx.x; ci < n_chunks; ci += gridDim.x * blockDim.x) {
        const PqChunkArg ch = chunks[ci];
        const uint32_t rlast = ch.row0 + (ch.nrows ? ch.nrows - 1 : 0);
        uint32_t *rec = views + (u64)ci * W;
        uint32_t *npw = rec + 2, *pw = rec + 2 + n_cols;
        uint32_t *rw = pw + (uint32_t)n_cols * 2 * PQ_MAXP;
        int dc = -1;
        bool fast = n_cols <= PQ_FASTC;
        for (int c = 0; c < n_cols; c++) {
            const uint32_t pb = col_pages[2 * (ch.rg * n_cols + c)], pe = col_pages[2 * (ch.rg * n_cols + c) + 1];
            uint32_t n = 0, p0 = 0;
            if (pe > pb) {
                uint32_t p = find_page(pages, pb, pe, ch.row0);
                p0 = p;
                for (; p < pe && pages[p].first_row <= rlast; p++) {
                    if (n == PQ_MAXP) {
                        n = 0;  // too many pages: per-row global search
                        break;
                    }
                    pw[c * 2 * PQ_MAXP + n] = pages[p].first_row;
                    pw[c * 2 * PQ_MAXP + PQ_MAXP + n] = p;
                    n++;
                }
            }
            npw[c] = n;
            const bool dict = n && pages[p0].kind != 0 && pages[p0].def_bytes == 0;
            if (dc < 0 && dict) dc = c;
            // straight-line decode: one REQUIRED page, PLAIN fixed-width (or the staged dictionary column)
            if (n != 1 || pages[p0].def_bytes != 0 || (c == id_col && !dict) ||
                (!dict && (pages[p0].kind != 0 || pages[p0].dict_ids)))
                fast = false;
            if (dict && c != dc) fast = false;
        }
        int dcol = -1;
        if (dc >= 0) {
            uint32_t tot = 0;
            for (uint32_t k = 0; k < npw[dc]; k++) {
                const uint32_t pi = pw[dc * 2 * PQ_MAXP + PQ_MAXP + k];
                const DPage &pg = pages[pi];
                if (pg.kind == 0) {  // a PLAIN page of the column has no runs
                    rw[k] = 0;
                    rw[PQ_MAXP + k] = tot;
                    rw[2 * PQ_MAXP + k] = 0;
                    continue;
                }
                const uint32_t nr = page_runs[PQ_PR * pi];
                const DRun *rr = runs + pg.run_base;
                const uint32_t i0 = ch.row0 > pg.first_row ? ch.row0 - pg.first_row : 0;
                const uint32_t i1 = rlast - pg.first_row;  // inclusive (clipped by the run search)
                const uint32_t lo = nr ? run_search(rr, 0, nr, i0) : 0;
                const uint32_t hi = nr ? run_search(rr, lo, nr, i1) + 1 : 0;
                rw[k] = pg.run_base + lo;
                rw[PQ_MAXP + k] = tot;
                rw[2 * PQ_MAXP + k] = hi - lo;
                tot += hi - lo;
            }
            if (tot <= PQ_MAXR) dcol = dc;
        }
        if (dc >= 0 && dcol < 0) fast = false;  // its runs are not staged
        rec[0] = (uint32_t)dcol;
        rec[1] = fast ? 1u : 0u;
    }
}

__global__ void __launch_bounds__(256, 4) k_pq_scan(const uint8_t *file, const DPage *pages, const DRun *runs,
                                                 const uint32_t *page_runs, const uint32_t *col_pages,
                                                 const PqChunkArg *chunks, uint32_t n_chunks,
                                                 const uint32_t *views, const __grid_constant__ PqScan S,
                                                 Ctl *ctl) {
    constexpr int PER = PQ_CHUNK / 256;
    __shared__ PqChunkView V;
    __shared__ DRun srun[PQ_MAXR];
    __shared__ uint32_t s_surv[8][PER * 32];  // per warp: its surviving rows
    __shared__ u64 s_poff[PQ_FASTC];
    __shared__ int s_pwid[PQ_FASTC];
    __shared__ DPage s_dpg;  // the straight-line decode's dictionary page
    __shared__ uint32_t s_dbw;
    const int nc = S.n_cols;
    const uint32_t W = pq_view_words(nc), PW = 2 + (uint32_t)nc + (uint32_t)nc * 2 * PQ_MAXP;
    // each thread holds words threadIdx.x and threadIdx.x + 256 of the next
    // chunk's view, and its row range, loaded while the block works on the
    // current chunk
    uint32_t rw[2] = {0, 0};
    PqChunkArg ch = {0, 0, 0};
    if (blockIdx.x < n_chunks) {
        ch = chunks[blockIdx.x];
        for (int h = 0; h < 2; h++)
            if (threadIdx.x + 256u * h < W) rw[h] = views[(u64)blockIdx.x * W + threadIdx.x + 256u * h];
    }
    for (uint32_t ci = blockIdx.x; ci < n_chunks; ci += gridDim.x) {
        // the chunk's view (k_pq_views)
        for (int h = 0; h < 2; h++) {
            const uint32_t w = threadIdx.x + 256u * h, x = rw[h];
            if (w >= W) continue;
            if (w == 0) {
                V.dcol = (int32_t)x;
            } else if (w == 1) {
                V.fast = x;
            } else if (w < 2 + (uint32_t)nc) {
                V.np[w - 2] = x;
            } else if (w < PW) {
                const uint32_t q = w - 2 - nc, c = q / (2 * PQ_MAXP), k = q % (2 * PQ_MAXP);
                if (k < PQ_MAXP) V.pfirst[c][k] = x;
                else V.pidx[c][k - PQ_MAXP] = x;
            } else {
                const uint32_t q = w - PW;
                if (q < PQ_MAXP) V.rlo[q] = x;
                else if (q < 2 * PQ_MAXP) V.rbeg[q - PQ_MAXP] = x;
                else V.rcnt[q - 2 * PQ_MAXP] = x;
            }
        }
        const PqChunkArg chc = ch;
        if (ci + gridDim.x < n_chunks) {
            const uint32_t cn = ci + gridDim.x;
            ch = chunks[cn];
            for (int h = 0; h < 2; h++)
                if (threadIdx.x + 256u * h < W) rw[h] = views[(u64)cn * W + threadIdx.x + 256u * h];
        }
        __syncthreads();
        if (threadIdx.x == PQ_FASTC && V.fast && V.dcol >= 0) {  // the staged dictionary column's page
            const uint32_t pi = V.pidx[V.dcol][0];
            s_dpg = pages[pi];
            s_dbw = page_runs[PQ_PR * pi + 1];
        }
        if (threadIdx.x < PQ_FASTC) {  // the straight-line decode's PLAIN columns
            const int c = threadIdx.x;
            s_poff[c] = 0;  // file offset of row 0 of the row group in the column's page (mod 2^64)
            s_pwid[c] = 0;  // 0: not a PLAIN column
            if (V.fast && c < nc && c != V.dcol) {
                const DPage &pg = pages[V.pidx[c][0]];
                s_pwid[c] = pg.width;
                s_poff[c] = pg.off - (u64)V.pfirst[c][0] * (u64)pg.width;
            }
        }
        // one predicate on a PLAIN column inside one page (the common case):
        // every load of the chunk is issued before any compare, and before the
        // run staging below
        const int fc = (S.n_filters == 1 && S.filters[0].op <= GB_CMP_GE) ? S.filters[0].col : -1;
        const bool fastf =
            fc >= 0 && V.np[fc] == 1 && pages[V.pidx[fc][0]].kind == 0 && pages[V.pidx[fc][0]].def_bytes == 0;
        u32 kmask = 0;  // the fast predicate's result, row j * 256 + threadIdx.x in bit j
        if (fastf) {
            const DPage &pg = pages[V.pidx[fc][0]];
            const uint8_t *base = file + pg.off;  // page payloads start at any byte
            const int wd = pg.width;
            const uint32_t first = pg.first_row;
            u64 xv[PER];
#pragma unroll
            for (int j = 0; j < PER; j++) {
                const uint32_t rr = (uint32_t)j * 256 + threadIdx.x;
                xv[j] = 0;
                if (rr < chc.nrows) xv[j] = load_plain(base + (u64)(chc.row0 + rr - first) * wd, wd);
            }
            if (V.dcol >= 0 && threadIdx.x < V.rcnt[0]) {  // the first staged run while the loads fly
                const uint32_t t = threadIdx.x;
                srun[V.rbeg[0] + t] = runs[V.rlo[0] + t];
            }
            const Filter f = S.filters[0];
            const bool dbl = S.out_type[fc] == GB_T_DOUBLE;
#pragma unroll
            for (int j = 0; j < PER; j++) {
                const uint32_t rr = (uint32_t)j * 256 + threadIdx.x;
                const bool k = rr < chc.nrows && (dbl ? cmp_f(f.op, __longlong_as_double((i64)xv[j]), f.dc)
                                                      : cmp_i(f.op, (i64)xv[j], f.ic));
                kmask |= (u32)k << j;
            }
        }
        if (V.dcol >= 0) {
            const int dc = V.dcol;
            for (uint32_t k = 0; k < V.np[dc]; k++)
                for (uint32_t t = threadIdx.x + (fastf && k == 0 ? blockDim.x : 0); t < V.rcnt[k]; t += blockDim.x)
                    srun[V.rbeg[k] + t] = runs[V.rlo[k] + t];
        }
        __syncthreads();
        const PqChunkArg ch = chc;
        bool keep[PER];
        u32 mine = 0;
        if (fastf) {
#pragma unroll
            for (int j = 0; j < PER; j++) {
                keep[j] = (kmask >> j) & 1u;
                mine += keep[j];
            }
        } else {
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const uint32_t rr = (uint32_t)j * 256 + threadIdx.x;
            keep[j] = rr < ch.nrows;
            if (!keep[j]) continue;
            const uint32_t r = ch.row0 + rr;
            if (S.str_match) {  // the VARCHAR key's string predicates, per dictionary entry
                bool valid;
                const u64 m = decode_staged(file, pages, runs, page_runs, col_pages, S.n_cols, ch.rg, S.id_col, r, V,
                                            srun, valid, true);
                keep[j] = valid && m != 0;
            }
            for (int q = 0; q < S.n_filters && keep[j]; q++) {
                const Filter &f = S.filters[q];
                if (f.op >= GB_CMP_STR_EQ) continue;  // folded into the dictionary match above
                bool valid;
                const u64 x = decode_staged(file, pages, runs, page_runs, col_pages, S.n_cols, ch.rg, f.col, r, V, srun,
                                            valid);
                if (!valid) keep[j] = false;  // a comparison with NULL keeps no row
                else if (f.op == GB_CMP_IN) keep[j] = in_set(f.ptr, f.n, (i64)x);
                else if (S.out_type[f.col] == GB_T_DOUBLE) keep[j] = cmp_f(f.op, __longlong_as_double((i64)x), f.dc);
                else keep[j] = cmp_i(f.op, (i64)x, f.ic);
            }
            mine += keep[j];
        }
        }
        // late materialisation with full warps: each warp lists its
        // survivors in shared memory, then decodes them 32 at a time
        (void)mine;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        u32 cnt = 0;
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const unsigned bm = __ballot_sync(FULL, keep[j]);
            if (keep[j]) s_surv[wid][cnt + __popc(bm & ((1u << lane) - 1u))] = ch.row0 + (uint32_t)j * 256 + threadIdx.x;
            cnt += __popc(bm);
        }
        u64 o = block_out_base(ctl, lane == 0 ? cnt : 0u);
        o = __shfl_sync(FULL, o, 0);
        __syncwarp();
        if (V.fast) {
            // every column in one REQUIRED page: the PLAIN loads of a survivor are
            // issued together, beside the dictionary column's run -> bits -> value chain
            const int dc = V.dcol;
            const uint32_t dfirst = dc >= 0 ? V.pfirst[dc][0] : 0;
            for (u32 e = lane; e < cnt; e += 32) {
                const u64 oe = o + e;
                if (oe >= S.out_cap) {
                    atomicOr(&ctl->err, (u32)ERR_OUT_OVERFLOW);
                    continue;
                }
                const uint32_t r = s_surv[wid][e];
                u64 x[PQ_FASTC];
#pragma unroll
                for (int c = 0; c < PQ_FASTC; c++)
                    x[c] = s_pwid[c] ? load_plain(file + (s_poff[c] + (u64)r * (u64)s_pwid[c]), s_pwid[c]) : 0;
                const u64 xk = dc >= 0 ? dict_value(file, s_dpg, srun + V.rbeg[0], 0, V.rcnt[0], s_dbw, r - dfirst) : 0;
#pragma unroll
                for (int c = 0; c < PQ_FASTC; c++) {
                    if (c < nc) {
                        const u64 val = c == dc ? xk : x[c];
                        const int t = S.out_type[c];
                        if (t == GB_T_SMALLINT) ((int16_t *)S.out[c])[oe] = (int16_t)(i64)val;
                        else if (t == GB_T_INTEGER) ((int32_t *)S.out[c])[oe] = (int32_t)(i64)val;
                        else ((u64 *)S.out[c])[oe] = val;
                    }
                }
            }
        } else
        for (u32 e = lane; e < cnt; e += 32) {
            const u64 oe = o + e;
            if (oe >= S.out_cap) {
                atomicOr(&ctl->err, (u32)ERR_OUT_OVERFLOW);
                continue;
            }
            const uint32_t r = s_surv[wid][e];
            for (int c = 0; c < S.n_cols; c++) {
                bool valid;
                u64 x = decode_staged(file, pages, runs, page_runs, col_pages, S.n_cols, ch.rg, c, r, V, srun, valid);
                if (!valid) {
                    if (c == S.id_col) x = ~0ull;  // the NULL string id
                    else if (S.out_valid[c]) atomicAnd((unsigned long long *)&S.out_valid[c][oe >> 6], ~(1ull << (oe & 63)));
                }
                switch (S.out_type[c]) {
                case GB_T_SMALLINT: ((int16_t *)S.out[c])[oe] = (int16_t)(i64)x; break;
                case GB_T_INTEGER: ((int32_t *)S.out[c])[oe] = (int32_t)(i64)x; break;
                default: ((u64 *)S.out[c])[oe] = x; break;
                }
            }
        }
        __syncthreads();  // the chunk view and survivor lists are rebuilt for the next chunk
    }
}

// ================================================================== C ABI
static gb_status pq_fail_if_err(Ctl &c) {
    if (c.err & ERR_CORRUPT) {
        set_error("malformed Parquet page data (RLE / bit-packed run outside its page)");
        return GB_ERR_CORRUPT;
    }
    if (c.err & ERR_OUT_OVERFLOW) {
        set_error("Parquet scan output overflow (internal invariant violated)");
        return GB_ERR_CUDA;
    }
    return GB_OK;
}

// Zone map of one row group: false when file column `fcol`'s statistics prove
// that no row passes `q` (IsRowGroupPruned / RowGroupMightMatch,
// physical_planner.cpp:1142-1150, parquet.cpp:3200-3240).  Statistics are
// read as INTEGER (4 bytes), BIGINT (8) or DOUBLE (8) like the reference's
// decode_stat (parquet.cpp:1185-1230), which reads none for SMALLINT.
static bool pq_rg_might_match(const gb_pq_file *f, uint32_t rg, int fcol, const Filter &q) {
    const PqChunk &ch = f->chunks[rg][fcol];
    if (!ch.has_stats) return true;
    const int t = f->cols[fcol].gtype;
    if (t == GB_T_INTEGER || t == GB_T_BIGINT) {
        const size_t w = t == GB_T_INTEGER ? 4 : 8;
        if (ch.stat_min.size() < w || ch.stat_max.size() < w) return true;
        int64_t mn, mx;
        if (w == 4) {
            int32_t a, b;
            memcpy(&a, ch.stat_min.data(), 4);
            memcpy(&b, ch.stat_max.data(), 4);
            mn = a;
            mx = b;
        } else {
            memcpy(&mn, ch.stat_min.data(), 8);
            memcpy(&mx, ch.stat_max.data(), 8);
        }
        const int64_t v = q.ic;
        switch (q.op) {
        case GB_CMP_EQ: return !(v < mn) && !(mx < v);
        case GB_CMP_GT: return !(mx < v) && !(mx == v);
        case GB_CMP_GE: return !(mx < v);
        case GB_CMP_LT: return !(v < mn) && !(mn == v);
        case GB_CMP_LE: return !(v < mn);
        case GB_CMP_NE: return !(mn == v && mx == v);
        default: return true;
        }
    }
    if (t == GB_T_DOUBLE) {
        if (ch.stat_min.size() < 8 || ch.stat_max.size() < 8) return true;
        double mn, mx;
        memcpy(&mn, ch.stat_min.data(), 8);
        memcpy(&mx, ch.stat_max.data(), 8);
        const double v = q.dc;
        switch (q.op) {
        case GB_CMP_EQ: return !(v < mn) && !(mx < v);
        case GB_CMP_GT: return !(mx < v) && !(mx == v);
        case GB_CMP_GE: return !(mx < v);
        case GB_CMP_LT: return !(v < mn) && !(mn == v);
        case GB_CMP_LE: return !(v < mn);
        case GB_CMP_NE: return !(mn == v && mx == v);
        default: return true;
        }
    }
    return true;
}

// Page descriptors of row groups [rg_begin, rg_end) and the given file
// columns (offsets relative to `base`), with run-table slots for the
// dictionary pages; col_pages gets one {begin, end} pair per (rg, column).
// The page metadata a batch decodes from: the file's own, or a copy whose
// offsets point into the batch's decompressed image.
struct PqView {
    const std::vector<std::vector<PqChunk>> *chunks;
    const std::vector<PqPage> *pages;
};

// Row groups a batch skips (zone maps) get empty page ranges: none of their
// bytes is read.
static gb_status pq_page_table(const gb_pq_file *f, const PqView &V, uint32_t rg_begin, uint32_t rg_end,
                               const int32_t *cols, int nc, uint64_t base, const std::vector<char> *live,
                               std::vector<DPage> &pages, std::vector<RunJob> &jobs,
                               std::vector<uint32_t> &col_pages, uint32_t &run_total) {
    for (uint32_t g = rg_begin; g < rg_end; g++) {
        const bool skip = live && !(*live)[g - rg_begin];
        for (int c = 0; c < nc; c++) {
            const PqChunk &ch = (*V.chunks)[g][cols[c]];
            const PqColumn &pc = f->cols[cols[c]];
            col_pages.push_back((uint32_t)pages.size());
            for (uint32_t p = ch.page_begin; p < ch.page_end && !skip; p++) {
                const PqPage &pp = (*V.pages)[p];
                DPage d{};
                d.off = pp.off - base;
                d.first_row = pp.first_row;
                d.n_values = pp.n_values;
                d.bytes = pp.bytes;
                d.kind = pp.kind;
                d.width = pc.width;
                const uint32_t pidx = (uint32_t)pages.size();
                if (pp.kind == 1) {
                    if (ch.dict_off < 0) {
                        set_error("dictionary-encoded page without a dictionary page");
                        return GB_ERR_CORRUPT;
                    }
                    d.dict_off = (uint64_t)ch.dict_off - base;
                    d.dict_n = ch.dict_n;
                    d.run_base = run_total;
                    d.run_cap = std::min<uint32_t>(pp.n_values, pp.bytes) + 1;
                    run_total += d.run_cap;
                    jobs.push_back({d.off, d.bytes, d.n_values, d.run_base, d.run_cap, pidx, 0u});
                }
                if (pp.def_bytes) {
                    // every header byte opens at most one run; bit-packed runs
                    // split every PQ_LEVEL_RUN entries
                    d.def_off = pp.def_off - base;
                    d.def_bytes = pp.def_bytes;
                    d.def_run_base = run_total;
                    d.def_run_cap = pp.def_bytes + pp.n_values / PQ_LEVEL_RUN + 2;
                    run_total += d.def_run_cap;
                    jobs.push_back({d.def_off, d.def_bytes, d.n_values, d.def_run_base, d.def_run_cap, pidx, 1u});
                }
                pages.push_back(d);
            }
            col_pages.push_back((uint32_t)pages.size());
        }
    }
    return GB_OK;
}

// Build the uploaded file's page index once: descriptors of every page and
// the run table of every dictionary page (k_pq_runs over the whole file).
static gb_status pq_build_index(gb_pq_file *f, cudaStream_t st) {
    std::lock_guard<std::mutex> lk(f->idx_mu);
    if (f->idx_ready) return GB_OK;
    const int nfc = (int)f->cols.size();
    std::vector<int32_t> all(nfc);
    for (int c = 0; c < nfc; c++) all[c] = c;
    std::vector<DPage> pages;
    std::vector<RunJob> jobs;
    std::vector<uint32_t> col_pages;
    uint32_t run_total = 0;
    gb_status s = pq_page_table(f, PqView{&f->chunks, &f->pages}, 0, (uint32_t)f->rg_rows.size(), all.data(), nfc, 0,
                                nullptr, pages, jobs, col_pages, run_total);
    if (s) return s;
    void *dp = nullptr, *ctl = nullptr;
    auto fail = [&](cudaError_t e, const char *what) {
        for (void *p : {f->idx_pages, f->idx_runs, f->idx_page_runs, dp, ctl})
            if (p) cudaFree(p);
        f->idx_pages = f->idx_runs = f->idx_page_runs = nullptr;
        (void)cudaGetLastError();
        return cuda_fail(e, what);
    };
    cudaError_t e;
    if ((e = cudaMalloc(&f->idx_pages, std::max<size_t>(pages.size() * sizeof(DPage), 16))) ||
        (e = cudaMalloc(&f->idx_runs, (size_t)run_total * sizeof(DRun) + 16)) ||
        (e = cudaMalloc(&f->idx_page_runs, pages.size() * PQ_PR * 4 + 16)) ||
        (e = cudaMalloc(&dp, jobs.size() * sizeof(RunJob) + 16)) || (e = cudaMalloc(&ctl, sizeof(Ctl))))
        return fail(e, "cudaMalloc (Parquet page index)");
    if ((e = cudaMemcpyAsync(f->idx_pages, pages.data(), pages.size() * sizeof(DPage), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(dp, jobs.data(), jobs.size() * sizeof(RunJob), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemsetAsync(f->idx_page_runs, 0, pages.size() * PQ_PR * 4 + 16, st)) ||
        (e = cudaMemsetAsync(ctl, 0, sizeof(Ctl), st)))
        return fail(e, "cudaMemcpy (Parquet page index)");
    if (!jobs.empty()) {
        k_pq_runs<<<(unsigned)jobs.size(), 128, 0, st>>>((const uint8_t *)f->dev, (const DPage *)f->idx_pages,
                                                         (const RunJob *)dp, (DRun *)f->idx_runs,
                                                         (uint32_t *)f->idx_page_runs, (Ctl *)ctl);
        if ((e = cudaGetLastError())) return fail(e, "k_pq_runs");
    }
    Ctl c;
    if ((e = cudaMemcpyAsync(&c, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st)) || (e = cudaStreamSynchronize(st)))
        return fail(e, "k_pq_runs");
    cudaFree(dp);
    cudaFree(ctl);
    if ((s = pq_fail_if_err(c))) {
        for (void *p : {f->idx_pages, f->idx_runs, f->idx_page_runs}) cudaFree(p);
        f->idx_pages = f->idx_runs = f->idx_page_runs = nullptr;
        return s;
    }
    f->idx_col_pages.swap(col_pages);
    f->idx_ready = true;
    return GB_OK;
}

// ------------------------------------------------ ungrouped dictionary histogram
// SUM / COUNT of one INT64 column without decoding it (TryDictHistogramAgg,
// include/slothdb/execution/dict_histogram.hpp:34, per row group
// ParquetReader::DecodeBigintColumnHistogram, src/storage/parquet.cpp:
// 2726-2897): a histogram of each row group's dictionary indices, then
// sum_idx count[idx] * dict[idx]; PLAIN pages of the column are summed as
// they are.  Sums are exact (128-bit) until the one rounding to double.
struct DHGroup {
    uint64_t dict_off;   // dictionary values (INT64, PLAIN) in the device file
    uint32_t dict_n;     // dictionary entries
    uint32_t hist_base;  // the row group's first histogram slot
};

__device__ __forceinline__ void block_add_i128(__int128 x, u64 cnt, u64 *out3) {
    __shared__ __int128 s_v[32];
    __shared__ u64 s_c[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        const u64 lo = __shfl_down_sync(FULL, (u64)x, o), hi = __shfl_down_sync(FULL, (u64)(x >> 64), o);
        x += (__int128)(((unsigned __int128)hi << 64) | lo);
        cnt += __shfl_down_sync(FULL, cnt, o);
    }
    if (lane == 0) {
        s_v[warp] = x;
        s_c[warp] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __int128 t = 0;
        u64 c = 0;
        for (int w = 0; w < nwarps; w++) {
            t += s_v[w];
            c += s_c[w];
        }
        out3[0] = (u64)t;
        out3[1] = (u64)(t >> 64);
        out3[2] = c;
    }
}

// One CTA per page of the column.  Dictionary pages: every index entry
// below the page's value count bumps its row group's histogram (an RLE run
// once, by its length; indices past the dictionary are skipped, as the
// reference does).  Each warp walks the runs over its slice of the page's
// entries: an RLE run is one atomic; a bit-packed run is unpacked 32 entries
// at a time, and lanes holding the same index as their left neighbour hand
// their count to the first lane of the group, so that a run of equal indices
// costs one atomic.  PLAIN pages: their values and count go to
// part[3 * page].  A page with NULLs sets *nulls (the reference then takes
// the fused path).
__global__ void k_pq_dict_hist(const uint8_t *file, const DPage *pages, const uint32_t *pidx, const DRun *runs,
                               const uint32_t *page_runs, const uint32_t *page_group, const DHGroup *groups,
                               uint32_t *hist, u64 *part, uint32_t *nulls) {
    const uint32_t p = pidx ? pidx[blockIdx.x] : blockIdx.x;  // pidx: the column's pages in a file's page index
    const DPage pg = pages[p];
    u64 *out3 = part + 3 * (u64)blockIdx.x;
    if (pg.def_bytes && page_runs[PQ_PR * p + 3] != pg.n_values) {
        if (threadIdx.x == 0) {
            atomicOr(nulls, 1u);
            out3[0] = out3[1] = out3[2] = 0;
        }
        return;
    }
    const uint32_t total = pg.n_values;
    if (pg.kind == 1) {
        const uint32_t nr = page_runs[PQ_PR * p], bw = page_runs[PQ_PR * p + 1];
        const DRun *rr = runs + pg.run_base;
        const DHGroup G = groups[page_group[blockIdx.x]];
        uint32_t *h = hist + G.hist_base;
        const uint32_t lane = threadIdx.x & 31, nw = blockDim.x >> 5, w = threadIdx.x >> 5;
        const uint32_t per = (total + nw - 1) / nw;
        const uint32_t a = min(total, w * per), b = min(total, a + per);  // this warp's entries
        if (nr > 0 && a < b) {
            for (uint32_t r = run_search(rr, 0, nr, a); r < nr; r++) {
                const DRun rn = rr[r];
                if (rn.start >= b) break;
                const uint32_t s0 = max(rn.start, a);
                const uint32_t s1 = (uint32_t)min((u64)rn.start + rn.cnt, (u64)b);
                if (s0 >= s1) continue;  // entries past the decoded ones
                if (rn.off == 0xffffffffu) {
                    if (lane == 0 && rn.val < G.dict_n) atomicAdd(&h[rn.val], s1 - s0);
                    continue;
                }
                const uint8_t *payload = file + pg.off + rn.off;
                for (uint32_t i0 = s0; i0 < s1; i0 += 32) {
                    const uint32_t i = i0 + lane;
                    uint32_t key = 0xffffffffu;  // no entry, or an index past the dictionary
                    if (i < s1) {
                        const uint32_t idx = load_bits(payload, (u64)(i - rn.start) * bw, bw);
                        if (idx < G.dict_n) key = idx;
                    }
                    const uint32_t left = __shfl_up_sync(FULL, key, 1);
                    const uint32_t heads = __ballot_sync(FULL, lane == 0 || key != left);
                    if (key != 0xffffffffu && (heads >> lane & 1u)) {
                        const uint32_t above = lane == 31 ? 0u : heads >> (lane + 1);
                        const uint32_t n = above ? (uint32_t)__ffs(above) : 32u - lane;
                        atomicAdd(&h[key], n);
                    }
                }
            }
        }
        if (threadIdx.x == 0) out3[0] = out3[1] = out3[2] = 0;
    } else {
        __int128 acc = 0;
        for (uint32_t i = threadIdx.x; i < total; i += blockDim.x) acc += (i64)load_plain(file + pg.off + 8 * (u64)i, 8);
        block_add_i128(acc, threadIdx.x == 0 ? total : 0, out3);
    }
}

static gb_status grow(void *&p, size_t &cap, size_t need);

// One CTA per row group: sum_idx count[idx] * dict[idx] and sum_idx count[idx].
__global__ void k_pq_dict_reduce(const uint8_t *file, const DHGroup *groups, const uint32_t *hist, u64 *part) {
    const DHGroup G = groups[blockIdx.x];
    __int128 acc = 0;
    u64 cnt = 0;
    for (uint32_t e = threadIdx.x; e < G.dict_n; e += blockDim.x) {
        const uint32_t c = hist[G.hist_base + e];
        if (!c) continue;
        acc += (__int128)c * (i64)load_plain(file + G.dict_off + 8 * (u64)e, 8);
        cnt += c;
    }
    block_add_i128(acc, cnt, part + 3 * (u64)blockIdx.x);
}

extern "C" {

gb_status gb_pq_open(const uint8_t *bytes, uint64_t size, gb_pq_file **out) {
    if (!bytes || !out) {
        set_error("null argument");
        return GB_ERR_INVALID;
    }
    *out = nullptr;
    gb_pq_file *f = new gb_pq_file();
    f->host = bytes;
    f->size = size;
    gb_status s = parse_footer(f);
    for (uint32_t g = 0; !s && g < f->chunks.size(); g++)
        for (uint32_t c = 0; !s && c < f->cols.size(); c++) {
            if (f->chunks[g][c].codec != 0 && f->chunks[g][c].codec != 1 && f->chunks[g][c].codec != 6) {
                set_error("Parquet column chunks compressed with codec %d are not supported on the GPU path "
                          "(uncompressed, SNAPPY and ZSTD are)", f->chunks[g][c].codec);
                s = GB_ERR_UNSUPPORTED;
                break;
            }
            f->compressed = f->compressed || f->chunks[g][c].codec != 0;
            s = parse_pages(f, g, c);
        }
    if (s) {
        delete f;
        return s;
    }
    *out = f;
    return GB_OK;
}

uint32_t gb_pq_num_row_groups(const gb_pq_file *f) { return f ? (uint32_t)f->rg_rows.size() : 0; }
uint64_t gb_pq_num_rows(const gb_pq_file *f) { return f ? f->num_rows : 0; }
uint32_t gb_pq_num_columns(const gb_pq_file *f) { return f ? (uint32_t)f->cols.size() : 0; }

gb_status gb_pq_column_info(const gb_pq_file *f, uint32_t col, char *name, uint32_t name_cap, int32_t *type) {
    if (!f || col >= f->cols.size()) return GB_ERR_INVALID;
    if (name && name_cap) {
        strncpy(name, f->cols[col].name.c_str(), name_cap - 1);
        name[name_cap - 1] = 0;
    }
    if (type) *type = f->cols[col].gtype;
    return GB_OK;
}

gb_status gb_pq_row_group_might_match(const gb_pq_file *f, uint32_t rg, const int32_t *col_map, uint32_t n_cols,
                                      const gb_filter *filters, uint32_t n_filters, int32_t *might) {
    if (!f || !might || rg >= f->rg_rows.size() || (n_filters && (!filters || !col_map))) {
        set_error("invalid arguments to gb_pq_row_group_might_match");
        return GB_ERR_INVALID;
    }
    *might = 1;
    for (uint32_t i = 0; i < n_filters; i++) {
        const gb_filter &g = filters[i];
        if (g.col < 0 || (uint32_t)g.col >= n_cols || col_map[g.col] < 0 || col_map[g.col] >= (int)f->cols.size()) {
            set_error("filter %u: column out of range", i);
            return GB_ERR_INVALID;
        }
        Filter q{g.col, g.op, g.i_const, g.d_const};
        if (!pq_rg_might_match(f, rg, col_map[g.col], q)) {
            *might = 0;
            break;
        }
    }
    return GB_OK;
}

gb_status gb_pq_dict_sum(gb_pq_file *f, uint32_t col, uint32_t rg_begin, uint32_t rg_end, int32_t mem, void *stream,
                         int64_t *count, double *sum) {
    if (!f || !count || !sum || col >= f->cols.size() || rg_begin > rg_end || rg_end > f->rg_rows.size()) {
        set_error("invalid arguments to gb_pq_dict_sum");
        return GB_ERR_INVALID;
    }
    *count = 0;
    *sum = 0.0;
    if (f->cols[col].gtype != GB_T_BIGINT) {
        set_error("the dictionary histogram sums INT64 columns");
        return GB_ERR_UNSUPPORTED;
    }
    if (rg_begin == rg_end) return GB_OK;
    for (uint32_t g = rg_begin; g < rg_end; g++) {
        const PqChunk &ch = f->chunks[g][col];
        if (ch.dict_off < 0) {
            set_error("row group %u of the column has no dictionary page", g);
            return GB_ERR_UNSUPPORTED;
        }
        if (ch.codec != 0) {
            set_error("the dictionary histogram reads uncompressed column chunks");
            return GB_ERR_UNSUPPORTED;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    gb_status s = GB_OK;
    std::lock_guard<std::mutex> lk(f->ds_mu);
    void **B = f->ds_buf;
    size_t *C = f->ds_cap;
    // the column's bytes: the resident file, or its row groups' byte range
    const uint8_t *dfile = nullptr;
    uint64_t base = 0, lo = ~0ull, hi = 0;
    void *copy = nullptr;
    if (mem == GB_MEM_DEVICE) {
        if (!f->dev) {
            set_error("gb_pq_upload the file before summing with GB_MEM_DEVICE");
            return GB_ERR_STATE;
        }
        dfile = (const uint8_t *)f->dev;
    } else {
        for (uint32_t g = rg_begin; g < rg_end; g++) {
            lo = std::min(lo, f->chunks[g][col].start);
            hi = std::max(hi, f->chunks[g][col].start + f->chunks[g][col].size);
        }
        if ((s = grow(B[9], C[9], hi - lo + 64))) return s;
        copy = B[9];
        dfile = (const uint8_t *)copy;
        base = lo;
    }
    std::vector<DPage> pages;
    std::vector<RunJob> jobs;
    std::vector<uint32_t> col_pages;
    uint32_t run_total = 0;
    const int32_t cols[1] = {(int32_t)col};
    std::vector<DHGroup> groups;
    std::vector<uint32_t> page_group;
    uint64_t hist_n = 0;
    void *d_pages = nullptr, *d_runs = nullptr, *d_page_runs = nullptr, *d_jobs = nullptr, *d_pg = nullptr,
         *d_groups = nullptr, *d_hist = nullptr, *d_part = nullptr, *d_ctl = nullptr;
    auto done = [&](gb_status r) { return r; };
    if (copy && cudaMemcpyAsync(copy, f->host + lo, hi - lo, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return done(cuda_fail(cudaGetLastError(), "cudaMemcpyAsync"));
    // a resident uncompressed file: its page index (descriptors and run
    // tables, built once for every column; a file it cannot index is tabled
    // per call)
    const bool indexed = mem == GB_MEM_DEVICE && !f->compressed && pq_build_index(f, st) == GB_OK;
    std::vector<uint32_t> pidx;
    if (indexed) {
        const size_t nfc = f->cols.size();
        for (uint32_t g = rg_begin; g < rg_end; g++) {
            col_pages.push_back((uint32_t)pidx.size());
            for (uint32_t q = f->idx_col_pages[2 * (g * nfc + col)]; q < f->idx_col_pages[2 * (g * nfc + col) + 1]; q++)
                pidx.push_back(q);
            col_pages.push_back((uint32_t)pidx.size());
        }
    } else if ((s = pq_page_table(f, PqView{&f->chunks, &f->pages}, rg_begin, rg_end, cols, 1, base, nullptr, pages,
                                  jobs, col_pages, run_total))) {
        return done(s);
    }
    for (uint32_t g = rg_begin; g < rg_end; g++) {
        const PqChunk &ch = f->chunks[g][col];
        if (hist_n + ch.dict_n > 0xffffffffull) return done(GB_ERR_UNSUPPORTED);
        groups.push_back({(uint64_t)ch.dict_off - base, ch.dict_n, (uint32_t)hist_n});
        hist_n += ch.dict_n;
        const uint32_t k = g - rg_begin;
        for (uint32_t q = col_pages[2 * k]; q < col_pages[2 * k + 1]; q++) page_group.push_back(k);
    }
    const size_t np = indexed ? pidx.size() : pages.size(), ng = groups.size();
    cudaError_t e;
    if ((s = grow(B[0], C[0], np * sizeof(DPage) + 16)) || (s = grow(B[1], C[1], (size_t)run_total * sizeof(DRun) + 16)) ||
        (s = grow(B[2], C[2], np * PQ_PR * 4 + 16)) || (s = grow(B[3], C[3], jobs.size() * sizeof(RunJob) + 16)) ||
        (s = grow(B[4], C[4], np * 4 + 16)) || (s = grow(B[5], C[5], ng * sizeof(DHGroup) + 16)) ||
        (s = grow(B[6], C[6], hist_n * 4 + 16)) || (s = grow(B[7], C[7], (np + ng) * 24 + 16)) ||
        (s = grow(B[8], C[8], sizeof(Ctl))) || (s = grow(B[10], C[10], pidx.size() * 4 + 16)))
        return s;
    d_pages = B[0], d_runs = B[1], d_page_runs = B[2], d_jobs = B[3], d_pg = B[4], d_groups = B[5], d_hist = B[6],
    d_part = B[7], d_ctl = B[8];
    if (indexed) {
        d_pages = f->idx_pages, d_runs = f->idx_runs, d_page_runs = f->idx_page_runs;
        if ((e = cudaMemcpyAsync(B[10], pidx.data(), pidx.size() * 4, cudaMemcpyHostToDevice, st)))
            return done(cuda_fail(e, "cudaMemcpyAsync (dictionary histogram)"));
    } else if ((e = cudaMemcpyAsync(d_pages, pages.data(), np * sizeof(DPage), cudaMemcpyHostToDevice, st)) ||
               (e = cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(RunJob), cudaMemcpyHostToDevice, st)) ||
               (e = cudaMemsetAsync(d_page_runs, 0, np * PQ_PR * 4 + 16, st))) {
        return done(cuda_fail(e, "cudaMemcpyAsync (dictionary histogram)"));
    }
    if ((e = cudaMemcpyAsync(d_pg, page_group.data(), np * 4, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(d_groups, groups.data(), ng * sizeof(DHGroup), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemsetAsync(d_hist, 0, hist_n * 4 + 16, st)) || (e = cudaMemsetAsync(d_ctl, 0, sizeof(Ctl), st)))
        return done(cuda_fail(e, "cudaMemcpyAsync (dictionary histogram)"));
    if (!jobs.empty()) {  // a batch's own run tables (the file in host memory)
        k_pq_runs<<<(unsigned)jobs.size(), 128, 0, st>>>(dfile, (const DPage *)d_pages, (const RunJob *)d_jobs,
                                                         (DRun *)d_runs, (uint32_t *)d_page_runs, (Ctl *)d_ctl);
        Ctl c;
        if ((e = cudaGetLastError()) || (e = cudaMemcpyAsync(&c, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st)) ||
            (e = cudaStreamSynchronize(st)))
            return done(cuda_fail(e, "k_pq_runs"));
        if ((s = pq_fail_if_err(c))) return done(s);
    }
    uint32_t *nulls = (uint32_t *)d_ctl;  // the control block's first word, zeroed above
    if ((e = cudaMemsetAsync(nulls, 0, 4, st))) return done(cuda_fail(e, "cudaMemsetAsync"));
    if (np)
        k_pq_dict_hist<<<(unsigned)np, 256, 0, st>>>(dfile, (const DPage *)d_pages,
                                                    indexed ? (const uint32_t *)B[10] : nullptr,
                                                    (const DRun *)d_runs, (const uint32_t *)d_page_runs,
                                                    (const uint32_t *)d_pg, (const DHGroup *)d_groups,
                                                    (uint32_t *)d_hist, (u64 *)d_part, nulls);
    k_pq_dict_reduce<<<(unsigned)ng, 256, 0, st>>>(dfile, (const DHGroup *)d_groups, (const uint32_t *)d_hist,
                                                  (u64 *)d_part + 3 * np);
    std::vector<u64> part(3 * (np + ng));
    uint32_t has_nulls = 0;
    if ((e = cudaGetLastError()) ||
        (e = cudaMemcpyAsync(part.data(), d_part, part.size() * 8, cudaMemcpyDeviceToHost, st)) ||
        (e = cudaMemcpyAsync(&has_nulls, nulls, 4, cudaMemcpyDeviceToHost, st)) || (e = cudaStreamSynchronize(st)))
        return done(cuda_fail(e, "k_pq_dict_hist"));
    if (has_nulls) {
        set_error("a page of the column holds NULLs (the histogram sums every row)");
        return done(GB_ERR_UNSUPPORTED);
    }
    __int128 t = 0;
    unsigned long long n = 0;
    for (size_t i = 0; i < np + ng; i++) {
        t += (__int128)(((unsigned __int128)part[3 * i + 1] << 64) | part[3 * i]);
        n += part[3 * i + 2];
    }
    *count = (int64_t)n;
    *sum = (double)t;
    return done(GB_OK);
}

gb_status gb_pq_upload(gb_pq_file *f, void *stream) {
    if (!f) return GB_ERR_INVALID;
    if (f->dev) return GB_OK;
    // 64 bytes of slack: the word loads of a level or index stream that ends
    // the file may touch up to 15 bytes past its last byte
    GB_CUDA(cudaMalloc(&f->dev, f->size + 64));
    GB_CUDA(cudaMemcpyAsync(f->dev, f->host, f->size, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    GB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return GB_OK;
}

void gb_pq_close(gb_pq_file *f) {
    if (!f) return;
    if (f->dev) cudaFree(f->dev);
    for (void *p : {f->idx_pages, f->idx_runs, f->idx_page_runs})
        if (p) cudaFree(p);
    for (void *p : f->ds_buf)
        if (p) cudaFree(p);
    delete f;
}

}  // extern "C"

// The aggregate-side ingest lives here so the handle's internals stay in
// gb_agg.cu: gb_agg_ingest_parquet decodes + filters + compacts a batch of row
// groups, then hands the compacted device columns to gb_agg_ingest.
struct PqScratch {
    void *file_dev = nullptr;
    size_t file_cap = 0;
    void *pages = nullptr, *runs = nullptr, *page_runs = nullptr, *dict_pages = nullptr, *col_pages = nullptr,
         *chunks = nullptr, *ctl = nullptr;
    size_t pages_cap = 0, runs_cap = 0, page_runs_cap = 0, dict_pages_cap = 0, col_pages_cap = 0, chunks_cap = 0,
           ctl_cap = 0;
    void *out[GB_MAX_COLS] = {};
    size_t out_cap_rows = 0;
    void *out_valid[GB_MAX_COLS] = {};  // validity words of OPTIONAL columns' output
    size_t out_valid_cap[GB_MAX_COLS] = {};
    // VARCHAR dictionary pages of a batch: descriptors, value sources,
    // compacted offsets and bytes
    void *dicts = nullptr, *dsrc = nullptr, *doffs = nullptr, *dbytes = nullptr, *dmatch = nullptr,
         *dcounts = nullptr;  // value counts of PLAIN BYTE_ARRAY pages
    size_t dicts_cap = 0, dsrc_cap = 0, doffs_cap = 0, dbytes_cap = 0, dmatch_cap = 0, dcounts_cap = 0;
    // compressed batches: the decompressed image, its jobs, the level lengths found inside
    void *img = nullptr, *ijobs = nullptr, *ilvl = nullptr;
    size_t img_cap = 0, ijobs_cap = 0, ilvl_cap = 0;
    void *views = nullptr;  // per chunk of the batch: its view (k_pq_views)
    size_t views_cap = 0;
    void *zjobs = nullptr, *zscratch = nullptr;  // ZSTD pieces and their decoders' tables
    size_t zjobs_cap = 0, zscratch_cap = 0;
};

static gb_status grow(void *&p, size_t &cap, size_t need) {
    if (need <= cap) return GB_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max(need, (size_t)4096);
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return cuda_fail(e, "cudaMalloc (parquet scratch)");
    }
    cap = want;
    return GB_OK;
}

static std::mutex g_pq_mu;
static std::map<gb_agg *, PqScratch *> g_pq_scratch;

static PqScratch *g_scratch_for(gb_agg *h) {
    std::lock_guard<std::mutex> lk(g_pq_mu);
    auto it = g_pq_scratch.find(h);
    if (it != g_pq_scratch.end()) return it->second;
    PqScratch *s = new PqScratch();
    g_pq_scratch[h] = s;
    return s;
}

void gb_pq_release_scratch(gb_agg *h) {
    PqScratch *s = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_pq_mu);
        auto it = g_pq_scratch.find(h);
        if (it == g_pq_scratch.end()) return;
        s = it->second;
        g_pq_scratch.erase(it);
    }
    for (void *p : {s->file_dev, s->pages, s->runs, s->page_runs, s->dict_pages, s->col_pages, s->chunks, s->ctl,
                    s->dicts, s->dsrc, s->doffs, s->dbytes, s->dmatch, s->dcounts, s->img, s->ijobs, s->ilvl, s->views, s->zjobs,
                    s->zscratch})
        if (p) cudaFree(p);
    for (void *p : s->out)
        if (p) cudaFree(p);
    for (void *p : s->out_valid)
        if (p) cudaFree(p);
    delete s;
}

// The batch's dictionary pages of VARCHAR file column `fcol`: walk, compact
// and encode their values into the handle's string dictionary.  *ids gets
// the ids of all values, page after page in row-group order (device).
// The string predicates on a batch's VARCHAR key.
struct PqStrFilters {
    int32_t n;
    int32_t op[GB_MAX_FILTERS];
    const void *ptr[GB_MAX_FILTERS];
    u64 len[GB_MAX_FILTERS];
};

// Per dictionary entry of a batch: 1 when its string passes every string
// predicate on the key (the dictionary match table of BuildTypedKeepMask,
// physical_planner.cpp:505-720: each entry is tested once, rows look it up).
__global__ void k_pq_dict_match(const uint8_t *bytes, const int64_t *offs, u64 n, const __grid_constant__ PqStrFilters F,
                                uint8_t *match) {
    for (u64 e = blockIdx.x * (u64)blockDim.x + threadIdx.x; e < n; e += (u64)gridDim.x * blockDim.x) {
        const int64_t b = offs[e], len = offs[e + 1] - b;
        bool m = true;
        for (int q = 0; q < F.n && m; q++) m = str_pred(F.op[q], bytes + b, (u64)len, F.ptr[q], F.len[q]);
        match[e] = m ? 1 : 0;
    }
}

// The batch's VARCHAR-key strings: each live row group's dictionary page,
// then its PLAIN data pages (plain_at[page] = {first entry, values} for
// every PLAIN page, page = index into V.pages).
static gb_status pq_varchar_dict(gb_agg *h, const PqView &V, PqScratch *S, const uint8_t *dfile, uint64_t base,
                                 uint32_t rg_begin, uint32_t rg_end, const std::vector<char> &live, int fcol,
                                 Ctl *dctl, cudaStream_t st, const int64_t **ids, const PqStrFilters &SF,
                                 const uint8_t **match, std::unordered_map<uint32_t, std::pair<uint64_t, uint32_t>> &plain_at) {
    gb_status s;
    // PLAIN pages: their value counts first (a walk that only counts)
    std::vector<uint32_t> plain_pages;
    std::vector<DDict> pd;
    for (uint32_t g = rg_begin; g < rg_end; g++) {
        if (!live[g - rg_begin]) continue;
        const PqChunk &ch = (*V.chunks)[g][fcol];
        for (uint32_t p = ch.page_begin; p < ch.page_end; p++) {
            const PqPage &pg = (*V.pages)[p];
            if (pg.kind != 0) continue;
            DDict d{};
            d.off = pg.off - base;
            d.n = pg.bytes / 4;  // a bound: every value has a 4-byte length
            d.bytes = pg.bytes;
            pd.push_back(d);
            plain_pages.push_back(p);
        }
    }
    std::vector<uint32_t> counts(pd.size(), 0);
    if (!pd.empty()) {
        if ((s = grow(S->dicts, S->dicts_cap, pd.size() * sizeof(DDict) + 16)) ||
            (s = grow(S->dcounts, S->dcounts_cap, pd.size() * 4 + 16)))
            return s;
        GB_CUDA(cudaMemcpyAsync(S->dicts, pd.data(), pd.size() * sizeof(DDict), cudaMemcpyHostToDevice, st));
        k_pq_dict_walk<<<(unsigned)pd.size(), 128, 0, st>>>(dfile, (const DDict *)S->dicts, nullptr, nullptr, dctl,
                                                            (uint32_t *)S->dcounts);
        GB_CUDA(cudaGetLastError());
        gb_agg_count_launch(h, 1);
        Ctl c;
        GB_CUDA(cudaMemcpyAsync(counts.data(), S->dcounts, pd.size() * 4, cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaMemcpyAsync(&c, dctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
        if ((s = pq_fail_if_err(c))) return s;
        for (size_t i = 0; i < pd.size(); i++) {
            const PqPage &pg = (*V.pages)[plain_pages[i]];
            // a REQUIRED page holds one value per row; an OPTIONAL one at most
            if (pg.def_bytes == 0 ? counts[i] != pg.n_values : counts[i] > pg.n_values)
                return pq_corrupt("PLAIN BYTE_ARRAY value count");
        }
    }
    std::vector<DDict> dd;
    uint64_t D = 0, B = 0;
    size_t pi = 0;
    for (uint32_t g = rg_begin; g < rg_end; g++) {
        if (!live[g - rg_begin]) continue;
        const PqChunk &ch = (*V.chunks)[g][fcol];
        if (ch.dict_off >= 0) {
            if ((uint64_t)ch.dict_n * 4 > ch.dict_bytes) return pq_corrupt("dictionary size");
            DDict d{};
            d.off = (uint64_t)ch.dict_off - base;
            d.entry_base = D;
            d.compact_base = B;
            d.n = ch.dict_n;
            d.bytes = ch.dict_bytes;
            D += d.n;
            B += (uint64_t)d.bytes - 4 * (uint64_t)d.n;
            dd.push_back(d);
        }
        for (; pi < plain_pages.size() && (*V.pages)[plain_pages[pi]].rg == g; pi++) {
            DDict d = pd[pi];
            d.entry_base = D;
            d.compact_base = B;
            d.n = counts[pi];
            plain_at[plain_pages[pi]] = {D, counts[pi]};
            D += d.n;
            B += (uint64_t)d.bytes - 4 * (uint64_t)d.n;
            dd.push_back(d);
        }
    }
    if (D == 0) {
        set_error("VARCHAR column with an empty dictionary");
        return GB_ERR_UNSUPPORTED;
    }
    if ((s = grow(S->dicts, S->dicts_cap, dd.size() * sizeof(DDict) + 16)) ||
        (s = grow(S->dsrc, S->dsrc_cap, D * 8 + 16)) || (s = grow(S->doffs, S->doffs_cap, (D + 1) * 8 + 16)) ||
        (s = grow(S->dbytes, S->dbytes_cap, B + 16)))
        return s;
    const int64_t total = (int64_t)B;
    GB_CUDA(cudaMemcpyAsync(S->dicts, dd.data(), dd.size() * sizeof(DDict), cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync((int64_t *)S->doffs + D, &total, 8, cudaMemcpyHostToDevice, st));
    k_pq_dict_walk<<<(unsigned)dd.size(), 128, 0, st>>>(dfile, (const DDict *)S->dicts, (u64 *)S->dsrc,
                                                        (int64_t *)S->doffs, dctl, nullptr);
    GB_CUDA(cudaGetLastError());
    Ctl c;
    GB_CUDA(cudaMemcpyAsync(&c, dctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if ((s = pq_fail_if_err(c))) return s;  // no value is copied from a page that failed its walk
    k_pq_dict_copy<<<(unsigned)std::min<uint64_t>((D + 255) / 256, (uint64_t)sm_count() * 8), 256, 0, st>>>(
        dfile, (const u64 *)S->dsrc, (const int64_t *)S->doffs, D, (uint8_t *)S->dbytes);
    GB_CUDA(cudaGetLastError());
    gb_agg_count_launch(h, 2);
    *match = nullptr;
    if (SF.n) {
        if ((s = grow(S->dmatch, S->dmatch_cap, D + 16))) return s;
        k_pq_dict_match<<<(unsigned)std::min<uint64_t>((D + 255) / 256, (uint64_t)sm_count() * 8), 256, 0, st>>>(
            (const uint8_t *)S->dbytes, (const int64_t *)S->doffs, D, SF, (uint8_t *)S->dmatch);
        GB_CUDA(cudaGetLastError());
        gb_agg_count_launch(h, 1);
        *match = (const uint8_t *)S->dmatch;
    }
    return gb_agg_encode_strings(h, (const uint8_t *)S->dbytes, (const int64_t *)S->doffs, D, B, st, ids);
}

// ------------------------------------------------ compressed column chunks
// One piece of a batch's decompressed image: `src_len` bytes at file offset
// `src` copied (mode 0), inflated from a raw Snappy block (mode 1, the codec
// of parquet.cpp:44-90, the vendored snappy 1.2.1) or from ZSTD frames (mode
// 2, parquet.cpp:693-736) into `dst_len` bytes at image offset `dst`.  lvl_slot != ~0: the piece is a page v1 of an
// OPTIONAL column, whose first 4 bytes (the level length) go to lvl[slot].
struct InflateJob {
    uint64_t src, dst;
    uint32_t src_len, dst_len;
    uint32_t mode, lvl_slot;
};

// One warp per piece.  Snappy (the published format): a varint with the
// uncompressed length, then elements whose tag's low 2 bits say literal (00:
// length in the tag or in 1-4 following bytes), or copy with a 1-, 2- or
// 4-byte offset (01/10/11) of an earlier output position, possibly
// overlapping the bytes it writes.
//
// The warp decodes a round of elements at a time.  Lane L reads the 8
// compressed bytes at ip + L (one aligned word per lane, redistributed by
// shuffles) and decodes the element a tag there would be; the chain of real
// tags from ip (each start plus its element's compressed size) is walked with
// shuffles over the lanes' sizes, up to the first start at or past ip + 32.
// An exclusive scan of the starts' lengths places each element in the output.
// Each output byte of the round gets its source in a per-warp shared map: a
// compressed position (literal) or an earlier output position (copy; an
// overlapping copy repeats its first `offset` bytes).  A source inside the
// round is followed through the map to a byte written before the round or a
// literal byte, so that all bytes of a round are independent and the warp
// writes them with one load and one store each.  A literal longer than 64
// bytes (the last element of its round) is copied by the whole warp after
// the round.  Every length and offset is checked against the piece's bounds;
// a malformed block sets ERR_CORRUPT and stops.
#define PQ_INF_MAP 1024   // output bytes of one round: at most 16 elements of at most 64 bytes
#define PQ_INF_LONG 64    // literals longer than this are copied by the warp
#define PQ_INF_LIT 0x80000000u

__device__ __forceinline__ void pq_inflate_piece(const uint8_t *__restrict__ file, const InflateJob J, uint8_t *img,
                                                 uint32_t *lvl, Ctl *ctl, uint32_t *map, const int lane) {
    const uint8_t *src = file + J.src;
    uint8_t *dst = img + J.dst;
    bool bad = false;
    if (J.mode == 0) {
        for (uint32_t i = lane; i < J.src_len; i += 32) dst[i] = src[i];
    } else {
        const uint32_t slen = J.src_len, dlen = J.dst_len;
        uint32_t ip = 0, op = 0;
        if (lane == 0) {  // the preamble: the uncompressed length
            uint64_t ulen = 0;
            int sh = 0;
            for (;;) {
                if (ip >= slen || sh > 28) {
                    bad = true;
                    break;
                }
                const uint8_t b = src[ip++];
                ulen |= (uint64_t)(b & 0x7f) << sh;
                if (!(b & 0x80)) break;
                sh += 7;
            }
            if (ulen != dlen) bad = true;
        }
        bad = __shfl_sync(FULL, (int)bad, 0) != 0;
        ip = __shfl_sync(FULL, ip, 0);
        while (!bad && op < dlen) {
            if (ip >= slen) {
                bad = true;
                break;
            }
            // bytes [ip + lane, ip + lane + 8): lanes 0..10 load the aligned words over
            // [ip, ip + 40) and the warp redistributes them
            const uint8_t *blk = (const uint8_t *)((uintptr_t)(src + ip) & ~(uintptr_t)3);
            uint32_t word = 0;
            if (lane < 11) {
                const uint8_t *wp = blk + 4 * lane;
                if (blk >= src && blk + 44 <= src + slen) {
                    word = __ldg((const uint32_t *)wp);
                } else {
                    for (int k = 0; k < 4; k++)
                        if (wp + k >= src && wp + k < src + slen) word |= (uint32_t)__ldg(wp + k) << (8 * k);
                }
            }
            const uint32_t sh0 = (uint32_t)((uintptr_t)(src + ip) & 3) + (uint32_t)lane;
            const uint32_t w0 = __shfl_sync(FULL, word, sh0 >> 2);
            const uint32_t w1 = __shfl_sync(FULL, word, (sh0 >> 2) + 1);
            const uint32_t w2 = __shfl_sync(FULL, word, (sh0 >> 2) + 2);
            const uint32_t lo = __funnelshift_r(w0, w1, 8 * (sh0 & 3)), hi = __funnelshift_r(w1, w2, 8 * (sh0 & 3));
            // the element a tag at ip + lane would be (selects, no branches)
            const uint32_t tag = lo & 0xffu, t = tag & 3u, l6 = tag >> 2;
            const uint32_t rest = (lo >> 8) | (hi << 24);  // bytes 1..4 after the tag
            const uint32_t nb = l6 >= 60 ? l6 - 59 : 0;     // a literal's length bytes
            const uint32_t lraw = nb ? rest & (0xffffffffu >> (32 - 8 * nb)) : l6;
            const uint32_t hdr = t == 0 ? 1 + nb : (t == 1 ? 2 : (t == 2 ? 3 : 5));
            const uint32_t len = t == 0 ? lraw + 1 : (t == 1 ? 4 + (l6 & 7u) : l6 + 1);  // 0 after a wrap
            const uint32_t off = t == 1 ? ((tag >> 5) << 8) | (rest & 0xffu) : (t == 2 ? rest & 0xffffu : rest);
            const uint32_t cs = t != 0 ? hdr : (lraw >= 0x7fff0000u ? 0x7fffffffu : hdr + lraw + 1);
            // the chain of starts from ip
            const uint32_t avail = min(32u, slen - ip);
            uint32_t pos = 0, mask = 0;
            while (pos < avail) {
                mask |= 1u << pos;
                pos += __shfl_sync(FULL, cs, pos);
            }
            const bool start = (mask >> lane) & 1u;
            // lengths clamped in the scan (16 starts of at most 2^26 cannot wrap); the one
            // element that may be longer, a long literal, is the round's last start
            uint32_t mylen = start ? min(len, 1u << 26) : 0, incl = mylen;
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, incl, d);
                if (lane >= d) incl += y;
            }
            const uint32_t excl = incl - mylen;  // round-relative output position
            uint32_t total = __shfl_sync(FULL, incl, 31);
            const uint32_t p = ip + (uint32_t)lane;  // compressed position of this lane's tag
            const uint64_t o = (uint64_t)op + excl;
            const bool live = start && o < dlen;  // elements after the last output byte are ignored
            const bool mybad = live && ((uint64_t)p + cs > slen || len == 0 || o + len > dlen ||
                                        (t != 0 && (off == 0 || off > o)));
            if (__any_sync(FULL, mybad)) {
                bad = true;
                break;
            }
            // outputs past dlen (trailing elements) and the long literal are not mapped
            if (total > dlen - op) total = dlen - op;
            const uint32_t lmask = __ballot_sync(FULL, live && t == 0 && len > PQ_INF_LONG);
            uint32_t mapped = total, lit_at = 0, lit_len = 0, lit_src = 0;
            if (lmask) {
                const int ll = __ffs(lmask) - 1;
                mapped = __shfl_sync(FULL, excl, ll);
                lit_len = __shfl_sync(FULL, len, ll);
                lit_src = __shfl_sync(FULL, p + hdr, ll);
                lit_at = op + mapped;
                total = mapped + lit_len;
            }
            if (mapped > PQ_INF_MAP) {  // unreachable: 16 starts of at most 64 bytes
                bad = true;
                break;
            }
            if (start && excl < mapped) {
                // a literal's byte b comes from q + b; a copy's from o - off + (b mod off)
                const uint32_t base = t == 0 ? PQ_INF_LIT | (p + hdr) : (uint32_t)o - off;
                const uint32_t per = t == 0 ? 0xffffffffu : off;
                for (uint32_t b = 0, r = 0; b < len; b++) {
                    map[excl + b] = base + r;
                    r = r + 1 == per ? 0 : r + 1;
                }
            }
            __syncwarp();
            for (uint32_t k = lane; k < mapped; k += 32) {
                uint32_t s = map[k];
                while (!(s & PQ_INF_LIT) && s >= op) s = map[s - op];
                dst[op + k] = (s & PQ_INF_LIT) ? __ldg(src + (s & ~PQ_INF_LIT)) : dst[s];
            }
            if (lit_len) {
                for (uint32_t b = lane; b < lit_len; b += 32) dst[lit_at + b] = __ldg(src + lit_src + b);
            }
            __syncwarp();
            op += total;
            ip += pos;
        }
    }
    if (bad && lane == 0) atomicOr(&ctl->err, (u32)ERR_CORRUPT);
    __syncwarp();
    if (lane == 0 && J.lvl_slot != ~0u) {
        uint32_t l4 = ~0u;  // too short to hold a level length: corrupt
        if (!bad && J.dst_len >= 4)
            l4 = (uint32_t)dst[0] | ((uint32_t)dst[1] << 8) | ((uint32_t)dst[2] << 16) | ((uint32_t)dst[3] << 24);
        lvl[J.lvl_slot] = l4;
    }
}

// Each warp claims pieces from a counter (the word after the last job, zero
// at launch) until none is left; the host lists the pieces longest first, so
// that the long pages start early and no warp idles beside a long one.
__global__ void __launch_bounds__(256) k_pq_inflate(const uint8_t *__restrict__ file, InflateJob *jobs,
                                                    uint32_t n, uint8_t *img, uint32_t *lvl, Ctl *ctl) {
    __shared__ uint32_t s_map[8][PQ_INF_MAP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *next = (uint32_t *)(jobs + n);
    for (;;) {
        uint32_t j = 0;
        if (lane == 0) j = atomicAdd(next, 1u);
        j = __shfl_sync(FULL, j, 0);
        if (j >= n) return;  // the whole warp
        pq_inflate_piece(file, jobs[j], img, lvl, ctl, s_map[warp], lane);
    }
}

// ZSTD pieces (mode 2): one warp per piece, claimed from a counter (the word
// after the last job) longest first, decoded by its first lane with the
// warp's 13.3 KB of tables in `scratch` (a frame is one serial stream;
// pieces on the lanes of one warp would serialise on their divergent
// branches).  The tables stay in global memory.  Launch bounds of 5 blocks
// an SM hold a thread to 96 registers: 20 warps per SM decode at once, which
// measured faster than 16 warps at 128 registers and than 24 or 32 warps,
// whose tighter bounds spill.  A frame that does not
// decode to exactly dst_len bytes sets ERR_CORRUPT.
__global__ void __launch_bounds__(128, 5) k_pq_unzstd(const uint8_t *__restrict__ file, InflateJob *jobs, uint32_t n,
                                                   uint8_t *img, uint32_t *lvl, Ctl *ctl, gbz::ZsScratch *scratch) {
    if ((threadIdx.x & 31) != 0) return;
    gbz::ZsScratch &Z = scratch[(blockIdx.x * blockDim.x + threadIdx.x) >> 5];
    uint32_t *next = (uint32_t *)(jobs + n);
    for (;;) {
        const uint32_t j = atomicAdd(next, 1u);
        if (j >= n) return;
        const InflateJob J = jobs[j];
        uint8_t *dst = img + J.dst;
        const int64_t got = gbz::zstd_decompress(file + J.src, J.src_len, dst, J.dst_len, Z);
        const bool bad = got != (int64_t)J.dst_len;
        if (bad) atomicOr(&ctl->err, (u32)ERR_CORRUPT);
        if (J.lvl_slot != ~0u) {
            uint32_t l4 = ~0u;  // too short to hold a level length: corrupt
            if (!bad && J.dst_len >= 4)
                l4 = (uint32_t)dst[0] | ((uint32_t)dst[1] << 8) | ((uint32_t)dst[2] << 16) | ((uint32_t)dst[3] << 24);
            lvl[J.lvl_slot] = l4;
        }
    }
}

// Build a batch's decompressed image: per live row group and mapped file
// column, an uncompressed chunk is copied whole, a SNAPPY chunk's
// dictionary page and data pages are inflated (page v2 levels copied as
// stored); ic / ip get the batch's page metadata with image offsets.  A page
// v1 of an OPTIONAL column learns its level length from the inflated bytes
// (one device round trip).
static gb_status pq_inflate_batch(gb_agg *h, const gb_pq_file *f, PqScratch *S, const uint8_t *dfile, uint64_t base,
                                  uint32_t rg_begin, uint32_t rg_end, const std::vector<char> &live,
                                  const int32_t *col_map, int nc, Ctl *dctl, cudaStream_t st,
                                  std::vector<std::vector<PqChunk>> &ic, std::vector<PqPage> &ip) {
    ic = f->chunks;
    ip = f->pages;
    std::vector<int32_t> fcols(col_map, col_map + nc);
    std::sort(fcols.begin(), fcols.end());
    fcols.erase(std::unique(fcols.begin(), fcols.end()), fcols.end());
    std::vector<InflateJob> jobs;
    std::vector<uint32_t> pending;
    uint64_t pos = 0;
    auto place = [&](uint64_t n) {
        const uint64_t at = pos;
        pos += (n + 15) & ~15ull;
        return at;
    };
    for (uint32_t g = rg_begin; g < rg_end; g++) {
        if (!live[g - rg_begin]) continue;
        for (int32_t fc : fcols) {
            PqChunk &ch = ic[g][fc];
            if (ch.codec == 0) {
                if (ch.size > 0xffffffffull) return pq_corrupt("column chunk size");
                const uint64_t at = place(ch.size);
                jobs.push_back({ch.start - base, at, (uint32_t)ch.size, (uint32_t)ch.size, 0u, ~0u});
                const int64_t d = (int64_t)at - (int64_t)ch.start;
                if (ch.dict_off >= 0) ch.dict_off += d;
                for (uint32_t p = ch.page_begin; p < ch.page_end; p++) {
                    ip[p].off = (uint64_t)((int64_t)ip[p].off + d);
                    if (ip[p].def_bytes) ip[p].def_off = (uint64_t)((int64_t)ip[p].def_off + d);
                }
                continue;
            }
            const uint32_t cm = ch.codec == 6 ? 2u : 1u;  // ZSTD or SNAPPY
            if (ch.dict_off >= 0) {
                const uint64_t at = place(ch.dict_bytes);
                jobs.push_back({ch.dict_src - base, at, ch.dict_src_bytes, ch.dict_bytes, cm, ~0u});
                ch.dict_off = (int64_t)at;
            }
            for (uint32_t p = ch.page_begin; p < ch.page_end; p++) {
                PqPage &pg = ip[p];
                const uint64_t at = place((uint64_t)pg.lvl_copy + pg.raw_bytes);
                if (pg.lvl_copy) {
                    jobs.push_back({pg.src_off - pg.lvl_copy - base, at, pg.lvl_copy, pg.lvl_copy, 0u, ~0u});
                    pg.def_off = at;
                    pg.def_bytes = pg.lvl_copy;
                }
                jobs.push_back({pg.src_off - base, at + pg.lvl_copy, pg.src_bytes, pg.raw_bytes, pg.stored ? 0u : cm,
                                pg.lvl_pending ? (uint32_t)pending.size() : ~0u});
                if (pg.lvl_pending) pending.push_back(p);
                pg.off = at + pg.lvl_copy;
                pg.bytes = pg.raw_bytes;
            }
        }
    }
    // the ZSTD pieces in a list of their own (a kernel of their own)
    std::vector<InflateJob> zjobs;
    for (size_t k = 0; k < jobs.size();) {
        if (jobs[k].mode == 2) {
            zjobs.push_back(jobs[k]);
            jobs[k] = jobs.back();
            jobs.pop_back();
        } else {
            k++;
        }
    }
    // longest first (a stored piece costs about a sixteenth of an inflated
    // one per byte), then a zero word: the kernels' claim counters
    auto longest = [](const InflateJob &a, const InflateJob &b) {
        return (a.mode ? (uint64_t)a.dst_len * 16 : a.dst_len) > (b.mode ? (uint64_t)b.dst_len * 16 : b.dst_len);
    };
    std::stable_sort(jobs.begin(), jobs.end(), longest);
    std::stable_sort(zjobs.begin(), zjobs.end(), longest);
    const size_t n_jobs = jobs.size(), n_z = zjobs.size();
    jobs.push_back({0, 0, 0, 0, 0, 0});
    zjobs.push_back({0, 0, 0, 0, 0, 0});
    const size_t z_blocks = std::min<size_t>((n_z + 3) / 4, (size_t)sm_count() * 16);  // 4 warps per block
    gb_status s;
    if ((s = grow(S->img, S->img_cap, pos + 64)) || (s = grow(S->ijobs, S->ijobs_cap, jobs.size() * sizeof(InflateJob) + 16)) ||
        (s = grow(S->ilvl, S->ilvl_cap, pending.size() * 4 + 16)) ||
        (n_z && ((s = grow(S->zjobs, S->zjobs_cap, zjobs.size() * sizeof(InflateJob) + 16)) ||
                 (s = grow(S->zscratch, S->zscratch_cap, z_blocks * 4 * sizeof(gbz::ZsScratch))))))
        return s;
    if (n_z) {
        GB_CUDA(cudaMemcpyAsync(S->zjobs, zjobs.data(), zjobs.size() * sizeof(InflateJob), cudaMemcpyHostToDevice, st));
        gb_prof_mark *pm = gb_agg_prof_begin(h, "k_pq_unzstd", st);
        k_pq_unzstd<<<(unsigned)z_blocks, 128, 0, st>>>(dfile, (InflateJob *)S->zjobs, (uint32_t)n_z,
                                                         (uint8_t *)S->img, (uint32_t *)S->ilvl, dctl,
                                                         (gbz::ZsScratch *)S->zscratch);
        gb_agg_prof_end(h, pm, st);
        GB_CUDA(cudaGetLastError());
        gb_agg_count_launch(h, 1);
    }
    if (n_jobs) {
        GB_CUDA(cudaMemcpyAsync(S->ijobs, jobs.data(), jobs.size() * sizeof(InflateJob), cudaMemcpyHostToDevice, st));
        gb_prof_mark *pm = gb_agg_prof_begin(h, "k_pq_inflate", st);
        const unsigned grid = (unsigned)std::min<size_t>((n_jobs + 7) / 8, (size_t)sm_count() * 6);
        k_pq_inflate<<<grid, 256, 0, st>>>(dfile, (InflateJob *)S->ijobs, (uint32_t)n_jobs, (uint8_t *)S->img,
                                           (uint32_t *)S->ilvl, dctl);
        gb_agg_prof_end(h, pm, st);
        GB_CUDA(cudaGetLastError());
        gb_agg_count_launch(h, 1);
    }
    std::vector<uint32_t> lvl(pending.size());
    if (!pending.empty())
        GB_CUDA(cudaMemcpyAsync(lvl.data(), S->ilvl, pending.size() * 4, cudaMemcpyDeviceToHost, st));
    Ctl c;
    GB_CUDA(cudaMemcpyAsync(&c, dctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if ((s = pq_fail_if_err(c))) return s;  // nothing is decoded from a malformed block
    for (size_t k = 0; k < pending.size(); k++) {
        PqPage &pg = ip[pending[k]];
        const uint32_t l4 = lvl[k];
        if (l4 == ~0u || 4 + (uint64_t)l4 > pg.raw_bytes || (l4 == 0 && pg.n_values > 0))
            return pq_corrupt("definition levels");
        pg.def_off = pg.off + 4;
        pg.def_bytes = l4;
        pg.off += 4 + (uint64_t)l4;
        pg.bytes = pg.raw_bytes - 4 - l4;
    }
    return GB_OK;
}

extern "C" gb_status gb_agg_ingest_parquet(gb_agg *h, gb_pq_file *f, uint32_t rg_begin, uint32_t rg_end,
                                           const int32_t *col_map, int32_t mem, void *stream) {
    if (!h || !f || !col_map || rg_end > f->rg_rows.size() || rg_begin > rg_end) {
        set_error("invalid arguments to gb_agg_ingest_parquet");
        return GB_ERR_INVALID;
    }
    if (rg_begin == rg_end) return GB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    AggView v;
    gb_status s = gb_agg_view(h, &v);
    if (s) return s;
    const int nc = v.n_cols;
    if (nc > 8) {
        set_error("at most 8 Parquet columns per GROUP BY on the GPU path");
        return GB_ERR_UNSUPPORTED;
    }
    for (int c = 0; c < nc; c++) {
        const int fc = col_map[c];
        if (fc < 0 || fc >= (int)f->cols.size()) {
            set_error("column map entry %d out of range", c);
            return GB_ERR_INVALID;
        }
        const PqColumn &pc = f->cols[fc];
        if (pc.gtype == 0) {
            set_error("Parquet column '%s' has a physical type the GPU path does not decode", pc.name.c_str());
            return GB_ERR_UNSUPPORTED;
        }
        if (pc.repetition == 2) {
            set_error("Parquet column '%s' is REPEATED; the GPU path reads flat columns", pc.name.c_str());
            return GB_ERR_UNSUPPORTED;
        }
        if (pc.repetition == 1 && !((v.nullable_mask >> c) & 1ull)) {
            set_error("Parquet column '%s' is OPTIONAL: declare spec column %d nullable", pc.name.c_str(), c);
            return GB_ERR_INVALID;
        }
        const int want = v.col_types[c];
        const bool ok = want == pc.gtype || (want == GB_T_INTEGER && pc.gtype == GB_T_SMALLINT) ||
                        (want == GB_T_BIGINT && (pc.gtype == GB_T_INTEGER || pc.gtype == GB_T_SMALLINT)) ||
                        (want == GB_T_SMALLINT && pc.gtype == GB_T_INTEGER);
        if (!ok) {
            set_error("column %d: spec type %d does not match Parquet column '%s'", c, want, pc.name.c_str());
            return GB_ERR_INVALID;
        }
    }
    // a VARCHAR column is the group key, dictionary-encoded in the file
    int vc = -1;
    for (int c = 0; c < nc; c++) {
        if (v.col_types[c] != GB_T_VARCHAR) continue;
        if (c != v.str_col) {
            set_error("VARCHAR column %d is not the group key", c);
            return GB_ERR_UNSUPPORTED;
        }
        vc = c;
    }
    // string predicates must be on the VARCHAR key (tested per dictionary entry)
    PqStrFilters SF;
    memset(&SF, 0, sizeof SF);
    for (int q = 0; q < v.n_filters; q++) {
        const Filter &fl = v.filters[q];
        if (fl.op < GB_CMP_STR_EQ) continue;
        if (fl.col != vc) {
            set_error("filter %d: string predicates apply to the dictionary-encoded VARCHAR key on the Parquet path", q);
            return GB_ERR_UNSUPPORTED;
        }
        SF.op[SF.n] = fl.op;
        SF.ptr[SF.n] = fl.ptr;
        SF.len[SF.n] = fl.n;
        SF.n++;
    }
    // zone maps: row groups whose statistics rule out a predicate are skipped
    std::vector<char> live(rg_end - rg_begin, 1);
    uint32_t n_live = 0;
    for (uint32_t g = rg_begin; g < rg_end; g++) {
        for (int q = 0; q < v.n_filters; q++) {
            // a SMALLINT spec over an INT32 file column compares narrowed
            // values: the file's int32 statistics do not bound them
            const int fc = col_map[v.filters[q].col];
            if (v.col_types[v.filters[q].col] == GB_T_SMALLINT && f->cols[fc].gtype == GB_T_INTEGER) continue;
            if (!pq_rg_might_match(f, g, fc, v.filters[q])) {
                live[g - rg_begin] = 0;
                break;
            }
        }
        n_live += live[g - rg_begin] ? 1u : 0u;
    }
    gb_agg_count_pruned(h, (rg_end - rg_begin) - n_live);
    if (n_live == 0) return GB_OK;
    PqScratch *S = g_scratch_for(h);
    // device bytes: the uploaded file, or this batch's byte range copied now
    uint64_t lo = ~0ull, hi = 0;
    for (uint32_t g = rg_begin; g < rg_end; g++) {
        if (!live[g - rg_begin]) continue;  // skipped row groups are not copied
        for (int c = 0; c < nc; c++) {
            const PqChunk &ch = f->chunks[g][col_map[c]];
            lo = std::min(lo, ch.start);
            hi = std::max(hi, ch.start + ch.size);
        }
    }
    const uint8_t *dfile;
    uint64_t base = 0;
    if (mem == GB_MEM_DEVICE) {
        if (!f->dev) {
            set_error("gb_pq_upload the file before ingesting with GB_MEM_DEVICE");
            return GB_ERR_STATE;
        }
        dfile = (const uint8_t *)f->dev;
    } else {
        if ((s = grow(S->file_dev, S->file_cap, hi - lo + 64))) return s;  // slack for word loads past a stream's end
        GB_CUDA(cudaMemcpyAsync(S->file_dev, f->host + lo, hi - lo, cudaMemcpyHostToDevice, st));
        dfile = (const uint8_t *)S->file_dev;
        base = lo;
    }
    // compressed column chunks: every page of the batch is inflated (or
    // copied) into one device image, and the batch decodes from that image
    // through a copy of the page metadata whose offsets point into it
    std::vector<std::vector<PqChunk>> img_chunks;
    std::vector<PqPage> img_pages;
    PqView V{&f->chunks, &f->pages};
    if (f->compressed) {
        if ((s = grow(S->ctl, S->ctl_cap, sizeof(Ctl)))) return s;
        GB_CUDA(cudaMemsetAsync(S->ctl, 0, sizeof(Ctl), st));
        if ((s = pq_inflate_batch(h, f, S, dfile, base, rg_begin, rg_end, live, col_map, nc, (Ctl *)S->ctl, st,
                                  img_chunks, img_pages)))
            return s;
        dfile = (const uint8_t *)S->img;
        base = 0;
        V = PqView{&img_chunks, &img_pages};
    }
    std::vector<PqChunkArg> chunks;
    uint64_t rows = 0;
    for (uint32_t g = rg_begin; g < rg_end; g++) {
        if (!live[g - rg_begin]) continue;
        for (uint64_t r0 = 0; r0 < f->rg_rows[g]; r0 += PQ_CHUNK)
            chunks.push_back({g - rg_begin, (uint32_t)r0, (uint32_t)std::min<uint64_t>(PQ_CHUNK, f->rg_rows[g] - r0)});
        rows += f->rg_rows[g];
    }
    const void *d_pages, *d_runs, *d_page_runs;
    std::vector<uint32_t> col_pages;
    if ((s = grow(S->chunks, S->chunks_cap, chunks.size() * sizeof(PqChunkArg) + 16)) ||
        (s = grow(S->ctl, S->ctl_cap, sizeof(Ctl))))
        return s;
    GB_CUDA(cudaMemsetAsync(S->ctl, 0, sizeof(Ctl), st));
    Ctl *dctl = (Ctl *)S->ctl;
    if (mem == GB_MEM_DEVICE && vc < 0 && !f->compressed) {
        // the resident file's page index (built once), columns picked per call
        if ((s = pq_build_index(f, st))) return s;
        const int nfc = (int)f->cols.size();
        for (uint32_t g = rg_begin; g < rg_end; g++)
            for (int c = 0; c < nc; c++) {
                col_pages.push_back(f->idx_col_pages[2 * (g * nfc + col_map[c])]);
                col_pages.push_back(f->idx_col_pages[2 * (g * nfc + col_map[c]) + 1]);
            }
        d_pages = f->idx_pages;
        d_runs = f->idx_runs;
        d_page_runs = f->idx_page_runs;
    } else {
        // this batch's page table (offsets relative to its byte range) and runs
        std::vector<DPage> pages;
        std::vector<RunJob> jobs;
        uint32_t run_total = 0;
        if ((s = pq_page_table(f, V, rg_begin, rg_end, col_map, nc, base, &live, pages, jobs, col_pages, run_total)))
            return s;
        if (vc >= 0) {
            // the VARCHAR key's data pages gather string ids: page after page,
            // each row group's dictionary entries start at its running base
            const int64_t *ids = nullptr;
            const uint8_t *match = nullptr;
            std::unordered_map<uint32_t, std::pair<uint64_t, uint32_t>> plain_at;
            if ((s = pq_varchar_dict(h, V, S, dfile, base, rg_begin, rg_end, live, col_map[vc], dctl, st, &ids, SF,
                                     &match, plain_at)))
                return s;
            uint64_t eb = 0;
            for (uint32_t g = rg_begin; g < rg_end; g++) {
                if (!live[g - rg_begin]) continue;
                const PqChunk &ch = (*V.chunks)[g][col_map[vc]];
                const uint32_t k = (g - rg_begin) * (uint32_t)nc + (uint32_t)vc;
                if (col_pages[2 * k + 1] - col_pages[2 * k] != ch.page_end - ch.page_begin) {
                    set_error("page table of the VARCHAR key out of step with its chunk");
                    return GB_ERR_INVALID;
                }
                for (uint32_t p = col_pages[2 * k]; p < col_pages[2 * k + 1]; p++) {
                    if (pages[p].kind == 1) {
                        pages[p].dict_ids = (uint64_t)(uintptr_t)(ids + eb);
                        pages[p].dict_match = match ? (uint64_t)(uintptr_t)(match + eb) : 0;
                    } else {  // PLAIN: value j is entry j of the page's strings
                        const auto it = plain_at.find(ch.page_begin + (p - col_pages[2 * k]));
                        if (it == plain_at.end()) {
                            set_error("PLAIN BYTE_ARRAY page without its strings");
                            return GB_ERR_INVALID;
                        }
                        pages[p].dict_ids = (uint64_t)(uintptr_t)(ids + it->second.first);
                        pages[p].dict_match = match ? (uint64_t)(uintptr_t)(match + it->second.first) : 0;
                        pages[p].dict_n = it->second.second;
                    }
                }
                if (ch.dict_off >= 0) eb += ch.dict_n;
                for (const auto &e : plain_at)
                    if ((*V.pages)[e.first].rg == g) eb += e.second.second;
            }
        }
        if ((s = grow(S->pages, S->pages_cap, pages.size() * sizeof(DPage) + 16)) ||
            (s = grow(S->runs, S->runs_cap, (size_t)run_total * sizeof(DRun) + 16)) ||
            (s = grow(S->page_runs, S->page_runs_cap, pages.size() * PQ_PR * 4 + 16)) ||
            (s = grow(S->dict_pages, S->dict_pages_cap, jobs.size() * sizeof(RunJob) + 16)))
            return s;
        GB_CUDA(cudaMemcpyAsync(S->pages, pages.data(), pages.size() * sizeof(DPage), cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemsetAsync(S->page_runs, 0, pages.size() * PQ_PR * 4 + 16, st));
        if (!jobs.empty()) {
            GB_CUDA(cudaMemcpyAsync(S->dict_pages, jobs.data(), jobs.size() * sizeof(RunJob), cudaMemcpyHostToDevice,
                                    st));
            gb_prof_mark *pm = gb_agg_prof_begin(h, "k_pq_runs", st);
            k_pq_runs<<<(unsigned)jobs.size(), 128, 0, st>>>(dfile, (const DPage *)S->pages,
                                                             (const RunJob *)S->dict_pages, (DRun *)S->runs,
                                                             (uint32_t *)S->page_runs, dctl);
            gb_agg_prof_end(h, pm, st);
            GB_CUDA(cudaGetLastError());
            gb_agg_count_launch(h, 1);
        }
        d_pages = S->pages;
        d_runs = S->runs;
        d_page_runs = S->page_runs;
    }
    if ((s = grow(S->col_pages, S->col_pages_cap, col_pages.size() * 4 + 16))) return s;
    GB_CUDA(cudaMemcpyAsync(S->col_pages, col_pages.data(), col_pages.size() * 4, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(S->chunks, chunks.data(), chunks.size() * sizeof(PqChunkArg), cudaMemcpyHostToDevice, st));
    // compacted output columns (batch rows bound the survivors)
    if (S->out_cap_rows < rows) {
        for (int c = 0; c < GB_MAX_COLS; c++)
            if (S->out[c]) {
                cudaFree(S->out[c]);
                S->out[c] = nullptr;
            }
        S->out_cap_rows = 0;
        for (int c = 0; c < nc; c++) {
            cudaError_t e = cudaMalloc(&S->out[c], rows * 8 + 64);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                return cuda_fail(e, "cudaMalloc (parquet columns)");
            }
        }
        S->out_cap_rows = rows;
    }
    // validity of the OPTIONAL columns' output (all ones; the scan clears NULLs)
    const size_t vwords = (size_t)(rows + 63) / 64 + 1;
    for (int c = 0; c < nc; c++) {
        if (c == vc || f->cols[col_map[c]].repetition != 1) continue;
        if ((s = grow(S->out_valid[c], S->out_valid_cap[c], vwords * 8))) return s;
        GB_CUDA(cudaMemsetAsync(S->out_valid[c], 0xff, vwords * 8, st));
    }
    PqScan P;
    memset(&P, 0, sizeof P);
    P.n_cols = nc;
    P.id_col = vc;
    P.str_match = SF.n ? 1 : 0;
    for (int c = 0; c < nc; c++) {
        P.out_type[c] = c == vc ? GB_T_BIGINT : v.col_types[c];  // VARCHAR: its string ids
        P.out[c] = S->out[c];
        P.out_valid[c] = (c != vc && f->cols[col_map[c]].repetition == 1) ? (uint64_t *)S->out_valid[c] : nullptr;
    }
    P.n_filters = v.n_filters;
    for (int q = 0; q < v.n_filters; q++) P.filters[q] = v.filters[q];
    P.out_cap = S->out_cap_rows;
    {
        if ((s = grow(S->views, S->views_cap, chunks.size() * pq_view_words(nc) * 4 + 16))) return s;
        const int vgrid = (int)std::min<size_t>((chunks.size() + 127) / 128, (size_t)sm_count() * 8);
        gb_prof_mark *pv = gb_agg_prof_begin(h, "k_pq_views", st);
        k_pq_views<<<std::max(vgrid, 1), 128, 0, st>>>((const DPage *)d_pages, (const DRun *)d_runs,
                                                       (const uint32_t *)d_page_runs, (const uint32_t *)S->col_pages,
                                                       (const PqChunkArg *)S->chunks, (uint32_t)chunks.size(), nc, vc,
                                                       (uint32_t *)S->views);
        gb_agg_prof_end(h, pv, st);
        // one wave: the blocks that fit on the SMs at once (4 each) loop over the chunks
        const int grid = (int)std::min<size_t>(chunks.size(), (size_t)sm_count() * 4);
        gb_prof_mark *pm = gb_agg_prof_begin(h, "k_pq_scan", st);
        k_pq_scan<<<std::max(grid, 1), 256, 0, st>>>(dfile, (const DPage *)d_pages, (const DRun *)d_runs,
                                                     (const uint32_t *)d_page_runs, (const uint32_t *)S->col_pages,
                                                     (const PqChunkArg *)S->chunks, (uint32_t)chunks.size(),
                                                     (const uint32_t *)S->views, P, dctl);
        gb_agg_prof_end(h, pm, st);
        GB_CUDA(cudaGetLastError());
        gb_agg_count_launch(h, 2);
    }
    Ctl c;
    GB_CUDA(cudaMemcpyAsync(&c, dctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if ((s = pq_fail_if_err(c))) return s;
    // the survivors go through the ordinary ingest (filters already applied)
    gb_col cols[GB_MAX_COLS];
    for (int q = 0; q < nc; q++) cols[q] = {S->out[q], (const uint64_t *)P.out_valid[q], nullptr};
    if (vc >= 0) return gb_agg_ingest_prefiltered_ids(h, cols, c.out_count, (const int64_t *)S->out[vc], stream);
    return gb_agg_ingest_prefiltered(h, cols, c.out_count, stream);
}
